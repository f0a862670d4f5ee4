#!/usr/bin/env python3
"""Benchmark of the pyramaterised hot path on GB300.

Workload (one step): the batched-sampling configuration at N = 20 -- the
hardware-efficient ansatz (RY, RZ on every qubit, CNOT ladder) with L = 20
layers (P = 800 angles), a batch of B = 256 parameter rows per launch, then
Meyer-Wallach Q over the batch and the 20100-pair fidelity histogram (the first
S = 201 states, 75 bins) with its KL expressibility.  Synthetic inputs:
theta ~ U[0, 2 pi) from a seeded generator.  The 4 GiB of states per step is
far larger than L2, so no flush is needed between steps.

`value` is circuit evals/s with theta resident on the device; `e2e` is the
same step through the public API (`PQC.run_batch` + measures) from host
parameter buffers with the scalar results read back.  `--impl reference`
times the CPU oracle (a numpy restatement of the reference's algorithm; the
reference itself needs QuTiP 4.7.2, which is not installable here) on all host
cores with a bounded per-step sample.
"""
import argparse
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "circuit evals/s + HBM GB/s (N=20); QFIM/s (N=16); serve p50/p99 vs plain"
UNIT = "circuit evals/s"


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--n-qubits", type=int, default=20)
    ap.add_argument("--layers", type=int, default=20)
    ap.add_argument("--batch", type=int, default=256)
    ap.add_argument("--pair-states", type=int, default=201)
    ap.add_argument("--nbins", type=int, default=75)
    ap.add_argument("--tile", type=int, default=0)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--cpu-sample-layers", type=int, default=2)
    return ap.parse_args()


def workload_config(a):
    return {
        "workload": (f"batched sampling: HE ladder N={a.n_qubits} L={a.layers} (RY,RZ all + CNOT 0->1->..), "
                     f"B={a.batch} theta rows/launch, Meyer-Wallach over the batch, "
                     f"{a.pair_states * (a.pair_states - 1) // 2}-pair fidelity histogram "
                     f"(S={a.pair_states}, {a.nbins} bins) + KL expressibility"),
        "n_qubits": a.n_qubits, "layers": a.layers, "batch": a.batch,
        "params_per_circuit": 2 * a.n_qubits * a.layers, "pair_states": a.pair_states, "nbins": a.nbins,
        "l2": "states (16 B x 2^N x B per step) are larger than the 129 MB L2; no flush needed",
        "parallelism": "replicas (independent batches per GPU)",
    }


# ---------------------------------------------------------------------- clocks
class ClockSampler:
    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
             "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
             "clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.idx = gpu_index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.idx}", f"--query-gpu={self.QUERY}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except (FileNotFoundError, OSError):
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, smax, reasons = [], None, set()
        names = ["active", "hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax = float(f[2])
            except ValueError:
                continue
            for n, v in zip(names[1:], f[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": smax, "reasons": sorted(reasons),
                "samples": len(sm)}


# ---------------------------------------------------------------------- CPU oracle timing
def oracle_sample(N, L, sample_layers, seed, reps=1):
    """Time the oracle on the first `sample_layers` layers of one circuit; returns (seconds, fraction of an eval)."""
    import pyramaterised_gb300 as pq
    from oracle import pqc_oracle as O

    c = pq.templates.hardware_efficient_ladder(N, sample_layers)
    th = np.random.default_rng(seed).random(c.n_columns()) * 2 * np.pi
    t0 = time.perf_counter()
    for _ in range(reps):
        psi = O.run(c.gates, N, th)
    dt = time.perf_counter() - t0
    assert abs(np.linalg.norm(psi) - 1) < 1e-9
    return dt, reps * sample_layers / L


def cpu_baseline(a, threads=1):
    """Oracle evals/s on `threads` host threads (each evaluates its own circuit sample)."""
    from concurrent.futures import ThreadPoolExecutor

    with ThreadPoolExecutor(max_workers=threads) as ex:
        t0 = time.perf_counter()
        res = list(ex.map(lambda s: oracle_sample(a.n_qubits, a.layers, a.cpu_sample_layers, s), range(threads)))
        wall = time.perf_counter() - t0
    evals = sum(r[1] for r in res)
    return evals / wall, wall, evals


# ---------------------------------------------------------------------- reference arm
def run_reference(a):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    threads = os.cpu_count() or 1
    try:
        import threadpoolctl

        threadpoolctl.threadpool_limits(1)
    except ImportError:
        pass
    for _ in range(a.warmup):
        cpu_baseline(a, threads)
    t = []
    evals_total = 0.0
    for _ in range(a.steps):
        v, wall, evals = cpu_baseline(a, threads)
        t.append(wall)
        evals_total += evals
    total = sum(t)
    value = evals_total / total
    sample = (f"each step: {threads} threads x the first {a.cpu_sample_layers} of {a.layers} layers of one "
              f"N={a.n_qubits} HE circuit (oracle numpy FP64), scaled to whole circuit evals")
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": a.gpus, "steps": a.steps, "warmup": a.warmup,
            "ms_per_step": 1e3 * total / a.steps, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "c128 (FP64)", "data": "synthetic", "config": workload_config(a), "impl": "reference",
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port", "sample": sample},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


# ---------------------------------------------------------------------- our arm
def run_ours(a):
    import torch
    import torch.distributed as dist

    import pyramaterised_gb300 as pq
    from pyramaterised_gb300 import _lib, engine

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    if world > 1:
        dist.init_process_group("nccl", device_id=dev)
    lib = _lib.load()
    N, L, B = a.n_qubits, a.layers, a.batch
    c = pq.templates.hardware_efficient_ladder(N, L)
    if a.tile:
        c.set_tile_qubits(a.tile)
    prog = c.program
    info = prog.info()
    P = c.n_columns()
    theta_host = torch.from_numpy(np.random.default_rng(1234 + rank).random((B, P)) * 2 * np.pi).pin_memory()
    theta = theta_host.to(dev)
    psi = torch.empty((B, 1 << N), dtype=torch.complex128, device=dev)
    S = min(a.pair_states, B)
    stream = torch.cuda.current_stream()

    run_ev = []

    def step(record=False):
        if record:
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
        prog.run(theta, 0, out=psi)
        if record:
            e1.record(stream)
            run_ev.append((e0, e1))
        Q = engine.mw(psi)
        _, counts, edges = engine.allpairs_fidelity_hist(psi[:S], a.nbins, keep_samples=False)
        kl = engine.expr_kl(counts, edges, float(2 ** N))
        return Q, counts, kl

    def barrier():
        if world > 1:
            dist.barrier()

    for _ in range(a.warmup):
        step()
    torch.cuda.synchronize()
    barrier()
    clocks = ClockSampler(local)
    clocks.start()
    time.sleep(0.3)
    launches0 = lib.pqc_launch_count()
    t0 = torch.cuda.Event(enable_timing=True)
    t1 = torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    t0.record(stream)
    for _ in range(a.steps):
        step(record=True)
    t1.record(stream)
    torch.cuda.synchronize()
    launches = lib.pqc_launch_count() - launches0
    ms = t0.elapsed_time(t1)
    barrier()
    run_ms = sum(e0.elapsed_time(e1) for e0, e1 in run_ev) / a.steps
    ms_t = torch.tensor([ms], dtype=torch.float64, device=dev)
    if world > 1:
        dist.all_reduce(ms_t, op=dist.ReduceOp.MAX)
    ms = float(ms_t.item())
    value = world * B * a.steps / (ms / 1e3)

    # e2e: public API from host buffers, results read back each step
    def e2e_step():
        states = c.run_batch(theta_host)
        Q = engine.mw(states)
        _, counts, edges = engine.allpairs_fidelity_hist(states[:S], a.nbins, keep_samples=False)
        kl = engine.expr_kl(counts, edges, float(2 ** N))
        out = torch.cat([Q.mean().reshape(1), Q.std(unbiased=False).reshape(1), kl, counts.to(torch.float64)])
        return out.cpu()

    e2e_step()
    torch.cuda.synchronize()
    barrier()
    w0 = time.perf_counter()
    for _ in range(a.steps):
        res = e2e_step()
    torch.cuda.synchronize()
    e2e_s = time.perf_counter() - w0
    e_t = torch.tensor([e2e_s], dtype=torch.float64, device=dev)
    if world > 1:
        dist.all_reduce(e_t, op=dist.ReduceOp.MAX)
    e2e_value = world * B * a.steps / float(e_t.item())
    clk = clocks.stop()

    # roofline of the dominant kernel (the fused sweep): algorithmic bytes = one read + one write of every
    # amplitude of the batch per sweep launch (16 B each way per amplitude)
    peaks = {}
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            peaks = json.load(f)
    except OSError:
        pass
    hbm_peak = float(peaks.get("hbm_gbs", 6800.0))
    peak_src = "measured" if "hbm_gbs" in peaks else "fallback"
    n_sweeps = info["n_sweeps"]
    bytes_per_launch = 32.0 * (1 << N) * B
    sweep_ms = run_ms / n_sweeps
    achieved = bytes_per_launch / (sweep_ms / 1e3) / 1e9
    # FP32-pipe work of the same launch: ~38 FP32 ops per amplitude per rotation (double-float 2-term dots)
    rot_per_sweep = 2 * N * L / n_sweeps
    fp32_ops = 38.0 * rot_per_sweep * (1 << N) * B
    traffic = os.environ.get("PQC_SWEEP_TRAFFIC_BYTES")
    hbm_total_gbs = bytes_per_launch * n_sweeps * a.steps / (ms / 1e3) / 1e9

    if rank != 0:
        return
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": a.steps, "warmup": a.warmup,
        "ms_per_step": ms / a.steps, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "c128", "data": "synthetic",
        "config": dict(workload_config(a), arithmetic="double-float (hi+lo fp32) on the FP32 pipes; complex128 I/O",
                       n_sweeps=n_sweeps, tile_qubits=info["tile_qubits"]),
        "hbm_gbs_step": hbm_total_gbs,
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": hbm_peak, "unit": "GB/s",
                     "frac": achieved / hbm_peak, "traffic": float(traffic) if traffic else None,
                     "kernel": "sweep_kernel<ArithDF>", "peak_source": peak_src,
                     "algorithmic_bytes_per_launch": bytes_per_launch, "launch_ms": sweep_ms,
                     "fp32_ops_per_launch": fp32_ops, "fp32_tflops": fp32_ops / (sweep_ms / 1e3) / 1e12},
        "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": int(theta_host.numel() * 8),
                "d2h_bytes_per_step": int(res.numel() * 8)},
        "gpu_launches": int(launches),
        "clocks": clk,
    }
    if not a.no_cpu_baseline:
        v, wall, evals = cpu_baseline(a, 1)
        line["cpu_baseline"] = {"value": v, "unit": UNIT, "cores": 1, "kind": "port",
                                "sample": f"first {a.cpu_sample_layers} of {a.layers} layers of one N={a.n_qubits} "
                                          f"HE circuit on the numpy FP64 oracle ({wall:.1f} s), scaled to evals"}
    print(json.dumps(line), flush=True)
    if world > 1:
        dist.destroy_process_group()


def main():
    a = parse()
    if a.impl == "reference":
        run_reference(a)
    else:
        run_ours(a)


if __name__ == "__main__":
    main()
