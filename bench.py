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
    ap.add_argument("--tile", type=int, default=0, help="force the sweep tile size (skips the autotuner)")
    ap.add_argument("--ctas", type=int, default=0, help="with --tile: CTAs per SM (2 or 3; 0 = default)")
    ap.add_argument("--threads", type=int, default=0, help="with --tile --ctas 3: threads per CTA (256 or 128)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--cpu-sample-layers", type=int, default=20)
    ap.add_argument("--cpu-seconds", type=float, default=10.0, help="CPU baseline: seconds of oracle work")
    ap.add_argument("--no-secondary", action="store_true", help="skip the other configurations")
    ap.add_argument("--no-autotune", action="store_true", help="default tile and launch shape, no tuning")
    ap.add_argument("--profile-case", default="", help="run one small workload for an ncu capture and exit")
    ap.add_argument("--serve-requests", type=int, default=10000, help="requests of the continuous-batching stream")
    ap.add_argument("--serve-rate", type=float, default=250.0, help="its Poisson arrival rate (per second)")
    ap.add_argument("--serve-plain-requests", type=int, default=1000,
                    help="prefix of that stream also served by the plain FIFO path (it runs about 37 requests/s)")
    ap.add_argument("--serve-low-requests", type=int, default=500, help="a second stream that both servers sustain")
    ap.add_argument("--serve-low-rate", type=float, default=25.0)
    ap.add_argument("--serve-max-qubits", type=int, default=22)
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


def _oracle_worker(args):
    N, L, sample_layers, seed, min_seconds = args
    t_end = time.perf_counter() + min_seconds
    done = 0.0
    while True:
        done += oracle_sample(N, L, sample_layers, seed)[1]
        seed += 1000
        if time.perf_counter() >= t_end:
            return done


def _oracle_rows(args):
    """Whole-circuit oracle states of the given theta rows (the HE ladder N, L) and the seconds they took."""
    import pyramaterised_gb300 as pq
    from oracle import pqc_oracle as O

    N, L, thetas = args
    c = pq.templates.hardware_efficient_ladder(N, L)
    t0 = time.perf_counter()
    states = [O.run(c.gates, N, t) for t in thetas]
    return np.stack(states), time.perf_counter() - t0


def _oracle_import(_):
    import pyramaterised_gb300  # noqa: F401  (templates for the sample circuit)
    from oracle import pqc_oracle  # noqa: F401
    return 0


_POOL = {}


def _oracle_pool(workers):
    """A pool of `workers` single-threaded processes (spawned, BLAS limited to one thread each)."""
    import multiprocessing as mp

    if workers not in _POOL:
        for v in ("OMP_NUM_THREADS", "OPENBLAS_NUM_THREADS", "MKL_NUM_THREADS"):
            os.environ[v] = "1"
        pool = mp.get_context("spawn").Pool(workers)
        pool.map(_oracle_import, range(workers))  # imports happen outside the timed calls
        _POOL[workers] = pool
    return _POOL[workers]


def cpu_baseline(a, threads=1, min_seconds=0.0):
    """Oracle evals/s on `threads` host cores (one single-threaded process each), each evaluating circuit
    samples (the first `cpu_sample_layers` layers of one circuit) until `min_seconds` have passed (at least
    one sample each)."""
    pool = _oracle_pool(threads)
    t0 = time.perf_counter()
    res = pool.map(_oracle_worker, [(a.n_qubits, a.layers, a.cpu_sample_layers, s, min_seconds)
                                    for s in range(threads)])
    wall = time.perf_counter() - t0
    evals = sum(res)
    return evals / wall, wall, evals


# ---------------------------------------------------------------------- reference arm
def run_reference(a):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    threads = os.cpu_count() or 1
    import copy

    light = copy.copy(a)
    light.cpu_sample_layers = min(2, a.cpu_sample_layers)
    for _ in range(a.warmup):  # warm-up steps on a 2-layer sample
        cpu_baseline(light, threads)
    t = []
    evals_total = 0.0
    for _ in range(a.steps):
        v, wall, evals = cpu_baseline(a, threads)
        t.append(wall)
        evals_total += evals
    total = sum(t)
    value = evals_total / total
    sample = (f"each step: {threads} single-threaded processes x one sample of {a.cpu_sample_layers} of "
              f"{a.layers} layers of an N={a.n_qubits} HE circuit (oracle numpy FP64), scaled to whole circuit "
              f"evals; circuit evaluation only (the step's measures are under 7% of the GPU step)")
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": a.gpus, "steps": a.steps, "warmup": a.warmup,
            "ms_per_step": 1e3 * total / a.steps, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "c128 (FP64)", "data": "synthetic", "config": workload_config(a), "impl": "reference",
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port", "sample": sample},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


# FP64 and FP32 GEMM rates of this GPU (cuBLAS, n = 8192) as `python bench.py --profile-case pipes` measured them:
# the denominators of the FP64-equivalent rates below.
FP64_GEMM_TFLOPS = 1.10
FP32_GEMM_TFLOPS = 69.8


# DRAM bytes of one sweep launch of the N = 20 HE ladder (L = 20, 2^13-amplitude tiles, 12-sweep plan) as ncu
# counted them at batch 16, per batch row: dram__bytes.sum.per_second x gpu__time_duration of the 15th sweep launch of
# `python bench.py --batch 16 --steps 2 --warmup 1 --no-cpu-baseline --no-secondary --tile 13 --ctas 1`
# (476.9 MB in 1179.7 us).  The bench scales the figure to its batch.
SWEEP_TRAFFIC_PER_ROW = 29806000.0


# ---------------------------------------------------------------------- secondary measures
def _timed(fn, reps, warm=1):
    """Device time per call of fn (CUDA events on the current stream, synchronised both sides)."""
    import torch

    for _ in range(warm):
        fn()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(reps):
        out = fn()
    e1.record()
    torch.cuda.synchronize()
    return e0.elapsed_time(e1) / reps, out


def secondary_measures(a, dev, value, hbm_peak):
    """The other configurations of the metric, each on a bounded sample (stated in each entry)."""
    import torch

    import pyramaterised_gb300 as pq
    from pyramaterised_gb300 import engine, serve

    out = {}
    N, L, B = a.n_qubits, a.layers, a.batch
    rng = np.random.default_rng(7)
    # TFIM-style ansatz at the same size
    c = pq.templates.tfim_style(N, L)
    c.autotune(B)
    th = torch.from_numpy(rng.random((B, c.n_columns())) * 2 * np.pi).to(dev)
    psi = torch.empty((B, 1 << N), dtype=torch.complex128, device=dev)
    ms, _ = _timed(lambda: c.program.run(th, 0, out=psi), 3)
    out["tfim_style"] = {"workload": f"TFIM-style N={N} L={L} (RX all, CNOT-RZ-CNOT open chain), B={B}",
                         "evals_per_s": B / ms * 1e3, "ms_per_launch_set": ms,
                         "n_sweeps": c.program.info()["n_sweeps"]}
    del psi
    # the plain one-circuit-per-launch path (FP64, one kernel per op, one circuit at a time)
    h = pq.templates.hardware_efficient_ladder(N, L)
    thp = torch.from_numpy(rng.random((4, h.n_columns())) * 2 * np.pi).to(dev)
    one = torch.empty((1, 1 << N), dtype=torch.complex128, device=dev)

    def plain4():
        for i in range(4):
            h.program.run(thp[i:i + 1], 0, mode="plain", out=one)
    ms, _ = _timed(plain4, 1)
    plain_eps = 4 / ms * 1e3
    out["plain_path"] = {"workload": f"HE N={N} L={L}, one circuit per launch sequence, FP64 op by op "
                                     f"({len(h.program._ops)} kernels per circuit), 4 circuits",
                         "evals_per_s": plain_eps, "fused_speedup": value / plain_eps}
    # complex64 sampling mode and its fidelity error against complex128
    h.autotune(B)
    thc = torch.from_numpy(rng.random((B, h.n_columns())) * 2 * np.pi).to(dev)
    ms64, s64 = _timed(lambda: h.program.run(thc, 0, mode="c64"), 3)
    s128 = h.program.run(thc, 0)
    S = min(a.pair_states, B)
    f128 = engine.allpairs_fidelity_hist(s128[:S], a.nbins)[0]
    f64 = engine.allpairs_fidelity_hist(s64[:S].to(torch.complex128), a.nbins)[0]
    # the counts-only histogram's first tier: the tensor-core Gram of the S states (tcgen05, TF32), whole call
    # (plane split, Gram, slice reduction); 8 flops per amplitude per (row block of 128, column block of 256) pair
    if S <= 256 and N >= 13:
        msg, (Gt, dfac) = _timed(lambda: engine.gram_tf32(s128[:S]), 3)
        n_mt = 2 if S > 128 else 1
        flops = n_mt * 128 * 256 * float(1 << N) * 8
        exact = engine.allpairs_fidelity_hist(s128[:S], a.nbins)[0]
        Gf = (Gt.abs() ** 2)[torch.triu_indices(S, S, 1, device=dev).unbind(0)]
        out["tensor_gram"] = {"workload": f"<a|b> of {S} states, N={N}, tcgen05.mma kind::tf32", "ms": msg,
                              "tflops_tf32": flops / (msg / 1e3) / 1e12, "delta_factor": dfac,
                              "max_abs_fidelity_error_vs_exact": float((Gf - exact).abs().max())}
        del Gt, Gf, exact
    # the same fused sweeps in native FP64 (complex128 arithmetic, the reference's precision) on the same batch
    ms_f64, sf = _timed(lambda: h.program.run(thc, 0, mode="f64"), 1)
    n_sw = h.program.info()["n_sweeps"]
    gbs = 32.0 * (1 << N) * B * n_sw / (ms_f64 / 1e3) / 1e9
    out["fp64_arm"] = {"workload": f"HE N={N} L={L}, B={B}, the fused sweeps in native FP64 arithmetic",
                       "evals_per_s": B / ms_f64 * 1e3, "ms_per_batch": ms_f64, "n_sweeps": n_sw,
                       "sweep_hbm_gbs": gbs, "hbm_frac": gbs / hbm_peak,
                       "max_abs_amp_diff_vs_double_float": float((sf - s128).abs().max())}
    del sf
    out["c64_mode"] = {"evals_per_s": B / ms64 * 1e3,
                       "max_abs_fidelity_error_vs_c128": float((f128 - f64).abs().max()), "pairs": int(f128.numel()),
                       "error_vs_fp64_oracle": "parity.c64_* (rows 0-1 of the main batch)"}
    del s64, s128, f128, f64
    # differentiation: <H> and its gradient by the adjoint, N=16 HE L=8 (P=256)
    d = pq.templates.hardware_efficient_ladder(16, 8)
    thd = torch.from_numpy(rng.random((64, d.n_columns())) * 2 * np.pi).to(dev)
    adj = {}
    for name, H in (("tfim_h1", pq.hamiltonian.tfim_open(16, 1.0)), ("xxz_d0.5", pq.hamiltonian.xxz_open(16, 0.5))):
        ms, _ = _timed(lambda: d.program.energy_grad(thd, H), 3)
        # algorithmic bytes per gradient (one row): 32 D (3 L ceil(N/13) + 1) -- the forward sweeps, the reverse
        # sweeps over psi and lambda, and lambda = H psi
        gbs = 32.0 * (1 << 16) * (3 * 8 * 2 + 1) * 64 / (ms / 1e3) / 1e9
        adj[name] = {"grads_per_s": 64 / ms * 1e3, "ms_per_64": ms, "alg_gbs": gbs, "hbm_frac": gbs / hbm_peak}
    out["adjoint"] = dict(adj, workload="HE N=16 L=8 P=256, batch of 64 theta rows, E and dE/dtheta",
                          alg_bytes_per_grad="32 D (3 L ceil(N/13) + 1) = 102.8 MB")
    # QFIM at N=16 P=256 (derivative states + Gram) and the effective quantum dimension
    m = pq.measure.Measurements(d)
    thq = rng.random((10, d.n_columns())) * 2 * np.pi

    def qfims():
        F = None
        for t in thq:
            d.run(list(t))
            F = m.get_QFI()
        return F
    d.run(list(thq[0]))  # warm-up: the first QFIM plans the derivative runs
    m.get_QFI()
    t0 = time.perf_counter()
    F = qfims()
    wall = time.perf_counter() - t0
    eqd = int((np.linalg.eigvalsh(F) > 1e-12).sum())
    # where a QFIM's device time goes (derivative states vs Gram), fused path against the plain path (one FP64
    # kernel per op, every derivative circuit from the start) with the same Gram
    th1 = torch.from_numpy(thq[:1]).to(dev)
    psi1 = d.program.run(th1, 0)
    ms_fd, dps = _timed(lambda: d.program.gradient_states(th1), 3)
    ms_g, _ = _timed(lambda: engine.qfim(psi1, dps), 3)
    ms_pd, pdps = _timed(lambda: d.program.gradient_states(th1, plain=True), 1)
    plain_err = float((pdps - dps).abs().max())
    del dps, pdps
    out["qfim"] = {"workload": "HE N=16 L=8, full 256x256 QFIM, 10 random theta (host loop through Measurements, "
                               "after one warm-up QFIM)",
                   "qfim_per_s": len(thq) / wall, "eff_quantum_dim_last": eqd,
                   "device_ms": {"derivative_states": ms_fd, "gram": ms_g, "plain_derivative_states": ms_pd},
                   "device_qfim_per_s": 1e3 / (ms_fd + ms_g), "plain_qfim_per_s": 1e3 / (ms_pd + ms_g),
                   "fused_over_plain": (ms_pd + ms_g) / (ms_fd + ms_g),
                   "plain_vs_fused_max_abs_dpsi": plain_err}
    # rooflines: derivative states 32 D ceil(N/13) P L / 2 bytes per theta against HBM, the Gram 4 P^2 D flops per
    # theta (a real SYRK over 2 D) against the FP64 and FP32 GEMM rates (its double-float MACs run on the FP32 pipes)
    ds_gbs = 32.0 * (1 << 16) * 2 * 256 * 8 / 2 / (ms_fd / 1e3) / 1e9
    gram_tf = 4.0 * 256 * 256 * (1 << 16) / (ms_g / 1e3) / 1e12
    out["qfim"]["roofline"] = {"derivative_states_alg_gbs": ds_gbs, "derivative_states_hbm_frac": ds_gbs / hbm_peak,
                               "gram_fp64_equiv_tflops": gram_tf, "gram_over_fp64_gemm": gram_tf / FP64_GEMM_TFLOPS,
                               "gram_over_fp32_gemm": gram_tf / FP32_GEMM_TFLOPS}
    # magic: NPQC-style N=12, 64 states
    g = pq.templates.npqc_style(12, 12)
    thm = torch.from_numpy(rng.random((64, g.n_columns())) * 2 * np.pi).to(dev)
    sm = g.program.run(thm, 0)
    ms, _ = _timed(lambda: engine.magic(sm, 2.0), 2)
    mg = (11 + 2 * 12) * 4.0 ** 12 * 64 / (ms / 1e3) / 1e12  # (11 + 2N) 4^N flops per state
    out["magic"] = {"workload": "NPQC-style N=12 L=12, 64 states, Renyi-2 over all 4^N Paulis",
                    "states_per_s": 64 / ms * 1e3, "fp64_equiv_tflops": mg, "over_fp64_gemm": mg / FP64_GEMM_TFLOPS,
                    "over_fp32_gemm": mg / FP32_GEMM_TFLOPS}
    # serving: continuous batching against the plain FIFO path on the same seeded streams -- the full stream at a
    # rate that only the batched server sustains (the plain path serves its first requests), and a slower stream
    # that both sustain
    if a.serve_requests > 0:
        def serve_pair(reqs, n_plain):
            srv = serve.Server(hbm_budget=48 << 30, n_streams=4, max_rows=256)
            srv.prepare(reqs)
            t0 = time.perf_counter()
            res = srv.run(reqs, realtime=True)
            fused = serve.latency_summary(res, time.perf_counter() - t0)
            sub = reqs[:n_plain]
            pl = serve.PlainServer()
            pl.prepare(sub)
            t0 = time.perf_counter()
            pres = pl.run(sub, realtime=True)
            plain = serve.latency_summary(pres, time.perf_counter() - t0)
            fused_sub = serve.latency_summary({r.rid: res[r.rid] for r in sub})
            return {"continuous_batching": fused, "continuous_batching_same_prefix": fused_sub, "plain_fifo": plain}

        mix = (f"N~U{{6..{a.serve_max_qubits}}}, HE or TFIM-style, L~U{{2..2N}}, 40% fidelity pair / 30% MW / "
               "20% E+grad (TFIM h=1) / 10% QFIM P<=128")
        reqs = serve.synthetic_stream(a.serve_requests, a.serve_rate, seed=0, n_range=(6, a.serve_max_qubits))
        out["serve"] = dict(serve_pair(reqs, min(a.serve_plain_requests, len(reqs))),
                            workload=(f"{a.serve_requests} requests, Poisson arrivals at {a.serve_rate}/s (seed 0), "
                                      f"{mix}; the plain FIFO path serves the first {a.serve_plain_requests}"))
        if a.serve_low_requests > 0:
            low = serve.synthetic_stream(a.serve_low_requests, a.serve_low_rate, seed=1, n_range=(6, a.serve_max_qubits))
            out["serve_low_rate"] = dict(serve_pair(low, len(low)),
                                         workload=(f"{a.serve_low_requests} requests, Poisson arrivals at "
                                                   f"{a.serve_low_rate}/s (seed 1), {mix}; both servers"))
    return out


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
    tune = None
    if a.tile:
        c.set_tile_qubits(a.tile)
        c._ctas_per_sm = a.ctas
        c._sweep_threads = a.threads
    elif not a.no_autotune:
        tune = {f"k{k}_ctas{o}_t{t}": round(ms, 3) for (k, o, t), ms in c.autotune(B).items()}
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
    if prog.status() != 0:
        raise SystemExit("a sweep's bulk tile load timed out during the timed region (pqc_program_status)")
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

    # roofline of the dominant kernel (the fused sweep).  Algorithmic bytes per eval follow the layer-sweep model
    # of a statevector engine with 2^13-amplitude tiles: every layer reads and writes the state ceil(N/13) times,
    # 32 B per amplitude, B_eval = 32 * 2^N * L * ceil(N/13).  One launch is one of the plan's n_sweeps sweeps over
    # the batch, so it carries B * B_eval / n_sweeps of that work; the bytes it really moves (one read and one
    # write of the batch, ncu traffic) are reported beside it.
    peaks = {}
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            peaks = json.load(f)
    except OSError:
        pass
    hbm_peak = float(peaks.get("hbm_gbs", 6800.0))
    peak_src = "measured" if "hbm_gbs" in peaks else "fallback"
    n_sweeps = info["n_sweeps"]
    b_eval = 32.0 * (1 << N) * L * (-(-N // 13)) if N > 13 else 16.0 * (1 << N)
    bytes_per_launch = b_eval * B / n_sweeps
    moved_per_launch = 32.0 * (1 << N) * B
    sweep_ms = run_ms / n_sweeps
    achieved = bytes_per_launch / (sweep_ms / 1e3) / 1e9
    traffic = SWEEP_TRAFFIC_PER_ROW * B if (N, L) == (20, 20) else None
    # gate arithmetic in FP64-equivalent flops (6 per amplitude per RY or RZ, CNOTs free): 12 N L 2^N per eval
    flops_eval = 12.0 * N * L * (1 << N)
    hbm_total_gbs = moved_per_launch * n_sweeps * a.steps / (ms / 1e3) / 1e9

    if rank != 0:
        return
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": a.steps, "warmup": a.warmup,
        "ms_per_step": ms / a.steps, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "c128", "data": "synthetic",
        "config": dict(workload_config(a), arithmetic="double-float (hi+lo fp32) on the FP32 pipes; complex128 I/O",
                       n_sweeps=n_sweeps, tile_qubits=info["tile_qubits"],
                       ctas_per_sm=getattr(prog, "ctas_per_sm", 0) or (1 if info["tile_qubits"] >= 13 else 3),
                       threads_per_cta=getattr(prog, "sweep_threads", 0) or (512 if info["tile_qubits"] >= 13 else 256),
                       autotune_ms_per_batch=tune),
        "hbm_gbs_step": hbm_total_gbs,
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": hbm_peak, "unit": "GB/s",
                     "frac": achieved / hbm_peak, "traffic": traffic,
                     "traffic_source": "ncu dram bytes of one sweep launch at batch 16 (bench.py --batch 16 --tile 13 "
                                       "--ctas 1), scaled by rows" if traffic else None,
                     "kernel": "sweep_kernel<ArithDF>", "peak_source": peak_src,
                     "algorithmic_bytes_per_eval": b_eval, "algorithmic_bytes_per_launch": bytes_per_launch,
                     "launch_ms": sweep_ms, "moved_bytes_per_launch": moved_per_launch,
                     "moved_gbs": moved_per_launch / (sweep_ms / 1e3) / 1e9,
                     "fp64_equiv_tflops": flops_eval * value / 1e12},
        "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": int(theta_host.numel() * 8),
                "d2h_bytes_per_step": int(res.numel() * 8)},
        "gpu_launches": int(launches),
        "clocks": clk,
    }
    # expressibility of the last step's first S states at the configured bins and at the reference's own bin
    # count int(0.0075 M) (measure.py:153: 150 bins for 20100 pairs), d = 2^N Haar reference (not timed)
    M = S * (S - 1) // 2
    ref_bins = max(1, int(0.0075 * M))
    expr = {"pairs": M}
    for nb in (a.nbins, ref_bins):
        _, cnt, edg = engine.allpairs_fidelity_hist(psi[:S], nb, keep_samples=False)
        kl = float(engine.expr_kl(cnt, edg, float(2 ** N)).item())
        expr[f"kl_{nb}_bins"] = kl if np.isfinite(kl) else None
        expr[f"counts_{nb}_bins_first_bin"] = int(cnt[0].item())
    if any(v is None for k, v in expr.items() if k.startswith("kl_")):
        expr["note"] = ("the reference's Haar density (d-1)(1-F)^(d-2) (measure.py:171-180) underflows to zero in "
                        f"every bin at d = 2^{N}, so its KL is nan (reported as null), as numpy gives it")
    line["expressibility"] = expr
    if not a.no_secondary:
        line["secondary"] = secondary_measures(a, dev, value, hbm_peak)
    if not a.no_cpu_baseline:
        # the oracle on one host core evaluates rows 0 and 1 of the benchmark's theta: the timed CPU baseline,
        # and the FP64 check of the double-float (value) and complex64 states of the same rows
        rows = theta_host[:2].numpy()
        ref, wall = _oracle_pool(1).apply(_oracle_rows, ((N, L, rows),))
        line["cpu_baseline"] = {"value": len(rows) / wall, "unit": UNIT, "cores": 1, "kind": "port",
                                "sample": f"{len(rows)} whole circuit evals (rows 0-1 of the benchmark's theta, "
                                          f"N={N} HE ladder, L={L}) on the numpy FP64 oracle, one thread, "
                                          f"{wall:.1f} s"}
        got = prog.run(theta[:2], 0).cpu().numpy()
        s64 = prog.run(theta[:2], 0, mode="c64").cpu().numpy().astype(np.complex128)

        def f01(x):
            return abs(np.vdot(x[0], x[1])) ** 2
        line["parity"] = {"rows": len(rows), "oracle": "numpy FP64 restatement of PQC.run (circuit.py:118-125)",
                          "c128_max_abs_amp_error": float(np.abs(got - ref).max()),
                          "c128_fidelity_error": abs(f01(got) - f01(ref)),
                          "c64_max_abs_amp_error": float(np.abs(s64 - ref).max()),
                          "c64_max_state_l2_error": float(np.linalg.norm(s64 - ref, axis=1).max()),
                          "c64_fidelity_error": abs(f01(s64) - f01(ref))}
    print(json.dumps(line), flush=True)
    if world > 1:
        dist.destroy_process_group()


def profile_case(name):
    """Small fixed workloads for ncu captures (a few launches of one kernel each)."""
    import torch

    import pyramaterised_gb300 as pq

    rng = np.random.default_rng(0)
    if name == "adjoint":  # adj_sweep_kernel: HE N=16 L=8, 16 rows, TFIM h=1, two calls
        c = pq.templates.hardware_efficient_ladder(16, 8)
        H = pq.hamiltonian.tfim_open(16, 1.0)
        th = torch.from_numpy(rng.random((16, c.n_columns())) * 2 * np.pi).cuda()
        for _ in range(2):
            E, g = c.program.energy_grad(th, H)
    elif name == "qfim":  # derivative states + Gram: HE N=16 L=8, P=256, two QFIMs
        c = pq.templates.hardware_efficient_ladder(16, 8)
        m = pq.measure.Measurements(c)
        c.run(list(rng.random(c.n_columns()) * 2 * np.pi))
        for _ in range(2):
            m.get_QFI()
    elif name == "fidgram":  # counts-only 20100-pair histogram, HE N=18 L=4, S=201: tensor-core vs FP32 tier
        import os

        c = pq.templates.hardware_efficient_ladder(18, 4)
        psi = c.run_batch(rng.random((201, c.n_columns())) * 2 * np.pi)
        res = {}
        for tier in ("tensor", "fp32"):
            if tier == "fp32":
                os.environ["PQC_NO_TENSOR_GRAM"] = "1"
            for _ in range(2):
                pq.engine.allpairs_fidelity_hist(psi, 75, keep_samples=False)
            torch.cuda.synchronize()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            for _ in range(3):
                counts = pq.engine.allpairs_fidelity_hist(psi, 75, keep_samples=False)[1]
            e1.record()
            torch.cuda.synchronize()
            res[tier + "_ms"] = e0.elapsed_time(e1) / 3
            res[tier + "_counts"] = counts.cpu().tolist()
        os.environ.pop("PQC_NO_TENSOR_GRAM", None)
        assert res["tensor_counts"] == res["fp32_counts"]
        print(json.dumps({"profile_case": name, "tensor_ms": res["tensor_ms"], "fp32_ms": res["fp32_ms"]}))
        return
    elif name == "pipes":  # FP64 vs FP32 arithmetic rates on this GPU, through cuBLAS GEMMs (n = 8192)
        n = 8192
        res = {}
        for dt in (torch.float64, torch.float32):
            a = torch.randn(n, n, dtype=dt, device="cuda")
            b = torch.randn(n, n, dtype=dt, device="cuda")
            torch.matmul(a, b)
            torch.cuda.synchronize()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            for _ in range(5):
                torch.matmul(a, b)
            e1.record()
            torch.cuda.synchronize()
            res[str(dt).split(".")[-1] + "_gemm_tflops"] = 5 * 2 * n ** 3 / (e0.elapsed_time(e1) / 1e3) / 1e12
        print(json.dumps({"profile_case": name, "tf32_allowed": torch.backends.cuda.matmul.allow_tf32, **res}))
        return
    else:
        raise SystemExit(f"unknown profile case {name!r}")
    torch.cuda.synchronize()
    print(json.dumps({"profile_case": name, "ok": True}))


def main():
    a = parse()
    if a.profile_case:
        profile_case(a.profile_case)
        return
    if a.impl == "reference":
        run_reference(a)
    else:
        run_ours(a)


if __name__ == "__main__":
    main()
