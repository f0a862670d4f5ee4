"""Continuous-batching request loop for measure requests on one GPU.

A request asks for one measure of one circuit from a family (ansatz, N):
  fidelity  |<psi(theta_a)|psi(theta_b)>|^2        (measure.py:123-139, one pair)
  mw        Meyer-Wallach Q of psi(theta)           (measure.py:226-237)
  energy    <H> and d<H>/dtheta for TFIM h=1        (measure.py:461-471, circuit.py:132-137)
  qfim      the P x P QFIM of psi(theta), P <= 128  (measure.py:33-71)
with depth `layers` (1..2N).  The reference evaluates each request as its own
QuTiP circuit; here requests of one family share one program built at the
family's maximum depth 2N and run together, each row cut to its own depth by a
per-row op limit (pqc_run_limited / pqc_energy_grad row_limit).  QFIM requests
run on exact-depth programs (their derivative plans are cached per depth).

`Server.run` admits requests as they arrive while earlier batches are still on
the GPU: each batch goes to its own CUDA stream, so batches overlap on the
device, and a request is admitted as soon as a stream is free and its states
fit the HBM budget (16 B x 2^N per state, plus derivative states, adjoint
buffers and measure workspaces).  `PlainServer` is the comparison: first in,
first out, one request at a time, one circuit per launch sequence, FP64 op by
op.  Every row of a batched call is computed independently of the other rows,
so a request's result does not depend on what it was batched with.
"""
from __future__ import annotations

import math
import time
from collections import OrderedDict, deque
from dataclasses import dataclass

import numpy as np
import torch

from . import engine, templates
from .hamiltonian import tfim_open

KINDS = ("fidelity", "mw", "energy", "qfim")
ANSATZE = ("he", "tfim")


# ---------------------------------------------------------------------- requests
@dataclass
class Request:
    rid: int
    kind: str
    n_qubits: int
    ansatz: str
    layers: int
    theta: np.ndarray      # [P] (or [2, P] for fidelity), P = params of `layers` layers
    arrival: float = 0.0   # seconds after the start of the stream


@dataclass
class Result:
    rid: int
    value: object          # float, (E, grad[P]) or QFIM [P, P] (numpy)
    done: float            # seconds after the start of the stream
    latency: float


def params_per_layer(ansatz, N):
    return 2 * N if ansatz == "he" else 2 * N - 1


def build_ansatz(ansatz, N, L):
    if ansatz == "he":
        return templates.hardware_efficient_ladder(N, L)
    if ansatz == "tfim":
        return templates.tfim_style(N, L)
    raise ValueError(f"unknown ansatz {ansatz!r}")


def synthetic_stream(n, rate, seed=0, n_range=(6, 22), mix=(0.4, 0.3, 0.2, 0.1), qfim_max_params=128):
    """Seeded stream of `n` requests with Poisson arrivals at `rate` per second.

    Qubit count uniform over n_range, ansatz HE or TFIM-style with equal odds, depth uniform over
    2..2N layers (QFIM requests: up to the depth that keeps P <= qfim_max_params), kind drawn from
    `mix` (fidelity, mw, energy, qfim), angles uniform on [0, 2 pi)."""
    rng = np.random.default_rng(seed)
    t = np.cumsum(rng.exponential(1.0 / rate, n)) if rate > 0 else np.zeros(n)
    out = []
    p = np.asarray(mix, dtype=np.float64)
    p = p / p.sum()
    for i in range(n):
        N = int(rng.integers(n_range[0], n_range[1] + 1))
        ansatz = ANSATZE[int(rng.integers(0, 2))]
        kind = KINDS[int(rng.choice(4, p=p))]
        ppl = params_per_layer(ansatz, N)
        lmax = 2 * N if kind != "qfim" else max(1, min(2 * N, qfim_max_params // ppl))
        L = int(rng.integers(min(2, lmax), lmax + 1))
        rows = 2 if kind == "fidelity" else 1
        th = rng.random((rows, L * ppl)) * 2 * np.pi
        out.append(Request(i, kind, N, ansatz, L, th if rows == 2 else th[0], float(t[i])))
    return out


# ---------------------------------------------------------------------- programs
class Family:
    """Programs of one (ansatz, N): the maximum-depth program with per-depth op limits, exact-depth programs
    (built on demand), and the TFIM Hamiltonian of the energy requests."""

    def __init__(self, ansatz, N):
        self.ansatz, self.N = ansatz, N
        self.lmax = 2 * N
        self.ppl = params_per_layer(ansatz, N)
        full = build_ansatz(ansatz, N, self.lmax)
        self.program = full.program
        gpl = len(full.gates) // self.lmax
        last = self.program.lowered.gate_last
        self.op_limit = [0] + [last[L * gpl - 1] + 1 for L in range(1, self.lmax + 1)]
        for v in self.op_limit:  # layer boundaries never cut a fused CNOT-RZ-CNOT triple
            if not self.program.lib.pqc_program_limit_ok(self.program.handle, int(v)):
                raise ValueError(f"layer boundary {v} is not a valid op limit")
        self.P = self.program.n_params
        self.H = tfim_open(N, 1.0)
        self._exact = OrderedDict()

    def exact(self, L):
        p = self._exact.get(L)
        if p is None:
            p = build_ansatz(self.ansatz, self.N, L).program
            self._exact[L] = p
        return p

    def pad(self, theta_rows):
        """[R, P_L] angle rows -> [R, P] (zeros beyond each row's depth: those ops are cut off)."""
        out = np.zeros((len(theta_rows), self.P))
        for i, t in enumerate(theta_rows):
            out[i, :len(t)] = t
        return out


class Families:
    def __init__(self):
        self._f = {}

    def get(self, ansatz, N):
        k = (ansatz, N)
        f = self._f.get(k)
        if f is None:
            f = Family(ansatz, N)
            self._f[k] = f
        return f


def _pinned(a, dtype):
    t = torch.from_numpy(np.ascontiguousarray(a, dtype=dtype))
    return t.pin_memory().to(engine.device(), non_blocking=True)


# ---------------------------------------------------------------------- batch execution
def state_bytes(N):
    return 16 << N


def request_bytes(req):
    """HBM held by a request while it runs (states, derivative states, adjoint buffers, workspaces)."""
    S = state_bytes(req.n_qubits)
    P = req.theta.shape[-1]
    if req.kind == "fidelity":
        return 2 * S + 256
    if req.kind == "mw":
        return S + 4096
    if req.kind == "energy":
        # psi, lambda, the output state of the workspace and the per-tile measure partials
        tiles = 1 << max(0, req.n_qubits - 11)
        return 3 * S + 8 * tiles * P + 64 * P
    return (P + 2) * S + 16 * P * P


def request_rows(req):
    """State rows a request occupies in its batch."""
    if req.kind == "fidelity":
        return 2
    if req.kind == "qfim":
        return req.theta.shape[-1] + 1
    return 1


def take_batch(queue, free_bytes, max_rows, max_batch_bytes):
    """Pop from `queue` (a deque in arrival order) the requests of one batch: the family (ansatz, N) of the
    request waiting longest, in arrival order, while the batch stays within `max_rows` state rows and within
    min(free_bytes, max_batch_bytes) of HBM.  The first request is taken whenever it fits `free_bytes`.
    The requests left behind keep their order."""
    if not queue:
        return []
    head = queue[0]
    key = (head.ansatz, head.n_qubits)
    take, rest = [], []
    rows = nbytes = 0
    for r in queue:
        if (r.ansatz, r.n_qubits) != key:
            rest.append(r)
            continue
        rb, nr = request_bytes(r), request_rows(r)
        fits = rb <= free_bytes if not take else (rows + nr <= max_rows and nbytes + rb <= min(free_bytes, max_batch_bytes))
        if fits:
            take.append(r)
            rows += nr
            nbytes += rb
        else:
            rest.append(r)
    queue.clear()
    queue.extend(rest)
    return take


class Batch:
    """Requests of one family launched together on one stream."""

    def __init__(self, fam, reqs, stream):
        self.fam, self.reqs, self.stream = fam, reqs, stream
        self.out = {}
        self.event = torch.cuda.Event()
        self.bytes = sum(request_bytes(r) for r in reqs)

    def launch(self):
        fam = self.fam
        with torch.cuda.stream(self.stream):
            state_reqs = [r for r in self.reqs if r.kind in ("fidelity", "mw")]
            if state_reqs:
                rows, lims = [], []
                for r in state_reqs:
                    th = r.theta if r.kind == "fidelity" else r.theta[None, :]
                    rows += list(th)
                    lims += [fam.op_limit[r.layers]] * len(th)
                theta = _pinned(fam.pad(rows), np.float64)
                lim = _pinned(np.array(lims), np.int32)
                X = fam.program.run(theta, row_limit=lim)
                fid_rows, mw_rows, pos = [], [], 0
                for r in state_reqs:
                    if r.kind == "fidelity":
                        fid_rows.append(pos)
                        pos += 2
                    else:
                        mw_rows.append(pos)
                        pos += 1
                if fid_rows:
                    ia = _pinned(np.array(fid_rows), np.int64)
                    ov = engine.overlaps(X, X, ia, ia + 1)
                    F = ov.real ** 2 + ov.imag ** 2
                    k = 0
                    for r in state_reqs:
                        if r.kind == "fidelity":
                            self.out[r.rid] = F[k]
                            k += 1
                if mw_rows:
                    Q = engine.mw(X[_pinned(np.array(mw_rows), np.int64)])
                    k = 0
                    for r in state_reqs:
                        if r.kind == "mw":
                            self.out[r.rid] = Q[k]
                            k += 1
            e_reqs = [r for r in self.reqs if r.kind == "energy"]
            if e_reqs:
                theta = _pinned(fam.pad([r.theta for r in e_reqs]), np.float64)
                lim = _pinned(np.array([fam.op_limit[r.layers] for r in e_reqs]), np.int32)
                E, G = fam.program.energy_grad(theta, fam.H, row_limit=lim)
                for k, r in enumerate(e_reqs):
                    self.out[r.rid] = (E[k], G[k, :r.theta.shape[-1]])
            for r in self.reqs:
                if r.kind == "qfim":
                    prog = fam.exact(r.layers)
                    th = _pinned(r.theta[None, :], np.float64)
                    psi = prog.run(th)
                    dpsi = prog.gradient_states(th)
                    self.out[r.rid] = engine.qfim(psi, dpsi)
            self.event.record(self.stream)

    def results(self):
        res = {}
        for rid, v in self.out.items():
            if isinstance(v, tuple):
                res[rid] = (float(v[0]), v[1].cpu().numpy())
            elif v.dim() == 2:
                res[rid] = v.cpu().numpy()
            else:
                res[rid] = float(v)
        return res


class Server:
    """Continuous batching: batches per (ansatz, N) on a pool of streams, admitted by HBM budget."""

    def __init__(self, hbm_budget=48 << 30, n_streams=4, max_rows=256, max_batch_bytes=8 << 30):
        self.hbm_budget = int(hbm_budget)
        self.max_rows = int(max_rows)
        self.max_batch_bytes = int(max_batch_bytes)
        self.streams = [torch.cuda.Stream() for _ in range(n_streams)]
        self.families = Families()

    def prepare(self, requests):
        """Build every program and derivative / adjoint plan the stream needs (outside the timed loop)."""
        seen = set()
        for r in requests:
            fam = self.families.get(r.ansatz, r.n_qubits)
            if r.kind == "qfim" and (r.ansatz, r.n_qubits, r.layers) not in seen:
                seen.add((r.ansatz, r.n_qubits, r.layers))
                prog = fam.exact(r.layers)
                prog.gradient_states(np.zeros((1, prog.n_params)))
            if r.kind == "energy" and (r.ansatz, r.n_qubits, "e") not in seen:
                seen.add((r.ansatz, r.n_qubits, "e"))
                fam.program.energy_grad(np.zeros((1, fam.P)), fam.H)
        torch.cuda.synchronize()

    def run(self, requests, realtime=True):
        """Serve `requests` (sorted by arrival); returns {rid: Result}.  realtime=False admits every request at
        time 0 (offline throughput)."""
        reqs = sorted(requests, key=lambda r: r.arrival)
        for r in reqs:
            if request_bytes(r) > self.hbm_budget:
                raise ValueError(f"request {r.rid} needs {request_bytes(r)} bytes, over the HBM budget")
        results = {}
        waiting = deque()
        inflight = []
        free = list(self.streams)
        used = 0
        i = 0
        t0 = time.perf_counter()
        while i < len(reqs) or waiting or inflight:
            now = time.perf_counter() - t0
            while i < len(reqs) and (not realtime or reqs[i].arrival <= now):
                waiting.append(reqs[i])
                i += 1
            progressed = False
            for b in list(inflight):
                if b.event.query():
                    done = time.perf_counter() - t0
                    for rid, v in b.results().items():
                        arr = b.arrival[rid]
                        results[rid] = Result(rid, v, done, done - arr)
                    used -= b.bytes
                    free.append(b.stream)
                    inflight.remove(b)
                    progressed = True
            while free and waiting:
                take = take_batch(waiting, self.hbm_budget - used, self.max_rows, self.max_batch_bytes)
                if not take:
                    break
                fam = self.families.get(take[0].ansatz, take[0].n_qubits)
                b = Batch(fam, take, free.pop(0))
                b.arrival = {r.rid: (r.arrival if realtime else 0.0) for r in take}
                b.launch()
                used += b.bytes
                inflight.append(b)
                progressed = True
            if not progressed:
                nxt = reqs[i].arrival - (time.perf_counter() - t0) if (realtime and i < len(reqs)) else 1.0
                time.sleep(max(0.0, min(nxt, 2e-4)))
        return results


class PlainServer:
    """First in, first out; one request at a time; each circuit run op by op in FP64 (one kernel per op)."""

    def __init__(self):
        self.families = Families()

    def prepare(self, requests):
        for r in requests:
            fam = self.families.get(r.ansatz, r.n_qubits)
            prog = fam.exact(r.layers)
            if r.kind == "qfim":
                prog.gradient_states(np.zeros((1, prog.n_params)), plain=True)
            if r.kind == "energy":
                prog.energy_grad(np.zeros((1, prog.n_params)), fam.H, plain=True)
        torch.cuda.synchronize()

    def one(self, r):
        fam = self.families.get(r.ansatz, r.n_qubits)
        prog = fam.exact(r.layers)
        if r.kind == "fidelity":
            a = prog.run(r.theta[0][None, :], mode="plain")
            b = prog.run(r.theta[1][None, :], mode="plain")
            return float(engine.fidelity_pairs(a, b)[0])
        if r.kind == "mw":
            return float(engine.mw(prog.run(r.theta[None, :], mode="plain"))[0])
        if r.kind == "energy":
            E, G = prog.energy_grad(r.theta[None, :], fam.H, plain=True)
            return float(E[0]), G[0].cpu().numpy()
        psi = prog.run(r.theta[None, :], mode="plain")
        dpsi = prog.gradient_states(r.theta[None, :], plain=True)
        return engine.qfim(psi, dpsi).cpu().numpy()

    def run(self, requests, realtime=True):
        reqs = sorted(requests, key=lambda r: r.arrival)
        results = {}
        t0 = time.perf_counter()
        for r in reqs:
            if realtime:
                wait = r.arrival - (time.perf_counter() - t0)
                if wait > 0:
                    time.sleep(wait)
            v = self.one(r)
            torch.cuda.synchronize()
            done = time.perf_counter() - t0
            arr = r.arrival if realtime else 0.0
            results[r.rid] = Result(r.rid, v, done, done - arr)
        return results


def latency_summary(results, wall=None):
    lat = np.array([r.latency for r in results.values()])
    span = wall if wall is not None else max(r.done for r in results.values())
    return {"requests": len(lat), "p50_ms": float(np.percentile(lat, 50) * 1e3),
            "p99_ms": float(np.percentile(lat, 99) * 1e3), "mean_ms": float(lat.mean() * 1e3),
            "requests_per_s": len(lat) / span if span > 0 else math.inf}
