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


class Staging:
    """Pinned host buffers of one stream slot, reused by every batch that runs on that slot.

    A batch packs all of its host inputs (angle rows, op limits) into `h2d` and sends them with one asynchronous
    copy, and gathers all of its results on the device into one vector that one asynchronous copy returns into
    `d2h`.  A slot takes its next batch only after the previous batch's completion event, by which time both
    copies of that batch are done, so the buffers are reused without synchronising the host.  They grow (a new
    pinned allocation) only when a batch needs more than any earlier one."""

    ALIGN = 256

    def __init__(self, h2d_bytes=1 << 20, d2h_values=1 << 17):
        self.h2d = torch.empty(int(h2d_bytes), dtype=torch.uint8).pin_memory()
        self.d2h = torch.empty(int(d2h_values), dtype=torch.float64).pin_memory()

    def upload(self, arrays, dev):
        """Device tensors holding `arrays` (numpy), sent with one copy on the current stream."""
        offs, total = [], 0
        for a in arrays:
            offs.append(total)
            total += -(-a.nbytes // self.ALIGN) * self.ALIGN
        if total > self.h2d.numel():
            self.h2d = torch.empty(2 * total, dtype=torch.uint8).pin_memory()
        host = self.h2d.numpy()
        for a, o in zip(arrays, offs):
            host[o:o + a.nbytes] = np.ascontiguousarray(a).reshape(-1).view(np.uint8)
        dbuf = torch.empty(max(total, 1), dtype=torch.uint8, device=dev)
        dbuf[:total].copy_(self.h2d[:total], non_blocking=True)
        return [dbuf[o:o + a.nbytes].view(_TORCH_DTYPE[a.dtype.str]).reshape(a.shape) for a, o in zip(arrays, offs)]

    def download(self, flat):
        """Start the copy of the device vector `flat` (float64) into the pinned buffer; returns its host view
        (valid once the stream has passed the copy)."""
        n = flat.numel()
        if n > self.d2h.numel():
            self.d2h = torch.empty(2 * n, dtype=torch.float64).pin_memory()
        self.d2h[:n].copy_(flat, non_blocking=True)
        return self.d2h[:n].numpy()


_TORCH_DTYPE = {np.dtype(np.float64).str: torch.float64, np.dtype(np.int32).str: torch.int32,
                np.dtype(np.int64).str: torch.int64}


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


def take_small_batch(queue, free_bytes, max_rows, max_batch_bytes, max_qubits):
    """Pop the fidelity and Meyer-Wallach requests of every family of at most `max_qubits` qubits, in arrival
    order, within `max_rows` state rows and min(free_bytes, max_batch_bytes) of HBM (the first one whenever it
    fits free_bytes); they run as one `MultiBatch`.  The requests left behind keep their order."""
    take, rest = [], []
    rows = nbytes = 0
    for r in queue:
        if r.kind not in ("fidelity", "mw") or r.n_qubits > max_qubits:
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


def _state_rows(fam, reqs):
    """Angle rows and op limits of the fidelity pairs (rows 2j, 2j + 1) then the MW rows of one family."""
    fid = [r for r in reqs if r.kind == "fidelity"]
    mws = [r for r in reqs if r.kind == "mw"]
    rows = [t for r in fid for t in r.theta] + [r.theta for r in mws]
    lims = [fam.op_limit[r.layers] for r in fid for _ in range(2)] + [fam.op_limit[r.layers] for r in mws]
    return fid, mws, fam.pad(rows), np.array(lims, dtype=np.int32)


class Batch:
    """Requests of one family launched together on one stream slot.

    `launch` enqueues everything on the slot's stream without waiting for the device: one packed input copy, the
    kernels, one packed result copy and the completion event.  `results` reads the pinned result buffer after
    the event (no device synchronisation)."""

    def __init__(self, fam, reqs, slot):
        self.fam, self.reqs = fam, reqs
        self.stream, self.staging = slot
        self.slot = slot
        self.layout = []  # (rid, kind, offset(s), size, shape) in the packed result vector
        self.host = None
        self.event = torch.cuda.Event()
        self.bytes = sum(request_bytes(r) for r in reqs)

    def launch(self):
        fam = self.fam
        dev = engine.device()
        parts, pos = [], 0

        def add(t):
            """Offset of t's values in the packed result vector."""
            nonlocal pos
            t = t.reshape(-1)
            parts.append(t)
            pos += t.numel()
            return pos - t.numel()

        with torch.cuda.stream(self.stream):
            fid = [r for r in self.reqs if r.kind == "fidelity"]
            mws = [r for r in self.reqs if r.kind == "mw"]
            e_reqs = [r for r in self.reqs if r.kind == "energy"]
            q_reqs = [r for r in self.reqs if r.kind == "qfim"]
            host = []
            if fid or mws:  # fidelity pairs first (rows 2j, 2j + 1), then the MW rows
                host += list(_state_rows(fam, fid + mws)[2:])
            if e_reqs:
                host += [fam.pad([r.theta for r in e_reqs]),
                         np.array([fam.op_limit[r.layers] for r in e_reqs], dtype=np.int32)]
            host += [np.ascontiguousarray(r.theta[None, :], dtype=np.float64) for r in q_reqs]
            dev_in = self.staging.upload(host, dev)
            k = 0
            if fid or mws:
                theta, lim = dev_in[0:2]
                k = 2
                X = fam.program.run(theta, row_limit=lim)
                nf = 2 * len(fid)
                if fid:
                    ov = engine.overlaps(X, X, torch.arange(0, nf, 2, device=dev), torch.arange(1, nf, 2, device=dev))
                    o = add(ov.real ** 2 + ov.imag ** 2)
                    self.layout += [(r.rid, "scalar", o + j, 1, None) for j, r in enumerate(fid)]
                if mws:
                    o = add(engine.mw(X[nf:]))
                    self.layout += [(r.rid, "scalar", o + j, 1, None) for j, r in enumerate(mws)]
            if e_reqs:
                theta, lim = dev_in[k:k + 2]
                k += 2
                E, G = fam.program.energy_grad(theta, fam.H, row_limit=lim)
                oe, og, nc = add(E), add(G), G.shape[1]
                self.layout += [(r.rid, "energy", (oe + j, og + j * nc), r.theta.shape[-1], None)
                                for j, r in enumerate(e_reqs)]
            for r in q_reqs:
                prog = fam.exact(r.layers)
                th = dev_in[k]
                k += 1
                P = r.theta.shape[-1]
                o = add(engine.qfim(prog.run(th), prog.gradient_states(th)))
                self.layout.append((r.rid, "matrix", o, P * P, (P, P)))
            flat = torch.cat(parts) if parts else torch.zeros(1, dtype=torch.float64, device=dev)
            self.host = self.staging.download(flat)
            self.event.record(self.stream)

    def results(self):
        res = {}
        for rid, kind, off, n, shape in self.layout:
            if kind == "scalar":
                res[rid] = float(self.host[off])
            elif kind == "energy":
                oe, og = off
                res[rid] = (float(self.host[oe]), self.host[og:og + n].copy())
            else:
                res[rid] = self.host[off:off + n].reshape(shape).copy()
        return res


class MultiBatch(Batch):
    """Fidelity and Meyer-Wallach requests of several small families on one stream slot: their circuits run
    with shared launches (`engine.run_multi`: one coefficient launch, one conversion launch and one sweep
    launch for every family of up to 13 qubits), then each family's overlaps and MW reductions."""

    def __init__(self, families, reqs, slot):
        super().__init__(None, reqs, slot)
        self.families = families

    def launch(self):
        dev = engine.device()
        groups = {}
        for r in self.reqs:
            groups.setdefault((r.ansatz, r.n_qubits), []).append(r)
        parts, pos = [], 0

        def add(t):
            nonlocal pos
            t = t.reshape(-1)
            parts.append(t)
            pos += t.numel()
            return pos - t.numel()

        with torch.cuda.stream(self.stream):
            plan, host = [], []
            for key, reqs in groups.items():
                fam = self.families.get(*key)
                fid, mws, th, lim = _state_rows(fam, reqs)
                plan.append((fam, fid, mws))
                host += [th, lim]
            dev_in = self.staging.upload(host, dev)
            states = engine.run_multi([(fam.program, dev_in[2 * i], None, dev_in[2 * i + 1])
                                       for i, (fam, _, _) in enumerate(plan)])
            for (fam, fid, mws), X in zip(plan, states):
                nf = 2 * len(fid)
                if fid:
                    ov = engine.overlaps(X, X, torch.arange(0, nf, 2, device=dev), torch.arange(1, nf, 2, device=dev))
                    o = add(ov.real ** 2 + ov.imag ** 2)
                    self.layout += [(r.rid, "scalar", o + j, 1, None) for j, r in enumerate(fid)]
                if mws:
                    o = add(engine.mw(X[nf:]))
                    self.layout += [(r.rid, "scalar", o + j, 1, None) for j, r in enumerate(mws)]
            self.host = self.staging.download(torch.cat(parts))
            self.event.record(self.stream)


class Server:
    """Continuous batching: batches per (ansatz, N) on a pool of streams, admitted by HBM budget; fidelity and
    MW requests of families of up to `multi_max_qubits` qubits share batches across families (MultiBatch)."""

    def __init__(self, hbm_budget=48 << 30, n_streams=4, max_rows=256, max_batch_bytes=8 << 30, slots=None,
                 batch_cls=None, families=None, multi_max_qubits=13, multi_cls=None):
        """slots / batch_cls / families / multi_cls replace the CUDA stream slots, the batch executors and the
        program cache (the host loop can then run with the device work stubbed out); multi_max_qubits 0 keeps
        every batch to one family."""
        self.multi_max_qubits = int(multi_max_qubits)
        self.multi_cls = multi_cls or MultiBatch
        self.hbm_budget = int(hbm_budget)
        self.max_rows = int(max_rows)
        self.max_batch_bytes = int(max_batch_bytes)
        self.slots = list(slots) if slots is not None else [(torch.cuda.Stream(), Staging()) for _ in range(n_streams)]
        self.batch_cls = batch_cls or Batch
        self.families = families or Families()

    def prepare(self, requests):
        """Build every program and derivative / adjoint plan the stream needs, then run warm-up batches (outside
        the timed loop): one request of every (family, kind) on the first slot and one of every kind on each other
        slot.  The first launch of a kernel in a process (ours, and torch's around them, which the driver may
        have to load on first use: seconds on a fresh machine) and the first allocations on each slot's stream
        are paid here instead of by the first requests of the stream."""
        seen = set()
        warm = {}
        for r in requests:
            fam = self.families.get(r.ansatz, r.n_qubits)
            warm.setdefault((r.ansatz, r.n_qubits, r.kind), r)
            if r.kind == "qfim" and (r.ansatz, r.n_qubits, r.layers) not in seen:
                seen.add((r.ansatz, r.n_qubits, r.layers))
                prog = fam.exact(r.layers)
                prog.gradient_states(np.zeros((1, prog.n_params)))
            if r.kind == "energy" and (r.ansatz, r.n_qubits, "e") not in seen:
                seen.add((r.ansatz, r.n_qubits, "e"))
                fam.program.energy_grad(np.zeros((1, fam.P)), fam.H)
        smallest = {}
        for r in warm.values():
            if r.kind not in smallest or r.n_qubits < smallest[r.kind].n_qubits:
                smallest[r.kind] = r
        small = [r for r in warm.values() if r.kind in ("fidelity", "mw") and r.n_qubits <= self.multi_max_qubits]
        for i, slot in enumerate(self.slots):
            batches = [self.batch_cls(self.families.get(r.ansatz, r.n_qubits), [r], slot)
                       for r in (warm.values() if i == 0 else smallest.values())]
            if small:
                batches.append(self.multi_cls(self.families, small, slot))
            for b in batches:
                b.launch()
                b.event.synchronize()
                b.results()
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
        free = list(self.slots)
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
                    free.append(b.slot)
                    inflight.remove(b)
                    progressed = True
            while free and waiting:
                head = waiting[0]
                small = head.kind in ("fidelity", "mw") and head.n_qubits <= self.multi_max_qubits
                if small:
                    take = take_small_batch(waiting, self.hbm_budget - used, self.max_rows, self.max_batch_bytes,
                                            self.multi_max_qubits)
                else:
                    take = take_batch(waiting, self.hbm_budget - used, self.max_rows, self.max_batch_bytes)
                if not take:
                    break
                if small:
                    b = self.multi_cls(self.families, take, free.pop(0))
                else:
                    fam = self.families.get(take[0].ansatz, take[0].n_qubits)
                    b = self.batch_cls(fam, take, free.pop(0))
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
        """Build the programs and plans, then serve one request of every (family, kind) as a warm-up (as
        `Server.prepare` does)."""
        warm = {}
        for r in requests:
            fam = self.families.get(r.ansatz, r.n_qubits)
            prog = fam.exact(r.layers)
            warm.setdefault((r.ansatz, r.n_qubits, r.kind), r)
            if r.kind == "qfim":
                prog.gradient_states(np.zeros((1, prog.n_params)), plain=True)
            if r.kind == "energy":
                prog.energy_grad(np.zeros((1, prog.n_params)), fam.H, plain=True)
        for r in warm.values():
            self.one(r)
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
