"""Device-side engine calls on torch tensors.

Thin host layer over the C ABI: it owns program handles, allocates
caller-side workspaces from torch's caching allocator, and launches on
torch's current CUDA stream.  There is no CPU path: without a CUDA device or
the built library every call raises `EngineError`.
"""
import ctypes as C
import math

import numpy as np
import torch

from . import _lib
from ._lib import EngineError, check
from .lowering import Lowered

__all__ = ["Program", "EngineError", "device", "fidelity_pairs", "allpairs_fidelity_hist", "histogram",
           "expr_kl", "mw", "expect", "magic", "qfim", "overlaps", "hist_edges"]


def device():
    if not torch.cuda.is_available():
        raise EngineError("pyramaterised_gb300 needs a CUDA device (GB300); there is no CPU fallback")
    return torch.device("cuda", torch.cuda.current_device())


def _stream():
    return C.c_void_p(torch.cuda.current_stream().cuda_stream)


def _p(t):
    return C.c_void_p(t.data_ptr()) if t is not None else C.c_void_p(0)


def _to_dev(arr, dtype, dev):
    """Host array -> device tensor through pinned memory with an asynchronous copy (a pageable copy would
    wait for the stream's earlier work)."""
    t = torch.from_numpy(np.ascontiguousarray(arr, dtype=dtype))
    return t.pin_memory().to(dev, non_blocking=True)


def _ws(nbytes, dev):
    return torch.empty(max(int(nbytes), 256), dtype=torch.uint8, device=dev)


def _c128(x, dev):
    t = torch.as_tensor(x)
    if t.dtype != torch.complex128:
        t = t.to(torch.complex128)
    return t.to(dev).contiguous()


def _f64(x, dev):
    t = torch.as_tensor(x)
    if t.dtype != torch.float64:
        t = t.to(torch.float64)
    return t.to(dev).contiguous()


class Program:
    """A lowered, planned circuit on the device (`pqc_program`)."""

    def __init__(self, gates, n_qubits, tile_qubits=0):
        self.lib = _lib.load()
        self.dev = device()
        self.N = int(n_qubits)
        self.D = 1 << self.N
        self.lowered = Lowered(gates, self.N)
        self.n_params = self.lowered.n_params
        ops = np.ascontiguousarray(self.lowered.ops)
        self._ops = ops
        h = C.c_void_p()
        check(self.lib.pqc_program_create(ops.ctypes.data if len(ops) else None, len(ops), self.N, self.n_params,
                                          int(tile_qubits), C.byref(h)))
        self.handle = h
        self._grad_cache = None
        self._egrad_cache = None

    def __del__(self):
        h = getattr(self, "handle", None)
        if h is not None and h.value:
            try:
                self.lib.pqc_program_destroy(h)
            except Exception:
                pass
            self.handle = None

    def limits(self, row_limit, rows):
        """Per-row op limits as a device int32 tensor.  Host arrays are checked with pqc_program_limit_ok (a
        limit may not cut a CNOT-RZ-CNOT triple that the plan applies as one ZZ rotation); a CUDA tensor is
        taken as given, so its values must come from such checked limits."""
        if isinstance(row_limit, torch.Tensor) and row_limit.is_cuda:
            lim = row_limit.to(torch.int32).contiguous()
        else:
            arr = np.ascontiguousarray(np.asarray(row_limit, dtype=np.int32).reshape(-1))
            for v in np.unique(arr):
                if not self.lib.pqc_program_limit_ok(self.handle, int(v)):
                    raise ValueError(f"op limit {int(v)} cuts a CNOT-RZ-CNOT triple that runs as one ZZ rotation")
            lim = _to_dev(arr, np.int32, self.dev)
        if lim.numel() != rows:
            raise ValueError("row_limit needs one entry per row")
        return lim

    def set_occupancy(self, ctas_per_sm):
        """Sweep launch shape below 2^13-amplitude tiles: 3 (default) or 2 resident CTAs per SM."""
        self.set_launch(ctas_per_sm, 0)

    def set_launch(self, ctas_per_sm, threads=0):
        """Sweep launch shape below 2^13-amplitude tiles: (ctas_per_sm, threads) in (3, 128), (3, 256) or
        (2, 256); threads 0 (the default) takes 128 on grids of at least 2048 tiles and 256 below."""
        check(self.lib.pqc_program_set_launch(self.handle, int(ctas_per_sm), int(threads)))
        self.ctas_per_sm = int(ctas_per_sm)
        self.sweep_threads = int(threads)

    def info(self):
        ns, tq = C.c_int32(), C.c_int32()
        check(self.lib.pqc_program_info(self.handle, C.byref(ns), C.byref(tq)))
        return {"n_sweeps": ns.value, "tile_qubits": tq.value, "n_ops": len(self._ops)}

    def status(self):
        """Status bits raised by this program's kernels since the last call (0: every run was valid);
        reading synchronises the device.  Bit 1 (`_lib.PQC_STATUS_LOAD_TIMEOUT`): a bulk tile load timed out."""
        v = C.c_int32()
        check(self.lib.pqc_program_status(self.handle, C.byref(v)))
        return v.value

    # ------------------------------------------------------------------ init state
    def _psi0(self, psi0):
        """(pointer tensor or None, basis index)."""
        if psi0 is None:
            return None, 0
        if isinstance(psi0, (int, np.integer)):
            return None, int(psi0)
        t = _c128(psi0, self.dev).reshape(-1)
        if t.numel() != self.D:
            raise ValueError(f"initial state has {t.numel()} amplitudes, expected {self.D}")
        return t, 0

    def _theta(self, theta):
        th = _f64(theta, self.dev)
        if th.dim() == 1:
            th = th.reshape(1, -1)
        if th.shape[1] != self.n_params:
            raise ValueError(f"expected {self.n_params} parameters per row, got {th.shape[1]}")
        return th

    # ------------------------------------------------------------------ forward
    def run(self, theta, psi0=None, mode="c128", out=None, row_limit=None):
        """States [B, 2^N] for parameter rows theta [B, P].

        mode: c128 (fused sweeps, double-float arithmetic), f64 (the same sweeps in native FP64), c64 (FP32
        sampling mode) or plain (one FP64 kernel per op).

        row_limit: optional int32 [B]; row b applies only ops with index < row_limit[b]."""
        th = self._theta(theta)
        B = th.shape[0]
        p0, idx = self._psi0(psi0)
        dt = torch.complex64 if mode == "c64" else torch.complex128
        if out is None:
            out = torch.empty((B, self.D), dtype=dt, device=self.dev)
        ws = _ws(self.lib.pqc_run_workspace_size(self.handle, B), self.dev)
        if row_limit is not None:
            if mode != "c128":
                raise ValueError("row limits are supported by the c128 path")
            lim = self.limits(row_limit, B)
            check(self.lib.pqc_run_limited(self.handle, _p(th) if self.n_params else None, self.n_params, B, _p(p0),
                                           idx, _p(lim), _p(out), _p(ws), ws.numel(), _stream()))
            return out
        fn = {"c128": self.lib.pqc_run, "f64": self.lib.pqc_run_fp64, "c64": self.lib.pqc_run_c64,
              "plain": self.lib.pqc_run_plain}[mode]
        check(fn(self.handle, _p(th) if self.n_params else None, self.n_params, B, _p(p0), idx, _p(out), _p(ws),
                 ws.numel(), _stream()))
        return out

    # ------------------------------------------------------------------ derivatives
    def derivative_states(self, theta, psi0, gens, after, n_rows, op_limit=None, plain=False):
        """Run r of the circuit with generator gens[r] inserted after op after[r], summed into row gens[r].sel.

        plain=True takes the one-kernel-per-op FP64 path (runs must map 1:1 onto rows, no op_limit)."""
        th = self._theta(theta)
        if th.shape[0] != 1:
            raise ValueError("derivative states take one parameter row")
        p0, idx = self._psi0(psi0)
        out = torch.empty((n_rows, self.D), dtype=torch.complex128, device=self.dev)
        if n_rows == 0:
            return out
        gens = np.ascontiguousarray(gens)
        after = np.ascontiguousarray(after, dtype=np.int32)
        if plain:
            if op_limit is not None or len(gens) != n_rows:
                raise ValueError("the plain path takes one run per row and no op limit")
            ws = _ws(self.lib.pqc_derivative_states_plain_workspace_size(self.handle, len(gens)), self.dev)
            check(self.lib.pqc_derivative_states_plain(self.handle, _p(th) if self.n_params else None, _p(p0), idx,
                                                       gens.ctypes.data, after.ctypes.data, len(gens), _p(out),
                                                       _p(ws), ws.numel(), _stream()))
            return out
        ws = _ws(self.lib.pqc_derivative_states_workspace_size(self.handle, len(gens), n_rows), self.dev)
        lim = None
        if op_limit is not None:
            lim = torch.full((len(gens),), int(op_limit), dtype=torch.int32, device=self.dev)
        check(self.lib.pqc_derivative_states(self.handle, _p(th) if self.n_params else None, _p(p0), idx,
                                             gens.ctypes.data, after.ctypes.data, len(gens), n_rows, _p(lim), _p(out),
                                             _p(ws), ws.numel(), _stream()))
        return out

    def gradient_states(self, theta, psi0=None, plain=False, checkpoints=None):
        """`PQC.get_gradients` rows (circuit.py:174-192).

        checkpoints: number of stored intermediate states the derivative runs start from (layer
        checkpointing; None picks min(8, rows // 16), 0 or 1 runs every derivative circuit from the start)."""
        if self._grad_cache is None:
            self._grad_cache = self.lowered.gradient_runs()
        gens, after, n_rows = self._grad_cache
        comp = self.lowered.composite_rows
        K = min(8, n_rows // 16) if checkpoints is None else int(checkpoints)
        if comp and plain:
            raise ValueError("the plain path has no form for non-commuting shared_parameter blocks")
        if plain or K <= 1 or len(gens) == 0:
            out = self.derivative_states(theta, psi0, gens, after, n_rows, plain=plain)
        else:
            out = self.derivative_states_from_checkpoints(theta, psi0, gens, after, n_rows, K)
        for row, gi in comp:
            out[row] = self.composite_derivative(gi, theta, psi0)
        return out

    def composite_derivative(self, gi, theta, psi0=None):
        """`take_derivative` row of gate gi, a shared_parameter(commute=False) block over non-commuting members
        (gates.py:459-466): D psi_g with D = sum_k prod(layer with d_k g_k) conj(U) and psi_g the state after
        the block.  conj(U) psi_g = conj(U conj(psi_g)) runs the block's own program on the conjugated state;
        sum_k prod(layer with d_k g_k) is the sum of the block program's derivative rows (generator d_k right
        after member k) from there; the gates after the block then run from that sum.  Device states
        throughout; the block and suffix programs are built once per gate."""
        lo = self.lowered
        g = lo.gates[gi]
        th = self._theta(theta)
        if th.shape[0] != 1:
            raise ValueError("derivative states take one parameter row")
        cache = self.__dict__.setdefault("_composite", {})
        if gi not in cache:
            layer_prog = Program(list(g.layer), self.N)
            rest = lo.gates[gi + 1:]
            suffix = Program(rest, self.N) if rest else None
            cols = [c for j in range(gi + 1, len(lo.gates)) for c in lo.gate_cols[j]]
            cache[gi] = (layer_prog, suffix, torch.as_tensor(cols, dtype=torch.int64, device=self.dev))
        layer_prog, suffix, cols = cache[gi]
        psi_g = self.run(th, psi0, row_limit=[int(lo.gate_last[gi]) + 1])[0]
        t_layer = th[:, lo.gate_cols[gi][0]:lo.gate_cols[gi][0] + 1].expand(1, layer_prog.n_params).contiguous()
        phi = layer_prog.run(t_layer, psi_g.conj().resolve_conj())[0].conj().resolve_conj()
        chi = layer_prog.gradient_states(t_layer, phi, checkpoints=0).sum(0)
        if suffix is None:
            return chi
        return suffix.run(th.index_select(1, cols) if cols.numel() else th[:, :0], chi)[0]

    def checkpoint_ops(self, after, K):
        """K op indices (the first 0) at quantiles of the runs' insertion points, each a valid op limit."""
        pos = np.sort(np.asarray(after, dtype=np.int64) + 1)
        cuts = [0]
        for q in range(1, K):
            b = int(pos[(q * len(pos)) // K])
            while b > 0 and not self.lib.pqc_program_limit_ok(self.handle, b):
                b -= 1
            if b > cuts[-1]:
                cuts.append(b)
        return np.array(cuts, dtype=np.int32)

    def derivative_states_from_checkpoints(self, theta, psi0, gens, after, n_rows, K):
        """`derivative_states` with every run started from the nearest stored state at or before its
        generator: the states after cuts[k] ops are computed once (pqc_run_limited), then
        pqc_derivative_states_from applies only the remaining ops of each run."""
        th = self._theta(theta)
        if th.shape[0] != 1:
            raise ValueError("derivative states take one parameter row")
        gens = np.ascontiguousarray(gens)
        after = np.ascontiguousarray(after, dtype=np.int32)
        cuts = self.checkpoint_ops(after, K)
        ck = self.run(th.expand(len(cuts), -1).contiguous(), psi0, row_limit=cuts)
        k_of = np.searchsorted(cuts, after.astype(np.int64) + 1, side="right") - 1
        run_psi0 = _to_dev(k_of, np.int32, self.dev)
        run_start = _to_dev(cuts[k_of], np.int32, self.dev)
        out = torch.empty((n_rows, self.D), dtype=torch.complex128, device=self.dev)
        ws = _ws(self.lib.pqc_derivative_states_workspace_size(self.handle, len(gens), n_rows), self.dev)
        check(self.lib.pqc_derivative_states_from(self.handle, _p(th) if self.n_params else None, _p(ck),
                                                  _p(run_psi0), _p(run_start), gens.ctypes.data, after.ctypes.data,
                                                  len(gens), n_rows, _p(out), _p(ws), ws.numel(), _stream()))
        return out

    def energy_grad(self, theta, H, psi0=None, want_grad=True, row_limit=None, plain=False):
        """(E [B], dE/dtheta [B, P]) by the adjoint sweep.

        row_limit: optional int32 [B]; row b then evaluates only the first row_limit[b] ops
        (a depth prefix of the circuit) and the gradient columns of the gates inside it.
        plain=True takes the one-kernel-per-op FP64 adjoint (no row limits)."""
        th = self._theta(theta)
        B = th.shape[0]
        p0, idx = self._psi0(psi0)
        terms = H.device_tensor(self.dev)
        n_terms = len(H.terms)
        if want_grad:
            if self._egrad_cache is None:
                self._egrad_cache = self.lowered.energy_gradient_runs()
            gens, after, n_cols = self._egrad_cache
        else:
            gens, after, n_cols = np.zeros(0, dtype=_lib.OP_DTYPE), np.zeros(0, dtype=np.int32), 0
        gens = np.ascontiguousarray(gens)
        after = np.ascontiguousarray(after, dtype=np.int32)
        lim = None
        if row_limit is not None:
            lim = self.limits(row_limit, B)
        E = torch.empty(B, dtype=torch.float64, device=self.dev)
        grad = torch.zeros((B, max(n_cols, 1)), dtype=torch.float64, device=self.dev)
        ws = _ws(self.lib.pqc_energy_grad_workspace_size(self.handle, B, len(gens), n_cols), self.dev)
        if plain:
            if lim is not None:
                raise ValueError("the plain adjoint takes no row limits")
            check(self.lib.pqc_energy_grad_plain(self.handle, _p(th) if self.n_params else None, self.n_params, B,
                                                 _p(p0), idx, _p(terms), n_terms,
                                                 gens.ctypes.data if len(gens) else None,
                                                 after.ctypes.data if len(after) else None, len(gens), n_cols, _p(E),
                                                 _p(grad), _p(ws), ws.numel(), _stream()))
            return E, grad[:, :n_cols]
        check(self.lib.pqc_energy_grad(self.handle, _p(th) if self.n_params else None, self.n_params, B, _p(p0), idx,
                                       _p(terms), n_terms, gens.ctypes.data if len(gens) else None,
                                       after.ctypes.data if len(after) else None, len(gens), n_cols, _p(E), _p(grad),
                                       _p(lim) if lim is not None else None, _p(ws), ws.numel(), _stream()))
        return E, grad[:, :n_cols]


def run_multi(jobs, out=None):
    """States of several programs' parameter rows with shared launches (`pqc_run_multi`).

    jobs: list of (program, theta [B, P], psi0 or None, row_limit or None); returns one complex128 [B, 2^N]
    tensor per job (or writes into `out`, a matching list).  Every row equals `program.run(theta, psi0,
    row_limit=...)` bit for bit; the jobs share one coefficient launch, one conversion launch and one sweep
    launch per sweep index, so a mix of circuits of up to 13 qubits costs three launches."""
    if not jobs:
        return []
    lib = _lib.load()
    items = np.zeros(len(jobs), dtype=_lib.RUN_ITEM_DTYPE)
    keep, outs = [], []
    for i, (prog, theta, psi0, row_limit) in enumerate(jobs):
        th = prog._theta(theta)
        B = th.shape[0]
        p0, idx = prog._psi0(psi0)
        o = out[i] if out is not None else torch.empty((B, prog.D), dtype=torch.complex128, device=prog.dev)
        lim = prog.limits(row_limit, B) if row_limit is not None else None
        keep += [th, p0, lim, o]
        outs.append(o)
        items[i] = (prog.handle.value, th.data_ptr() if prog.n_params else 0, prog.n_params, B,
                    p0.data_ptr() if p0 is not None else 0, idx, lim.data_ptr() if lim is not None else 0,
                    o.data_ptr())
    ws = _ws(lib.pqc_run_multi_workspace_size(items.ctypes.data, len(items)), jobs[0][0].dev)
    check(lib.pqc_run_multi(items.ctypes.data, len(items), _p(ws), ws.numel(), _stream()))
    return outs


# ---------------------------------------------------------------------- CUDA graphs
class GraphedRun:
    """`Program.run` for a fixed batch size captured once in a CUDA graph and replayed.

    The coefficient kernels and every sweep launch of the plan replay with one call, which removes the host
    launch overhead that dominates small batches.  `theta` rows are copied into the captured input buffer; the
    returned tensor is the captured output buffer and is overwritten by the next call."""

    def __init__(self, program, batch, psi0=None, mode="c128"):
        self.program = program
        dt = torch.complex64 if mode == "c64" else torch.complex128
        self.theta = torch.zeros((int(batch), program.n_params), dtype=torch.float64, device=program.dev)
        self.out = torch.empty((int(batch), program.D), dtype=dt, device=program.dev)
        side = torch.cuda.Stream()
        side.wait_stream(torch.cuda.current_stream())
        with torch.cuda.stream(side):  # first call outside the capture (one-time device setup)
            program.run(self.theta, psi0, mode=mode, out=self.out)
        torch.cuda.current_stream().wait_stream(side)
        torch.cuda.synchronize()
        self.graph = torch.cuda.CUDAGraph()
        with torch.cuda.graph(self.graph):
            program.run(self.theta, psi0, mode=mode, out=self.out)

    def __call__(self, theta):
        th = _f64(theta, self.program.dev)
        if th.dim() == 1:
            th = th.reshape(1, -1)
        if tuple(th.shape) != tuple(self.theta.shape):
            raise ValueError(f"captured for theta of shape {tuple(self.theta.shape)}, got {tuple(th.shape)}")
        self.theta.copy_(th, non_blocking=True)
        self.graph.replay()
        return self.out


class GraphedMulti:
    """`run_multi` over fixed jobs -- programs of any qubit counts, depths and gate lists, each with a fixed
    batch size -- captured once in a CUDA graph and replayed.

    jobs: list of (program, batch, psi0 or None, row_limit or None).  One replay runs the shared coefficient and
    conversion launches and one sweep launch per sweep index for all jobs.  Call with one theta [batch, P] per
    job; the rows are copied into the captured input buffers and the returned list holds the captured output
    buffers (overwritten by the next call).  Every row equals `program.run(theta, psi0, row_limit=...)` bit
    for bit."""

    def __init__(self, jobs):
        if not jobs:
            raise ValueError("no jobs")
        self.programs = [j[0] for j in jobs]
        self.thetas, self.outs, run_jobs = [], [], []
        for prog, batch, psi0, row_limit in jobs:
            th = torch.zeros((int(batch), prog.n_params), dtype=torch.float64, device=prog.dev)
            o = torch.empty((int(batch), prog.D), dtype=torch.complex128, device=prog.dev)
            p0 = psi0 if psi0 is None or isinstance(psi0, (int, np.integer)) else _c128(psi0, prog.dev)
            lim = prog.limits(row_limit, int(batch)) if row_limit is not None else None  # host checks, before capture
            self.thetas.append(th)
            self.outs.append(o)
            run_jobs.append((prog, th, p0, lim))
        self._jobs = run_jobs
        side = torch.cuda.Stream()
        side.wait_stream(torch.cuda.current_stream())
        with torch.cuda.stream(side):  # first call outside the capture (one-time device setup)
            run_multi(run_jobs, out=self.outs)
        torch.cuda.current_stream().wait_stream(side)
        torch.cuda.synchronize()
        self.graph = torch.cuda.CUDAGraph()
        with torch.cuda.graph(self.graph):
            run_multi(run_jobs, out=self.outs)

    def __call__(self, thetas):
        if len(thetas) != len(self.thetas):
            raise ValueError(f"expected {len(self.thetas)} theta arrays, got {len(thetas)}")
        for dst, th in zip(self.thetas, thetas):
            t = _f64(th, dst.device)
            if t.dim() == 1:
                t = t.reshape(1, -1)
            if tuple(t.shape) != tuple(dst.shape):
                raise ValueError(f"captured for theta of shape {tuple(dst.shape)}, got {tuple(t.shape)}")
            dst.copy_(t, non_blocking=True)
        self.graph.replay()
        return self.outs


# ---------------------------------------------------------------------- autotuner
_TUNED = {}
# (tile qubits, CTAs per SM, threads per CTA)
TUNE_CANDIDATES = ((12, 2, 256), (12, 3, 256), (12, 3, 128), (13, 1, 512), (11, 3, 256), (11, 3, 128))


def autotune(gates, n_qubits, batch, candidates=TUNE_CANDIDATES, reps=2):
    """((tile_qubits, ctas_per_sm, threads), {candidate: ms}) of the fastest sweep configuration for this circuit
    at this batch size, timed with CUDA events on seeded angles.  Circuits of at most 13 qubits run as one sweep
    of the whole state and are not tuned.  Results are cached per (op table, batch)."""
    N = int(n_qubits)
    if N <= 13:
        return (0, 0, 0), {}
    low = Lowered(gates, N)
    key = (N, int(batch), hash(np.ascontiguousarray(low.ops).tobytes()))
    if key in _TUNED:
        return _TUNED[key]
    dev = device()
    th = torch.from_numpy(np.random.default_rng(0).random((batch, low.n_params)) * 2 * np.pi).to(dev)
    out = torch.empty((batch, 1 << N), dtype=torch.complex128, device=dev)
    timings = {}
    progs = {}
    for k, occ, thr in candidates:
        if k > N:
            continue
        prog = progs.get(k)
        if prog is None:
            prog = progs[k] = Program(gates, N, k)
        prog.set_launch(occ if occ in (2, 3) else 0, thr if occ == 3 else 0)
        prog.run(th, 0, out=out)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(reps):
            prog.run(th, 0, out=out)
        e1.record()
        torch.cuda.synchronize()
        timings[(k, occ, thr)] = e0.elapsed_time(e1) / reps
    best = min(timings, key=timings.get)
    _TUNED[key] = (best, timings)
    return _TUNED[key]


# ---------------------------------------------------------------------- measures
def _nq(psi):
    D = psi.shape[-1]
    N = int(round(math.log2(D)))
    if 1 << N != D:
        raise ValueError("state length must be a power of two")
    return N


def _states(psi):
    dev = device()
    t = _c128(psi, dev)
    if t.dim() == 1:
        t = t.reshape(1, -1)
    return t.reshape(t.shape[0], -1), dev


def overlaps(a, b, ia, ib):
    """<a[ia[k]] | b[ib[k]]> (complex128 [n])."""
    lib = _lib.load()
    A, dev = _states(a)
    Bt, _ = _states(b)
    N = _nq(A)
    ia = torch.as_tensor(ia, dtype=torch.int64).to(dev).contiguous()
    ib = torch.as_tensor(ib, dtype=torch.int64).to(dev).contiguous()
    n = ia.numel()
    out = torch.empty(n, dtype=torch.complex128, device=dev)
    ws = _ws(lib.pqc_overlaps_workspace_size(n, N), dev)
    check(lib.pqc_overlaps(_p(A), _p(Bt), _p(ia), _p(ib), n, N, _p(out), _p(ws), ws.numel(), _stream()))
    return out


def fidelity_pairs(a, b):
    """|<a_k|b_k>|^2 row by row."""
    A, dev = _states(a)
    n = A.shape[0]
    idx = torch.arange(n, dtype=torch.int64, device=dev)
    ov = overlaps(A, b, idx, idx)
    return ov.real ** 2 + ov.imag ** 2


_EDGES = {}


def hist_edges(nbins, dev=None):
    """np.histogram's edges for range (0, 1): np.linspace(0, 1, nbins + 1), uploaded once per (nbins, device)
    (a pageable upload would wait for the stream's queued work).  The returned tensor is shared: read only."""
    dev = dev or device()
    key = (int(nbins), str(dev))
    t = _EDGES.get(key)
    if t is None:
        t = _to_dev(np.linspace(0.0, 1.0, int(nbins) + 1), np.float64, dev)
        _EDGES[key] = t
    return t


def allpairs_fidelity_hist(psi, nbins, keep_samples=True):
    """(F [S(S-1)/2] in combinations order or None, counts int64 [nbins], edges)."""
    lib = _lib.load()
    X, dev = _states(psi)
    S = X.shape[0]
    N = _nq(X)
    M = S * (S - 1) // 2
    edges = hist_edges(nbins, dev)
    counts = torch.zeros(max(int(nbins), 1), dtype=torch.int64, device=dev)
    F = torch.empty(M, dtype=torch.float64, device=dev) if keep_samples else None
    ws = _ws(lib.pqc_fidelity_hist_workspace_size(S, N), dev)
    check(lib.pqc_fidelity_hist(_p(X), S, N, int(nbins), _p(edges), _p(F), _p(counts) if nbins >= 1 else None,
                                _p(ws), ws.numel(), _stream()))
    return F, counts, edges


def gram_tf32(psi):
    """(G complex128 [S, S] = <psi_a|psi_b> from the tensor cores, delta_factor): each component of G is within
    delta_factor ||a|| ||b|| of the exact value.  S <= 256 states of at least 13 qubits on a GB300."""
    lib = _lib.load()
    X, dev = _states(psi)
    S = X.shape[0]
    N = _nq(X)
    G = torch.empty((S, S), dtype=torch.complex128, device=dev)
    dfac = C.c_double(0.0)
    ws = _ws(lib.pqc_gram_tf32_workspace_size(S, N), dev)
    check(lib.pqc_gram_tf32(_p(X), S, N, _p(G), C.byref(dfac), _p(ws), ws.numel(), _stream()))
    return G, dfac.value


def histogram(F, nbins):
    lib = _lib.load()
    dev = device()
    Ft = _f64(F, dev).reshape(-1)
    edges = hist_edges(nbins, dev)
    counts = torch.zeros(int(nbins), dtype=torch.int64, device=dev)
    check(lib.pqc_histogram(_p(Ft), Ft.numel(), int(nbins), _p(edges), _p(counts), _stream()))
    return counts, edges


def expr_kl(counts, edges, d):
    lib = _lib.load()
    dev = counts.device
    out = torch.empty(1, dtype=torch.float64, device=dev)
    check(lib.pqc_expr_kl(_p(counts), counts.numel(), _p(edges), float(d), _p(out), _stream()))
    return out


def mw(psi):
    """Meyer-Wallach Q per state (float64 [B])."""
    lib = _lib.load()
    X, dev = _states(psi)
    B = X.shape[0]
    N = _nq(X)
    Q = torch.empty(B, dtype=torch.float64, device=dev)
    ws = _ws(lib.pqc_mw_workspace_size(B, N), dev)
    check(lib.pqc_mw(_p(X), B, N, _p(Q), _p(ws), ws.numel(), _stream()))
    return Q


def expect(psi, H):
    """<psi_b|H|psi_b> (float64 [B]) for a PauliSum H."""
    lib = _lib.load()
    X, dev = _states(psi)
    B = X.shape[0]
    N = _nq(X)
    if H.n_qubits != N:
        raise ValueError("Hamiltonian and state sizes differ")
    terms = H.device_tensor(dev)
    E = torch.empty(B, dtype=torch.float64, device=dev)
    ws = _ws(lib.pqc_expect_workspace_size(B, N, len(H.terms)), dev)
    check(lib.pqc_expect(_p(X), B, N, _p(terms), len(H.terms), _p(E), _p(ws), ws.numel(), _stream()))
    return E


def magic(psi, alpha=2.0):
    """Renyi-alpha stabiliser entropy per state (float64 [B])."""
    lib = _lib.load()
    X, dev = _states(psi)
    B = X.shape[0]
    N = _nq(X)
    M = torch.empty(B, dtype=torch.float64, device=dev)
    ws = _ws(lib.pqc_magic_workspace_size(B, N), dev)
    check(lib.pqc_magic(_p(X), B, N, float(alpha), _p(M), _p(ws), ws.numel(), _stream()))
    return M


def qfim(state, dpsi, fp64=False):
    """QFIM [P, P] (float64, device) from a reference state and derivative states (fp64: the Gram in native
    FP64 instead of double-float)."""
    lib = _lib.load()
    s, dev = _states(state)
    Dp, _ = _states(dpsi)
    P = Dp.shape[0]
    N = _nq(Dp)
    F = torch.empty((P, P), dtype=torch.float64, device=dev)
    if P == 0:
        return F
    ws = _ws(lib.pqc_qfim_workspace_size(P, N), dev)
    fn = lib.pqc_qfim_fp64 if fp64 else lib.pqc_qfim
    check(fn(_p(s), _p(Dp), P, N, _p(F), _p(ws), ws.numel(), _stream()))
    return F


def gram_cross(a, b):
    """G[i, j] = <a_i|b_j> (complex128 [na, nb], device)."""
    lib = _lib.load()
    A, dev = _states(a)
    Bm, _ = _states(b)
    N = _nq(A)
    if _nq(Bm) != N:
        raise ValueError("state sizes differ")
    na, nb = A.shape[0], Bm.shape[0]
    G = torch.empty((na, nb), dtype=torch.complex128, device=dev)
    if na == 0 or nb == 0:
        return G
    ws = _ws(lib.pqc_gram_cross_workspace_size(na, nb, N), dev)
    check(lib.pqc_gram_cross(_p(A), na, _p(Bm), nb, N, _p(G), _p(ws), ws.numel(), _stream()))
    return G


def qfim_blocked(program, theta, state, block_rows, psi0=None):
    """The QFIM of `PQC.get_gradients`' rows with at most 2 x block_rows derivative states on the device at once.

    F_pq = 4 Re(<d_p|d_q> - <d_p|state><state|d_q>), upper triangle mirrored (measure.py:33-71), assembled from
    Gram blocks: the states of row block I are kept while those of every later block J are recomputed, so the
    derivative runs cost (n_blocks + 1) / 2 times those of the unblocked path, in exchange for memory."""
    if program._grad_cache is None:
        program._grad_cache = program.lowered.gradient_runs()
    gens, after, P = program._grad_cache
    if program.lowered.composite_rows:
        raise ValueError("the blocked QFIM has no form for non-commuting shared_parameter blocks")
    s = _c128(state, program.dev).reshape(1, -1)
    F = torch.empty((P, P), dtype=torch.float64, device=program.dev)
    block_rows = max(1, int(block_rows))
    blocks = [(i0, min(P, i0 + block_rows)) for i0 in range(0, P, block_rows)]
    sel = gens["sel"]

    def states(i0, i1):
        m = (sel >= i0) & (sel < i1)
        g = gens[m].copy()
        g["sel"] -= i0
        d = program.derivative_states(theta, psi0, g, after[m], i1 - i0)
        v = gram_cross(s, d)[0]  # <state|d_p>
        return d, v

    for bi, (i0, i1) in enumerate(blocks):
        DI, vI = states(i0, i1)
        for j0, j1 in blocks[bi:]:
            DJ, vJ = (DI, vI) if j0 == i0 else states(j0, j1)
            blk = 4.0 * (gram_cross(DI, DJ) - vI.conj()[:, None] * vJ[None, :]).real
            if j0 == i0:
                blk = torch.triu(blk) + torch.triu(blk, 1).T
                F[i0:i1, i0:i1] = blk
            else:
                F[i0:i1, j0:j1] = blk
                F[j0:j1, i0:i1] = blk.T
            del DJ
    return F


def derivative_plan_order(ops, gens, after, n_qubits, tile_qubits=0):
    """Host-only: (order in which the derivative plan applies the forward ops and generators, n_sweeps); entries
    >= 0 are op indices, -(r + 1) is generator r."""
    lib = _lib.load()
    ops = np.ascontiguousarray(ops)
    gens = np.ascontiguousarray(gens)
    after = np.ascontiguousarray(after, dtype=np.int32)
    n, g = len(ops), len(gens)
    order = np.zeros(max(n + g, 1), dtype=np.int32)
    ns = C.c_int32()
    check(lib.pqc_derivative_plan_order(ops.ctypes.data if n else None, n, gens.ctypes.data if g else None,
                                        after.ctypes.data if g else None, g, int(n_qubits), int(tile_qubits),
                                        order.ctypes.data, C.byref(ns)))
    return order[:n + g], ns.value


def plan_order(ops, n_qubits, tile_qubits=0):
    """Host-only: (order of op indices as the sweep plan applies them, sweep index of each, n_sweeps)."""
    lib = _lib.load()
    ops = np.ascontiguousarray(ops)
    n = len(ops)
    order = np.zeros(max(n, 1), dtype=np.int32)
    sweep = np.zeros(max(n, 1), dtype=np.int32)
    ns = C.c_int32()
    check(lib.pqc_plan_order(ops.ctypes.data if n else None, n, int(n_qubits), int(tile_qubits), order.ctypes.data,
                             sweep.ctypes.data, C.byref(ns)))
    return order[:n], sweep[:n], ns.value
