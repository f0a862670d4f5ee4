"""The FP64 oracle spread over the host cores, for parity checks at benchmark sizes.

Test infrastructure: the oracle (`oracle/pqc_oracle.py`) evaluates one circuit
row or one derivative run per call; an N = 20, 20-layer circuit takes about
10 s on one core and the 256 derivative runs of an N = 16, P = 256 circuit
about a minute, so these helpers hand independent rows / runs to a pool of
single-threaded worker processes.  The pool is started with `spawn` (a forked
child of a process that has used CUDA hangs).  Circuits travel to the workers
as (template name, N, L) and are rebuilt there from `pyramaterised_gb300.templates`.
"""
import multiprocessing as mp
import os

import numpy as np

_BLAS_VARS = ("OMP_NUM_THREADS", "OPENBLAS_NUM_THREADS", "MKL_NUM_THREADS")


def _circuit(spec):
    import pyramaterised_gb300 as pq

    name, N, L = spec
    return getattr(pq.templates, name)(N, L)


def _run_rows(args):
    spec, thetas = args
    from oracle import pqc_oracle as O

    c = _circuit(spec)
    return [O.run(c.gates, spec[1], t) for t in thetas]


def _deriv_runs(args):
    spec, theta, tasks = args
    from oracle import pqc_oracle as O

    c = _circuit(spec)
    return [O.take_derivative(c.gates, spec[1], theta, gi, which) for gi, which in tasks]


def _magic(args):
    psi, alpha = args
    from oracle import measures_oracle as MO

    return MO.renyi_entropy_wht(psi, alpha)


def _warm(_):
    import pyramaterised_gb300  # noqa: F401
    from oracle import measures_oracle, pqc_oracle  # noqa: F401

    return 0


class OraclePool:
    """A spawned pool of single-threaded oracle workers (one per host core by default)."""

    def __init__(self, workers=None):
        self.workers = int(workers or os.cpu_count() or 1)
        saved = {v: os.environ.get(v) for v in _BLAS_VARS}
        for v in _BLAS_VARS:
            os.environ[v] = "1"
        try:
            self.pool = mp.get_context("spawn").Pool(self.workers)
        finally:
            for v, val in saved.items():
                if val is None:
                    os.environ.pop(v, None)
                else:
                    os.environ[v] = val
        self.pool.map(_warm, range(self.workers))

    def close(self):
        self.pool.terminate()
        self.pool.join()

    def states(self, spec, thetas):
        """O.run of every row of `thetas` [B, P] for the circuit `spec` = (template, N, L): [B, 2^N]."""
        thetas = np.asarray(thetas, dtype=np.float64)
        parts = self.pool.map(_run_rows, [(spec, thetas[i:i + 1]) for i in range(len(thetas))])
        return np.stack([s for p in parts for s in p])

    def gradient_states(self, spec, theta):
        """O.get_gradients rows (`circuit.py:174-192`) of one parameter row: [R, 2^N]."""
        from oracle import pqc_oracle as O

        tasks = O.gradient_tasks(_circuit(spec).gates)
        n = self.workers
        chunks = [tasks[i::n] for i in range(n)]
        parts = self.pool.map(_deriv_runs, [(spec, np.asarray(theta, dtype=np.float64), ch) for ch in chunks])
        out = [None] * len(tasks)
        for i, part in enumerate(parts):
            for j, s in enumerate(part):
                out[i + j * n] = s
        return np.stack(out)

    def magic(self, states, alpha=2.0):
        """MO.renyi_entropy_wht of each state."""
        return np.array(self.pool.map(_magic, [(np.asarray(s), alpha) for s in states]))
