"""pqc_run_multi: several programs -- different qubit counts, depths, gate lists, start states and per-row op
limits -- evaluated with shared launches, called through the C ABI.  Every row must equal the single-program
pqc_run / pqc_run_limited result bit for bit (the same per-tile arithmetic runs), and the oracle to 1e-10."""
import numpy as np
import pytest
import torch

import recipes
from oracle import pqc_oracle as O
import pyramaterised_gb300 as pq
from pyramaterised_gb300 import _lib, engine

pytestmark = pytest.mark.gpu


def _np(t):
    return t.detach().cpu().numpy()


def test_run_multi_matches_single_program_runs(cuda):
    rng = np.random.default_rng(3)
    circuits = [pq.templates.hardware_efficient_ladder(6, 3), pq.templates.tfim_style(9, 4),
                recipes.every_gate(pq, 7), pq.templates.npqc_style(12, 5),
                pq.templates.hardware_efficient_ladder(15, 3),  # two or more sweeps
                pq.templates.tfim_style(5, 2)]
    jobs, ref = [], []
    for i, c in enumerate(circuits):
        B = [3, 1, 2, 4, 2, 0][i]
        th = torch.from_numpy(rng.random((B, c.n_columns())) * 2 * np.pi).to(cuda)
        psi0 = None
        if i == 2:  # a start state
            v = rng.standard_normal(2 ** 7) + 1j * rng.standard_normal(2 ** 7)
            psi0 = torch.from_numpy(v / np.linalg.norm(v)).to(cuda)
        jobs.append((c.program, th, psi0, None))
        ref.append(c.program.run(th, psi0) if B else None)
    out = engine.run_multi(jobs)
    torch.cuda.synchronize()
    for i, (o, r) in enumerate(zip(out, ref)):
        if r is None:
            assert o.shape[0] == 0
            continue
        np.testing.assert_array_equal(_np(o), _np(r), err_msg=f"item {i}")
    c = circuits[0]
    np.testing.assert_allclose(_np(out[0]), O.run_batch(c.gates, 6, _np(jobs[0][1])), atol=1e-10)
    assert all(cc.program.status() == 0 for cc in circuits)


def test_run_multi_with_row_limits_matches_run_limited(cuda):
    # the serving pattern: each family's deepest program, every row cut to its own depth at a layer boundary
    rng = np.random.default_rng(4)
    fams = [(pq.templates.hardware_efficient_ladder(8, 16), 16), (pq.templates.tfim_style(11, 22), 22),
            (pq.templates.hardware_efficient_ladder(14, 6), 6)]
    jobs, ref = [], []
    for c, L in fams:
        gpl = len(c.gates) // L
        last = c.program.lowered.gate_last
        cut = [0] + [int(last[d * gpl - 1] + 1) for d in (1, L // 2, L)]
        th = torch.from_numpy(rng.random((len(cut), c.n_columns())) * 2 * np.pi).to(cuda)
        jobs.append((c.program, th, None, cut))
        ref.append(c.program.run(th, row_limit=cut))
    out = engine.run_multi(jobs)
    for o, r in zip(out, ref):
        np.testing.assert_array_equal(_np(o), _np(r))


def test_run_multi_rejects_bad_items(cuda):
    lib = _lib.load()
    c = pq.templates.hardware_efficient_ladder(5, 1)
    items = np.zeros(1, dtype=_lib.RUN_ITEM_DTYPE)
    items[0] = (c.program.handle.value, 0, c.n_columns(), 2, 0, 1 << 5, 0, 0)  # psi NULL, index out of range
    rc = lib.pqc_run_multi(items.ctypes.data, 1, None, 0, None)
    assert rc == -1  # PQC_ERR_INVALID
    assert "item 0" in _lib.last_error()


def test_graphed_multi_replays_match_run_multi(cuda):
    # one CUDA graph over circuits of different qubit counts (one- and multi-sweep plans), a start state and
    # per-row depth limits, replayed with new angles: bit-identical to direct runs
    rng = np.random.default_rng(11)
    c1, c2, c3 = (pq.templates.hardware_efficient_ladder(7, 3), pq.templates.tfim_style(10, 4),
                  pq.templates.hardware_efficient_ladder(15, 3))
    v = rng.standard_normal(2 ** 10) + 1j * rng.standard_normal(2 ** 10)
    psi0 = torch.from_numpy(v / np.linalg.norm(v)).to(cuda)
    gpl = len(c1.gates) // 3
    cut = [int(c1.program.lowered.gate_last[d * gpl - 1] + 1) for d in (1, 2, 3, 3)]
    g = engine.GraphedMulti([(c1.program, 4, None, cut), (c2.program, 3, psi0, None), (c3.program, 2, None, None)])
    for rep in range(2):
        ths = [torch.from_numpy(rng.random((b, c.n_columns())) * 2 * np.pi).to(cuda)
               for c, b in ((c1, 4), (c2, 3), (c3, 2))]
        outs = g(ths)
        torch.cuda.synchronize()
        np.testing.assert_array_equal(_np(outs[0]), _np(c1.program.run(ths[0], row_limit=cut)))
        np.testing.assert_array_equal(_np(outs[1]), _np(c2.program.run(ths[1], psi0)))
        np.testing.assert_array_equal(_np(outs[2]), _np(c3.program.run(ths[2])))
    np.testing.assert_allclose(_np(outs[2]), O.run_batch(c3.gates, 15, _np(ths[2])), atol=1e-10)
