"""Grid double-float arithmetic of the forward sweeps (pqc_program_set_grid), through the C ABI.

With the switch on, a program's double-float sweeps keep every amplitude's high word on a grid set by the
tile's norm bound.  Checked here: states against the FP64 oracle to 1e-10 (HE ladder with RY rotations and
TFIM-style with RX rotations, one-sweep and multi-sweep sizes, the 20-qubit benchmark circuits), per-row op
limits (the plan without relabelling), launch shapes bit-identical to each other, the multi-program launch
bit-identical to single-program runs, and the switch's refusal for a program with a non-unitary op.
"""
import numpy as np
import pytest
import torch

import recipes
from oracle import pqc_oracle as O
import pyramaterised_gb300 as pq
from pyramaterised_gb300 import _lib, engine

pytestmark = pytest.mark.gpu
AMP_TOL = 1e-10


def _np(t):
    return t.detach().cpu().numpy()


def _theta(c, rows, seed):
    return np.random.default_rng(seed).random((rows, c.n_columns())) * 2 * np.pi


@pytest.mark.parametrize("kind,N,L", [("he", 8, 8), ("tfim", 10, 6), ("he", 13, 13), ("he", 16, 6),
                                      ("tfim", 17, 4), ("npqc", 12, 6)])
def test_grid_states_match_oracle(cuda, kind, N, L):
    make = {"he": pq.templates.hardware_efficient_ladder, "tfim": pq.templates.tfim_style,
            "npqc": pq.templates.npqc_style}[kind]
    c = make(N, L)
    c.program.set_grid(True)
    th = _theta(c, 3, 11 + N)
    psi = _np(c.run_batch(th))
    ref = O.run_batch(c.gates, N, th)
    err = float(np.abs(psi - ref).max())
    print(f"grid {kind} N={N} L={L}: max |psi - oracle| = {err:.3e}")
    assert err < AMP_TOL
    assert c.program.status() == 0
    c.program.set_grid(False)
    plain = _np(c.run_batch(th))
    assert float(np.abs(plain - ref).max()) < AMP_TOL


def test_grid_n20_benchmark_states(cuda, oracle_pool):
    for name, make in (("hardware_efficient_ladder", pq.templates.hardware_efficient_ladder),
                       ("tfim_style", pq.templates.tfim_style)):
        c = make(20, 20)
        c.program.set_grid(True)
        th = _theta(c, 2, 5)
        psi = _np(c.run_batch(th))
        ref = oracle_pool.states((name, 20, 20), th)
        err = float(np.abs(psi - ref).max())
        print(f"grid {name} N=20 L=20: max |psi - oracle| = {err:.3e}")
        assert err < AMP_TOL
        assert c.program.status() == 0


def test_grid_special_angles_and_row_limits(cuda):
    # angles where cos or sin of the half angle vanishes or is tiny (form A/B switch, identity and pi rotations),
    # and per-row op limits (the plan without relabelling, inactive members of rotation pairs)
    N, L = 10, 4
    c = recipes.he_ladder(pq, N, L)
    c.program.set_grid(True)
    P = c.n_columns()
    rng = np.random.default_rng(7)
    special = np.array([0.0, np.pi, -np.pi, 3 * np.pi, np.pi / 2, np.pi - 1e-9, np.pi + 1e-6, 2 * np.pi, 1e-12])
    th = np.stack([rng.choice(special, P), rng.random(P) * 2 * np.pi,
                   np.where(rng.random(P) < 0.5, np.pi, rng.random(P) * 2 * np.pi), np.full(P, np.pi),
                   np.pi - 10.0 ** -rng.integers(1, 12, P)])
    np.testing.assert_allclose(_np(c.run_batch(th)), O.run_batch(c.gates, N, th), atol=AMP_TOL)
    G = len(c.gates)
    cuts = [G // 3, G, 1, G // 2 + 1, 0]
    got = _np(c.program.run(th, row_limit=cuts))
    for r, g in enumerate(cuts):
        gates = c.gates[:g]
        n = sum(int(x.param_count) if x.is_param else 0 for x in gates)
        np.testing.assert_allclose(got[r], O.run(gates, N, th[r, :n]), atol=AMP_TOL)
    assert c.program.status() == 0


@pytest.mark.parametrize("k", [4, 6, 8])
def test_grid_every_gate_small_tiles(cuda, k):
    # every gate class (fixed matrices, fSim, RXX/RYY/RZZ, CZ) with most qubits outside the tile: the grid
    # passes interleave with general ops, which leave the tile off the grid
    N = 9
    c = recipes.every_gate(pq, N)
    c.add_layer([pq.R_y(i, N) for i in range(N)] + [pq.CNOT([i, (i + 3) % N], N) for i in range(N)]
                + [pq.R_zz([0, 8], N), pq.CZ([8, 1], N), pq.R_xx([2, 7], N), pq.fSim([3, 6], N)])
    c.set_tile_qubits(k)
    c.program.set_grid(True)
    th = np.random.default_rng(k).random((2, c.n_columns())) * 2 * np.pi
    st = (np.random.default_rng(0).standard_normal(2 ** N) + 1j * np.random.default_rng(1).standard_normal(2 ** N))
    st /= np.linalg.norm(st)
    c.initial_state = st
    np.testing.assert_allclose(_np(c.run_batch(th)), O.run_batch(c.gates, N, th, st), atol=AMP_TOL)


def test_grid_launch_shapes_bit_identical(cuda):
    c = pq.templates.hardware_efficient_ladder(16, 8)
    c.program.set_grid(True)
    th = torch.from_numpy(_theta(c, 6, 21)).to(cuda)
    outs = []
    for tile, ctas, threads in ((12, 3, 128), (12, 3, 256), (12, 2, 256), (13, 0, 0)):
        p = engine.Program(c.gates, 16, tile_qubits=tile)
        p.set_grid(True)
        if ctas:  # 2^13-amplitude tiles always run 512 threads, one CTA per SM
            p.set_launch(ctas, threads)
        outs.append((tile, p.run(th, 0)))
    for tile, o in outs[1:]:
        if tile == outs[0][0]:
            assert torch.equal(o, outs[0][1])
    ref = O.run_batch(c.gates, 16, _np(th)[:2])
    for _, o in outs:
        assert float(np.abs(_np(o[:2]) - ref).max()) < AMP_TOL


def test_grid_multi_program_bit_identical(cuda):
    rng = np.random.default_rng(8)
    circuits = [pq.templates.hardware_efficient_ladder(6, 3), pq.templates.tfim_style(9, 4),
                pq.templates.npqc_style(12, 5), pq.templates.hardware_efficient_ladder(15, 3)]
    jobs, ref = [], []
    for c in circuits:
        c.program.set_grid(True)
        th = torch.from_numpy(rng.random((3, c.n_columns())) * 2 * np.pi).to(cuda)
        jobs.append((c.program, th, None, None))
        ref.append(c.program.run(th, None))
    out = engine.run_multi(jobs)
    torch.cuda.synchronize()
    for o, r in zip(out, ref):
        assert torch.equal(o, r)


def test_grid_refused_for_non_unitary_program(cuda):
    import ctypes as C

    from pyramaterised_gb300.lowering import _op

    lib = _lib.load()
    ops = np.array([_op(_lib.PQC_OP_PAULI, 0, pauli=1, m=[1.0])], dtype=_lib.OP_DTYPE)
    h = C.c_void_p()
    assert lib.pqc_program_create(ops.ctypes.data, 1, 2, 0, 0, C.byref(h)) == 0
    try:
        assert lib.pqc_program_set_grid(h, 1) != 0
        assert b"unitary" in lib.pqc_last_error()
        assert lib.pqc_program_set_grid(h, 0) == 0
    finally:
        lib.pqc_program_destroy(h)
