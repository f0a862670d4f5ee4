"""GPU parity: the CUDA path through the C ABI against the reference's golden
vectors and the FP64 oracle.

Tolerances (from the project's accuracy bar): 1e-10 absolute on amplitudes,
fidelities and energies; 1e-8 relative on QFIM entries; histogram counts
identical except for samples within 1e-12 of a bin edge.
"""
import numpy as np
import pytest
import torch

import recipes
from oracle import measures_oracle as MO
from oracle import pqc_oracle as O
import pyramaterised_gb300 as pq
from pyramaterised_gb300 import _lib, engine, gates
from test_oracle import _build

pytestmark = pytest.mark.gpu
AMP_TOL = 1e-10
QFIM_RTOL = 1e-8


def _np(t):
    return t.detach().cpu().numpy()


def _cases(golden):
    return sorted({k.rsplit("/", 1)[0] for k in golden.files if k.endswith("/state")})


def _with_init(c, golden, key):
    c.initial_state = golden[f"{key}/init"]
    return c


def test_forward_matches_reference_golden(cuda, golden):
    for key in _cases(golden):
        c = _with_init(_build(key), golden, key)
        th = golden[f"{key}/theta"]
        for mode in ("c128", "plain"):
            psi = _np(c.run_batch(th[None, :], mode=mode)[0])
            np.testing.assert_allclose(psi, golden[f"{key}/state"], atol=AMP_TOL, err_msg=f"{key} {mode}")
        psi = _np(c.run(list(th)))
        np.testing.assert_allclose(psi, golden[f"{key}/state"], atol=AMP_TOL, err_msg=key)


def test_energies_match_reference_golden(cuda, golden):
    for key in _cases(golden):
        c = _with_init(_build(key), golden, key)
        th = list(golden[f"{key}/theta"])
        N = c.n_qubits
        if N >= 2:
            assert abs(c.cost(th) - float(golden[f"{key}/energy_ZZ"])) < AMP_TOL, key
        if f"{key}/energy_H" in golden.files:
            c.set_H(pq.templates.TFIM_hamiltonian(N, 1.0, 0.5 if key.startswith("tpl") else 0.0))
            assert abs(c.cost(th) - float(golden[f"{key}/energy_H"])) < AMP_TOL, key


def test_gradient_states_and_qfim_match_reference_golden(cuda, golden):
    for key in _cases(golden):
        if f"{key}/grads" not in golden.files:
            continue
        c = _with_init(_build(key), golden, key)
        th = list(golden[f"{key}/theta"])
        c.state = c.run(th)
        grads = _np(c.get_gradients())
        np.testing.assert_allclose(grads, golden[f"{key}/grads"], atol=AMP_TOL, err_msg=key)
        F = pq.measure.Measurements(c).get_QFI()
        ref = golden[f"{key}/qfim"]
        np.testing.assert_allclose(F, ref, rtol=QFIM_RTOL, atol=QFIM_RTOL * max(1.0, np.abs(ref).max()), err_msg=key)
        F64 = _np(engine.qfim(c.state, c.get_gradients(), fp64=True))
        np.testing.assert_allclose(F64, ref, rtol=QFIM_RTOL, atol=QFIM_RTOL * max(1.0, np.abs(ref).max()), err_msg=key)


def test_qg_circuit_known_answers_on_gpu(cuda):
    c = recipes.qg_test_circuit(pq)
    E = c.cost(recipes.QG_DEFAULT_ANGLES)
    assert abs(E - 0.46135870050914374) < 1e-5
    assert pq.measure.Measurements(c).get_effective_quantum_dimension(1e-12) == 12


@pytest.mark.parametrize("N", [4, 6, 8])
def test_npqc_qfim_is_identity_on_gpu(cuda, N):
    for P in range(1, 2 ** (N // 2) + 1):
        layers, theta_ref = pq.templates.NPQC_layers(P, N)
        c = pq.PQC(N)
        for l in layers:
            c.add_layer(l)
        c.state = c.run(theta_ref)
        F = pq.measure.Measurements(c).get_QFI()
        masked = np.where(F < 1e-12, 0, F)
        assert np.count_nonzero(masked - np.diag(np.diag(masked))) == 0


def test_adjoint_gradient_matches_reference_golden(cuda, golden):
    for key in _cases(golden):
        if f"{key}/grad_vector" not in golden.files:
            continue
        c = _with_init(_build(key), golden, key)
        N = c.n_qubits
        if f"{key}/energy_H" in golden.files:
            c.set_H(pq.templates.TFIM_hamiltonian(N, 1.0, 0.5 if key.startswith("tpl") else 0.0))
        g = pq.measure.Measurements(c).get_gradient_vector(list(golden[f"{key}/theta"]))
        np.testing.assert_allclose(g, golden[f"{key}/grad_vector"], atol=1e-9, err_msg=key)


@pytest.mark.parametrize("build,N,L", [(recipes.he_ladder, 8, 4), (recipes.he_ladder, 12, 6),
                                       (recipes.tfim_style, 10, 3), (recipes.npqc_style, 14, 4),
                                       (recipes.he_ladder, 16, 3), (recipes.tfim_style, 17, 2)])
def test_forward_batch_matches_oracle(cuda, build, N, L):
    c = build(pq, N, L)
    P = c.n_columns()
    th = np.random.default_rng(N).random((3, P)) * 2 * np.pi
    ref = O.run_batch(c.gates, N, th)
    got = _np(c.run_batch(th))
    np.testing.assert_allclose(got, ref, atol=AMP_TOL)
    plain = _np(c.run_batch(th, mode="plain"))
    np.testing.assert_allclose(plain, ref, atol=AMP_TOL)
    f64 = _np(c.run_batch(th, mode="f64"))  # the same sweeps in native FP64
    np.testing.assert_allclose(f64, ref, atol=AMP_TOL)


@pytest.mark.parametrize("build,N,L", [(recipes.he_ladder, 14, 6), (recipes.tfim_style, 14, 4),
                                       (recipes.npqc_style, 13, 4)])
def test_scaled_rotations_at_special_angles(cuda, build, N, L):
    # The sweeps apply RY/RX as cos(t/2) * [[1, -tan], [tan, 1]]: angles where cos(t/2) vanishes or is tiny
    # exercise the growth bound (rotations past it take the general form) and the factor bookkeeping.
    c = build(pq, N, L)
    P = c.n_columns()
    rng = np.random.default_rng(7)
    special = np.array([0.0, np.pi, -np.pi, 3 * np.pi, np.pi / 2, np.pi - 1e-9, np.pi + 1e-6, 2 * np.pi])
    th = np.stack([rng.choice(special, P),
                   rng.random(P) * 2 * np.pi,
                   np.where(rng.random(P) < 0.5, np.pi, rng.random(P) * 2 * np.pi),
                   np.full(P, np.pi),
                   np.pi - 10.0 ** -rng.integers(1, 12, P)])
    ref = O.run_batch(c.gates, N, th)
    np.testing.assert_allclose(_np(c.run_batch(th)), ref, atol=AMP_TOL)
    np.testing.assert_allclose(_np(c.run_batch(th, mode="f64")), ref, atol=AMP_TOL)
    if build is recipes.he_ladder:
        # per-row limits run the unrelabelled plan with the same scaled rotations (one op per gate here)
        G = len(c.gates)
        cuts = [G // 3, G, 1, G // 2 + 1, 0]
        got = _np(c.program.run(th, row_limit=cuts))
        for r, g in enumerate(cuts):
            gates = c.gates[:g]
            n = sum(int(x.param_count) if x.is_param else 0 for x in gates)
            np.testing.assert_allclose(got[r], O.run(gates, N, th[r, :n]), atol=AMP_TOL)


@pytest.mark.parametrize("k", [4, 5, 6, 7, 8])
def test_forced_small_tiles_exercise_multi_sweep_paths(cuda, k):
    # every gate class with most qubits outside the tile: fixed-bit controls, tile phases, CZ/RZZ on fixed bits
    N = 9
    c = recipes.every_gate(pq, N)
    c.add_layer([pq.R_y(i, N) for i in range(N)] + [pq.CNOT([i, (i + 3) % N], N) for i in range(N)]
                + [pq.R_zz([0, 8], N), pq.CZ([8, 1], N), pq.R_xx([2, 7], N), pq.fSim([3, 6], N)])
    c.set_tile_qubits(k)
    assert c.program.info()["n_sweeps"] > 1
    P = c.n_columns()
    th = np.random.default_rng(k).random((2, P)) * 2 * np.pi
    psi0 = O.product_state([1, 0, 1, 1, 0, 0, 1, 0, 1])
    c.initial_state = psi0
    ref = O.run_batch(c.gates, N, th, psi0)
    np.testing.assert_allclose(_np(c.run_batch(th)), ref, atol=AMP_TOL)
    np.testing.assert_allclose(_np(c.run_batch(th, mode="f64")), ref, atol=AMP_TOL)
    st = (np.random.default_rng(0).standard_normal(2 ** N) + 1j * np.random.default_rng(1).standard_normal(2 ** N))
    st /= np.linalg.norm(st)
    c.initial_state = st
    np.testing.assert_allclose(_np(c.run_batch(th)), O.run_batch(c.gates, N, th, st), atol=AMP_TOL)


def test_measures_match_reference_golden(cuda, golden):
    gates.rng = np.random.default_rng(1)
    c = recipes.he_ladder(pq, 4, 4)
    m = pq.measure.Measurements(c)
    em = m.efficient_measurements(101)
    gates.rng = np.random.default_rng(1)
    full = m.efficient_measurements(101, full_data=True)
    np.testing.assert_allclose(full["Expr"], golden["em/he4/overlaps"], atol=AMP_TOL)
    np.testing.assert_allclose(full["Ent"], golden["em/he4/q"], atol=AMP_TOL)
    np.testing.assert_allclose(full["Magic"], golden["em/he4/magics"], atol=1e-9)
    np.testing.assert_allclose(full["GKP"], golden["em/he4/gkps"], atol=1e-9)
    assert abs(em["Expr"] - float(golden["em/he4/expr"])) < 1e-9
    np.testing.assert_allclose(em["Ent"], golden["em/he4/ent"], atol=1e-10)
    np.testing.assert_allclose(em["Magic"], golden["em/he4/magic"], atol=1e-9)
    np.testing.assert_allclose(em["GKP"], golden["em/he4/gkp"], atol=1e-9)
    gates.rng = np.random.default_rng(1)
    c3 = pq.templates.generate_circuit("generic_HE", 3, 3)
    assert abs(pq.measure.Measurements(c3).expressibility(150) - float(golden["expr/generic_HE3/value"])) < 1e-9
    gates.rng = np.random.default_rng(1)
    idle = pq.PQC(1)
    idle.add_layer([pq.I(0, 1)])
    e = pq.measure.Measurements(idle).efficient_measurements(400, measure_ent=False, measure_eom=False,
                                                             measure_GKP=False)["Expr"]
    assert abs(e - float(golden["em/idle/expr"])) < 1e-9
    gates.rng = np.random.default_rng(1)
    ca = pq.PQC(1)
    ca.add_layer([pq.H(0, 1), pq.R_z(0, 1)])
    e = pq.measure.Measurements(ca).efficient_measurements(400, measure_ent=False, measure_eom=False,
                                                           measure_GKP=False)["Expr"]
    assert abs(e - float(golden["em/circA/expr"])) < 1e-9
    gates.rng = np.random.default_rng(1)


def test_clifford_mode_matches_reference_golden(cuda, golden):
    import random

    gates.rng = np.random.default_rng(1)
    random.seed(5)
    c = recipes.he_ladder(pq, 3, 2)
    cl = pq.measure.Measurements(c).efficient_measurements(20, angles="clifford")
    np.testing.assert_allclose(cl["Magic"], golden["em/clifford3/magic"], atol=1e-9)
    np.testing.assert_allclose(cl["Ent"], golden["em/clifford3/ent"], atol=1e-10)
    assert abs(cl["Expr"] - float(golden["em/clifford3/expr"])) < 1e-9
    gates.rng = np.random.default_rng(1)


@pytest.mark.parametrize("N", [1, 2, 3, 4, 5, 6])
def test_magic_and_mw_match_reference_golden(cuda, golden, N):
    psi = golden[f"ket/{N}/psi"]
    m = pq.measure.Measurements(pq.PQC(N))
    assert abs(m.renyi_entropy_fast(psi) - float(golden[f"ket/{N}/magic"])) < 1e-9
    assert abs(m.gkp_fast(psi) - float(golden[f"ket/{N}/gkp"])) < 1e-9
    assert abs(m.single_Q(psi, N) - float(golden[f"ket/{N}/q"])) < AMP_TOL


def test_bell_state_on_gpu(cuda):
    bell = np.array([0, 1, -1, 0], dtype=np.complex128) / np.sqrt(2)
    m = pq.measure.Measurements(pq.PQC(2))
    assert abs(m.renyi_entropy_fast(bell)) < 1e-10
    assert abs(m.gkp_fast(bell)) < 1e-10
    assert abs(m.single_Q(bell, 2) - 1) < 1e-10


@pytest.mark.parametrize("N", [8, 10, 11, 12, 13])
def test_magic_wht_matches_oracle(cuda, oracle_pool, N):
    # N = 13 runs the radix-16 transform (its last pass is a partial one), smaller N the one-stage-per-pass kernel
    c = recipes.npqc_style(pq, N, N)
    th = np.random.default_rng(N).random((2 if N < 13 else 1, c.n_columns())) * 2 * np.pi
    states = c.run_batch(th)
    got = _np(engine.magic(states, 2.0))
    ref = oracle_pool.magic(_np(states), 2.0)
    np.testing.assert_allclose(got, ref, atol=1e-9, rtol=0)


def test_allpairs_histogram_matches_numpy(cuda):
    c = recipes.he_ladder(pq, 6, 3)
    th = np.random.default_rng(4).random((64, c.n_columns())) * 2 * np.pi
    states = c.run_batch(th)
    F, counts, edges = engine.allpairs_fidelity_hist(states, 75)
    ref_states = O.run_batch(c.gates, 6, th)
    Fr = MO.pair_fidelities(ref_states)
    np.testing.assert_allclose(_np(F), Fr, atol=AMP_TOL)
    ref_counts = np.histogram(Fr, bins=75, range=(0, 1))[0]
    near_edge = np.abs(Fr[:, None] - np.linspace(0, 1, 76)[None, :]).min(axis=1) < 1e-12
    assert near_edge.sum() == 0
    np.testing.assert_array_equal(_np(counts), ref_counts)


def test_histogram_edge_cases(cuda):
    F = np.array([0.0, 1.0, 1.0 + 2.0 ** -52, -1e-300, 0.5, 1 / 75, np.nan, 0.9999999999999999])
    counts, edges = engine.histogram(F, 75)
    np.testing.assert_array_equal(_np(counts), np.histogram(F[~np.isnan(F)], bins=75, range=(0, 1))[0])
    # identical states: F within 1e-12 of 1.0 may land in the last bin or be dropped (edge exemption)
    c = recipes.he_ladder(pq, 5, 2)
    th = np.random.default_rng(0).random((1, c.n_columns())) * 2 * np.pi
    s = c.run_batch(np.repeat(th, 3, axis=0))
    Fs, counts, _ = engine.allpairs_fidelity_hist(s, 10)
    assert np.all(np.abs(_np(Fs) - 1) < 1e-12)
    assert _np(counts).sum() <= 3 and _np(counts)[:-1].sum() == 0


def test_empty_and_degenerate_inputs(cuda):
    c = recipes.he_ladder(pq, 4, 1)
    assert c.run_batch(np.zeros((0, c.n_columns()))).shape == (0, 16)
    F, counts, _ = engine.allpairs_fidelity_hist(c.run_batch(np.zeros((1, c.n_columns()))), 5)
    assert F.numel() == 0 and int(counts.sum()) == 0
    assert pq.measure.Measurements(c).efficient_measurements(0)["Expr"] == -1
    empty = pq.PQC(3)
    empty.add_layer([])
    np.testing.assert_allclose(_np(empty.run([])), O.basis_state(3), atol=0)


def test_adjoint_matches_central_finite_differences(cuda):
    N = 8
    c = recipes.he_ladder(pq, N, 2)
    c.set_H(pq.hamiltonian.xxz_open(N, 0.5))
    th = np.random.default_rng(3).random(c.n_columns()) * 2 * np.pi
    E, g = c.program.energy_grad(th[None, :], c.H, 0)
    h = 1e-6
    fd = []
    for j in range(len(th)):
        tp, tm = th.copy(), th.copy()
        tp[j] += h
        tm[j] -= h
        Ep = float(c.cost_batch(tp[None, :])[0])
        Em = float(c.cost_batch(tm[None, :])[0])
        fd.append((Ep - Em) / (2 * h))
    np.testing.assert_allclose(_np(g[0]), fd, atol=2e-8)
    ref = O.gradient_vector(c.gates, N, th, O.xxz_open(N, 0.5))
    np.testing.assert_allclose(_np(g[0]), ref, atol=1e-10)


def test_complex64_sampling_mode_error_is_bounded(cuda):
    c = recipes.he_ladder(pq, 12, 12)
    th = np.random.default_rng(0).random((4, c.n_columns())) * 2 * np.pi
    exact = c.run_batch(th)
    approx = c.run_batch(th, mode="c64").to(torch.complex128)
    err = float((exact - approx).abs().max())
    assert err < 1e-5
    Fe = engine.fidelity_pairs(exact[:2], exact[2:])
    Fa = engine.fidelity_pairs(approx[:2], approx[2:])
    assert float((Fe - Fa).abs().max()) < 1e-5


@pytest.mark.parametrize("N,L", [(20, 20)])
def test_full_size_properties(cuda, N, L):
    # size-independent checks at the benchmark size: unit norm, agreement of the fused and plain paths,
    # and an inverse-circuit round trip back to |0...0>
    c = pq.templates.hardware_efficient_ladder(N, L)
    th = np.random.default_rng(1).random((2, c.n_columns())) * 2 * np.pi
    psi = c.run_batch(th)
    norms = torch.linalg.vector_norm(psi, dim=1)
    assert float((norms - 1).abs().max()) < 1e-12
    plain = c.run_batch(th, mode="plain")
    assert float((psi - plain).abs().max()) < AMP_TOL
    inv = pq.PQC(N)
    layer = [pq.CNOT([i, i + 1], N) for i in reversed(range(N - 1))]
    layer += [pq.R_z(i, N) for i in reversed(range(N))] + [pq.R_y(i, N) for i in reversed(range(N))]
    inv.add_layer(layer, n=L)
    P = c.n_columns()
    rows = th.reshape(2, L, 2 * N)[:, ::-1, :]
    inv_th = -np.concatenate([rows[:, :, N:][:, :, ::-1], rows[:, :, :N][:, :, ::-1]], axis=2).reshape(2, P)
    inv.initial_state = psi[0]
    back = inv.run_batch(inv_th[:1])
    assert abs(float(back[0, 0].abs()) - 1) < 1e-10
    Q = engine.mw(psi)
    assert float(Q.min()) > 0.5
    # every bulk tile load of these multi-sweep runs completed within its wait limit
    assert c.program.status() == 0 and inv.program.status() == 0


@pytest.mark.parametrize("N", [12, 13, 14, 17, 20, 22])
def test_meyer_wallach_matches_oracle(cuda, N):
    # N >= 12 runs the two-pass kernel over runs of 2^11-amplitude tiles; random states (not circuit
    # outputs) give every qubit a non-trivial reduced state
    rows = 3 if N < 22 else 2
    rng = np.random.default_rng(N)
    st = rng.standard_normal((rows, 2 ** N)) + 1j * rng.standard_normal((rows, 2 ** N))
    st /= np.linalg.norm(st, axis=1, keepdims=True)
    st[0] = O.run(recipes.he_ladder(pq, N, 2).gates, N, rng.random(4 * N) * 2 * np.pi)
    Q = _np(engine.mw(torch.from_numpy(st).cuda()))
    want = np.array([MO.single_Q(s, N) for s in st])
    np.testing.assert_allclose(Q, want, atol=1e-11, rtol=0)


def test_launch_shapes_give_identical_states(cuda):
    # the sweep kernel's launch variants (CTAs per SM) run the same arithmetic: bit-identical states
    c = pq.templates.hardware_efficient_ladder(16, 4)
    th = np.random.default_rng(2).random((3, c.n_columns())) * 2 * np.pi
    ref = _np(c.run_batch(th))
    for ctas, threads in ((3, 0), (3, 128), (2, 0)):
        c.program.set_launch(ctas, threads)
        np.testing.assert_array_equal(_np(c.run_batch(th)), ref)
    timings = c.autotune(3)
    assert timings and all(ms > 0 for ms in timings.values())
    np.testing.assert_allclose(_np(c.run_batch(th)), O.run_batch(c.gates, 16, th), atol=AMP_TOL)


@pytest.mark.parametrize("rows", [1, 7, 64])
def test_blocked_qfim_matches_full(cuda, rows):
    # derivative states produced and contracted in row blocks (the path taken when P x 2^N exceeds the budget)
    c = recipes.every_gate(pq, 6)
    c.add_layer([pq.R_y(i, 6) for i in range(6)] + [pq.fSim([0, 1], 6)])
    th = np.random.default_rng(rows).random(c.n_columns()) * 2 * np.pi
    c.run(list(th))
    m = pq.measure.Measurements(c)
    full = m.get_QFI()
    blocked = engine.qfim_blocked(c.program, th[None, :], c.state, rows).cpu().numpy()
    np.testing.assert_allclose(blocked, full, rtol=QFIM_RTOL, atol=1e-12)
    budget = m.get_QFI(max_state_bytes=3 * 16 * 2 ** 6)
    np.testing.assert_allclose(budget, full, rtol=QFIM_RTOL, atol=1e-12)


def test_gram_cross_matches_oracle(cuda):
    rng = np.random.default_rng(5)
    a = rng.standard_normal((37, 2 ** 9)) + 1j * rng.standard_normal((37, 2 ** 9))
    b = rng.standard_normal((45, 2 ** 9)) + 1j * rng.standard_normal((45, 2 ** 9))
    G = _np(engine.gram_cross(torch.from_numpy(a), torch.from_numpy(b)))
    np.testing.assert_allclose(G, np.conj(a) @ b.T, rtol=1e-12, atol=1e-10)


def test_cnot_rz_cnot_runs_as_one_zz_rotation(cuda):
    # the forward plan applies each CNOT-RZ-CNOT of the TFIM-style ansatz as one diagonal ZZ rotation; limits
    # inside such a triple are rejected, limits at gate boundaries give the oracle's prefix circuits
    N, L = 14, 3
    c = pq.templates.tfim_style(N, L)
    low = c.program.lowered
    kinds = low.ops["kind"]
    i = next(j for j in range(len(kinds) - 2)
             if kinds[j] == _lib.PQC_OP_CNOT and kinds[j + 1] == _lib.PQC_OP_RZ and kinds[j + 2] == _lib.PQC_OP_CNOT)
    lib = c.program.lib
    assert lib.pqc_program_limit_ok(c.program.handle, i) == 1
    assert lib.pqc_program_limit_ok(c.program.handle, i + 1) == 0
    assert lib.pqc_program_limit_ok(c.program.handle, i + 2) == 0
    assert lib.pqc_program_limit_ok(c.program.handle, i + 3) == 1
    th = np.random.default_rng(8).random((3, c.n_columns())) * 2 * np.pi
    with pytest.raises(ValueError):
        c.program.run(th, row_limit=[i + 1] * 3)
    cuts = [i, i + 3, len(c.gates)]
    got = _np(c.program.run(th, row_limit=cuts))
    for b, g in enumerate(cuts):
        gates = c.gates[:g]  # one op per gate in this ansatz
        P = sum(int(x.param_count) if x.is_param else 0 for x in gates)
        np.testing.assert_allclose(got[b], O.run(gates, N, th[b, :P]), atol=AMP_TOL)
    assert c.program.info()["n_sweeps"] < pq.templates.hardware_efficient_ladder(N, L).program.info()["n_sweeps"] + 1


@pytest.mark.parametrize("build,N,K", [(lambda pq_, n: recipes.he_ladder(pq_, n, 4), 14, 5),
                                       (lambda pq_, n: recipes.every_gate(pq_, n), 7, 3),
                                       (lambda pq_, n: recipes.fsim_mix(pq_, n), 6, 4),
                                       (lambda pq_, n: pq_.templates.tfim_style(n, 3), 15, 8)])
def test_checkpointed_derivative_states_match(cuda, build, N, K):
    # layer checkpointing: runs start from stored intermediate states instead of the initial state
    c = build(pq, N)
    th = np.random.default_rng(N + K).random((1, c.n_columns())) * 2 * np.pi
    full = _np(c.program.gradient_states(th, checkpoints=0))
    ck = _np(c.program.gradient_states(th, checkpoints=K))
    np.testing.assert_allclose(ck, full, atol=AMP_TOL)
    ref = O.get_gradients(c.gates, N, th[0])
    np.testing.assert_allclose(ck, ref, atol=AMP_TOL)


@pytest.mark.parametrize("name,N,p,K", [("NPQC", 10, 5, 4), ("Circuit_9", 9, 4, 3), ("generic_HE", 14, 3, 5),
                                         ("NPQC", 14, 4, 3)])
def test_reordered_and_regrouped_plans_match_oracle(cuda, name, N, p, K):
    # The planner reorders commuting ops so that rotations pair and diagonal ops share phase-block passes (the
    # NPQC layers interleave RY and RZ), and moves each derivative generator later past ops it commutes with so
    # that it splits no such pass.  States, per-row op limits and checkpointed derivative runs must all still
    # give the oracle's results.
    c = pq.templates.generate_circuit(name, N, p)
    if name == "NPQC":
        c = pq.PQC(N)
        for layer in pq.templates.NPQC_layers(p, N)[0]:
            c.add_layer(layer)
    P = c.n_columns()
    th = np.random.default_rng(N + p).random((3, P)) * 2 * np.pi
    psi0 = None  # these templates start from |0...0>
    ref = O.run_batch(c.gates, N, th, psi0)
    np.testing.assert_allclose(_np(c.run_batch(th)), ref, atol=AMP_TOL)
    last = c.program.lowered.gate_last
    G = len(c.gates)
    cut_gates = [G // 3, G, (2 * G) // 3]
    limits = [int(last[g - 1]) + 1 for g in cut_gates]
    got = _np(c.program.run(th, row_limit=limits))
    for r, g in enumerate(cut_gates):
        gates = c.gates[:g]
        n = sum(int(x.param_count) if x.is_param else 0 for x in gates)
        np.testing.assert_allclose(got[r], O.run(gates, N, th[r, :n], psi0), atol=AMP_TOL)
    full = _np(c.program.gradient_states(th[:1], checkpoints=0))
    ck = _np(c.program.gradient_states(th[:1], checkpoints=K))
    plain = _np(c.program.gradient_states(th[:1], plain=True))
    np.testing.assert_allclose(full, plain, atol=AMP_TOL)
    np.testing.assert_allclose(ck, plain, atol=AMP_TOL)
    np.testing.assert_allclose(ck, O.get_gradients(c.gates, N, th[0], psi0), atol=AMP_TOL)


@pytest.mark.parametrize("name,N,p,K", [("generic_HE", 15, 3, 5), ("qg_circuit", 14, 3, 4), ("fsim", 12, 3, 3),
                                         ("Circuit_2", 16, 2, 6)])
def test_relabelled_derivative_sweeps_match_unrelabelled(cuda, monkeypatch, name, N, p, K):
    # Derivative runs take relabelled sweeps (CNOTs folded into the tile index, generators applied through the
    # index masks) when they apply every op of the sweep, and the unrelabelled twin when their checkpoint start
    # falls inside it.  Against the twin alone and against the oracle, from the start and from checkpoints.
    c = pq.templates.generate_circuit(name, N, p)  # the program-level calls below start from |0...0>
    th = np.random.default_rng(N * p).random((1, c.n_columns())) * 2 * np.pi
    got = {}
    for ck in (0, K):
        got[ck] = _np(c.program.gradient_states(th, checkpoints=ck))
    monkeypatch.setenv("PQC_NO_LAZY_DERIV", "1")
    for ck in (0, K):
        plain = _np(c.program.gradient_states(th, checkpoints=ck))
        np.testing.assert_allclose(got[ck], plain, atol=1e-13)
    monkeypatch.delenv("PQC_NO_LAZY_DERIV")
    ref = O.get_gradients(c.gates, N, th[0])
    for ck in (0, K):
        np.testing.assert_allclose(got[ck], ref, atol=AMP_TOL)


@pytest.mark.parametrize("N,L,B", [(8, 4, 5), (16, 3, 2)])
def test_cuda_graph_replay_matches_direct_runs(cuda, N, L, B):
    c = pq.templates.hardware_efficient_ladder(N, L)
    g = engine.GraphedRun(c.program, B)
    for seed in (0, 1):
        th = np.random.default_rng(seed).random((B, c.n_columns())) * 2 * np.pi
        got = _np(g(th)).copy()
        np.testing.assert_array_equal(got, _np(c.program.run(th)))
    np.testing.assert_allclose(got, O.run_batch(c.gates, N, th), atol=AMP_TOL)


def _counts(psi, nbins, keep):
    F, counts, _ = engine.allpairs_fidelity_hist(psi, nbins, keep_samples=keep)
    return _np(counts), (None if F is None else _np(F))


@pytest.mark.parametrize("N,S", [(10, 60), (6, 70), (6, 90), (7, 129), (8, 201)])
def test_certified_histogram_counts_equal_exact_counts(cuda, N, S):
    # counts-only histograms come from an FP32 Gram with a certified error bound; pairs it cannot place are
    # recomputed in double-float, so the counts equal those of the double-float path (S covers full, partial
    # and nearly empty 64-state tiles)
    c = recipes.he_ladder(pq, N, 4)
    th = np.random.default_rng(21 + S).random((S, c.n_columns())) * 2 * np.pi
    psi = c.run_batch(th)
    fast, _ = _counts(psi, 75, False)
    exact, F = _counts(psi, 75, True)
    np.testing.assert_array_equal(fast, exact)
    np.testing.assert_array_equal(fast, np.histogram(F, bins=75, range=(0, 1))[0])


def test_certified_histogram_refines_pairs_at_bin_edges(cuda):
    # pairs whose fidelity sits 1e-9 from a bin edge cannot be placed by the FP32 bound and are recomputed
    N, nbins = 9, 10
    D = 2 ** N
    base = np.zeros(D, complex)
    base[0] = 1.0
    states = [base]
    for edge in (0.2, 0.5, 0.7):
        for off in (-1e-9, 1e-9):
            t = np.arccos(np.sqrt(edge + off))
            s = np.zeros(D, complex)
            s[0], s[3] = np.cos(t), np.sin(t)
            states.append(s)
    rng = np.random.default_rng(3)
    for _ in range(20):
        v = rng.standard_normal(D) + 1j * rng.standard_normal(D)
        states.append(v / np.linalg.norm(v))
    psi = torch.from_numpy(np.array(states))
    fast, _ = _counts(psi, nbins, False)
    exact, F = _counts(psi, nbins, True)
    np.testing.assert_array_equal(fast, exact)
    ref = np.array([abs(np.vdot(states[a], states[b])) ** 2 for a in range(len(states)) for b in range(a + 1, len(states))])
    np.testing.assert_array_equal(fast, np.histogram(ref, bins=nbins, range=(0, 1))[0])


def test_certified_histogram_falls_back_when_many_pairs_are_undecided(cuda):
    # 4950 pairs all within 1e-9 of the last edge: more than the refinement list holds, so every pair is
    # recounted with the double-float Gram
    N, S = 8, 100
    D = 2 ** N
    rng = np.random.default_rng(4)
    v = rng.standard_normal(D) + 1j * rng.standard_normal(D)
    v /= np.linalg.norm(v)
    states = []
    for i in range(S):
        w = v + 1e-6 * (rng.standard_normal(D) + 1j * rng.standard_normal(D)) / np.sqrt(D)
        states.append(w / np.linalg.norm(w))
    psi = torch.from_numpy(np.array(states))
    fast, _ = _counts(psi, 75, False)
    exact, _ = _counts(psi, 75, True)
    np.testing.assert_array_equal(fast, exact)
    assert fast.sum() == S * (S - 1) // 2
