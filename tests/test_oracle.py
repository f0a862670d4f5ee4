"""The oracle against the reference: its own known-answer tests and the golden
vectors produced by running the reference's code (tests/golden/make_golden.py)."""
import numpy as np
import pytest

import recipes
from oracle import measures_oracle as MO
from oracle import pqc_oracle as O
import pyramaterised_gb300 as pq


def _theta_for(golden, key):
    return golden[f"{key}/theta"]


def test_basic_gates_known_answers():
    # tests.py:64-87: fixed_R_y(pi/2)|0> -> 1/sqrt(2); H H |0> = |0>
    c = pq.PQC(1)
    c.add_layer([pq.fixed_R_y(0, 1, np.pi / 2)])
    psi = O.run(c.gates, 1, [])
    assert np.isclose(np.real(psi[1]), 1 / np.sqrt(2))
    c2 = pq.PQC(1)
    c2.add_layer([pq.H(0, 1)], n=2)
    assert np.allclose(O.run(c2.gates, 1, []), [1, 0], atol=1e-12)


def test_qg_circuit_known_answers(golden):
    # tests.py:158-213: energy 0.46135870050914374 (+-1e-5) and effective dimension 12
    c = recipes.qg_test_circuit(pq)
    th = recipes.QG_DEFAULT_ANGLES
    psi = O.run(c.gates, 4, th)
    E = O.expect(O.PauliTerms(O.zz_hamiltonian_terms(4)), psi, 4)
    assert abs(E - 0.46135870050914374) < 1e-5
    assert abs(E - float(golden["qg_test/energy_ZZ"])) < 1e-12
    grads = O.get_gradients(c.gates, 4, th)
    F = O.get_QFI(psi, grads)
    assert O.effective_quantum_dimension(F, 1e-12) == 12 == int(golden["qg_test/eqd"])
    np.testing.assert_allclose(F, golden["qg_test/qfim"], atol=1e-12)


@pytest.mark.parametrize("N", [4, 6, 8])
def test_npqc_qfim_is_diagonal(N):
    # tests.py:103-128
    for P in range(1, 2 ** (N // 2) + 1):
        layers, theta_ref = pq.templates.NPQC_layers(P, N)
        c = pq.PQC(N)
        for l in layers:
            c.add_layer(l)
        psi = O.run(c.gates, N, theta_ref)
        F = O.get_QFI(psi, O.get_gradients(c.gates, N, theta_ref))
        masked = np.where(F < 1e-12, 0, F)
        assert np.count_nonzero(masked - np.diag(np.diag(masked))) == 0


def test_bell_state_known_answers(golden):
    # tests.py:284-295: (|01> - |10>)/sqrt(2) has magic 0, GKP 0 and Q 1
    bell = np.array([0, 1, -1, 0], dtype=np.complex128) / np.sqrt(2)
    assert abs(MO.renyi_entropy_wht(bell)) < 1e-10
    assert abs(MO.gkp(bell)) < 1e-10
    assert abs(MO.single_Q(bell, 2) - 1) < 1e-10
    assert abs(float(golden["bell/magic"])) < 1e-10


def _golden_cases(golden):
    keys = sorted({k.rsplit("/", 1)[0] for k in golden.files if k.endswith("/state")})
    return keys


def _build(key):
    parts = key.split("/")
    if parts[0] == "tpl":
        return recipes.template_circuit(pq, parts[1], int(parts[2]), int(parts[3]))
    if parts[0] == "ansatz":
        return getattr(recipes, parts[1])(pq, int(parts[2]), int(parts[3]))
    if parts[0] == "special":
        return getattr(recipes, parts[1])(pq, 4)
    if parts[0] == "qg_test":
        return recipes.qg_test_circuit(pq)
    if parts[0] == "shared_nc":
        return recipes.shared_noncommuting(pq, int(parts[1]))
    raise KeyError(key)


def test_oracle_matches_reference_golden(golden):
    for key in _golden_cases(golden):
        c = _build(key)
        N = c.n_qubits
        th = golden[f"{key}/theta"]
        psi0 = golden[f"{key}/init"]
        psi = O.run(c.gates, N, th, psi0)
        np.testing.assert_allclose(psi, golden[f"{key}/state"], atol=1e-12, err_msg=key)
        if f"{key}/grads" in golden.files:
            grads = O.get_gradients(c.gates, N, th, psi0)
            np.testing.assert_allclose(grads, golden[f"{key}/grads"], atol=1e-12, err_msg=key)
            F = O.get_QFI(psi, grads)
            np.testing.assert_allclose(F, golden[f"{key}/qfim"], atol=1e-10, err_msg=key)
        H = O.PauliTerms(O.zz_hamiltonian_terms(N)) if N >= 2 else None
        if f"{key}/energy_H" in golden.files:
            H = O.tfim_reference(N, 1.0, 0.5 if key.startswith("tpl") else 0.0)
            assert abs(O.expect(H, psi, N) - float(golden[f"{key}/energy_H"])) < 1e-12, key
        if f"{key}/grad_vector" in golden.files:
            gv = O.gradient_vector(c.gates, N, th, H, psi0)
            np.testing.assert_allclose(gv, golden[f"{key}/grad_vector"], atol=1e-12, err_msg=key)


def test_oracle_measures_match_reference_golden(golden):
    # efficient_measurements(101) on the HE ladder with the global rng (measure.py:370-459)
    c = recipes.he_ladder(pq, 4, 4)
    P = 32
    th = np.random.default_rng(1).random((101, P)) * 2 * np.pi
    states = O.run_batch(c.gates, 4, th)
    res = MO.efficient_measurements(states, 4, full_data=True)
    np.testing.assert_allclose(res["Expr"], golden["em/he4/overlaps"], atol=1e-12)
    np.testing.assert_allclose(res["Ent"], golden["em/he4/q"], atol=1e-12)
    np.testing.assert_allclose(res["Magic"], golden["em/he4/magics"], atol=1e-10)
    np.testing.assert_allclose(res["GKP"], golden["em/he4/gkps"], atol=1e-10)
    summ = MO.efficient_measurements(states, 4)
    assert abs(summ["Expr"] - float(golden["em/he4/expr"])) < 1e-12
    np.testing.assert_allclose(summ["Ent"], golden["em/he4/ent"], atol=1e-12)


def test_pair_order_is_combinations_order():
    rs = np.random.default_rng(2)
    S = rs.standard_normal((7, 8)) + 1j * rs.standard_normal((7, 8))
    np.testing.assert_allclose(MO.pair_fidelities(S), MO.pair_fidelities_loop(S), rtol=1e-13)


@pytest.mark.parametrize("N", [1, 2, 3, 4, 5, 6])
def test_magic_wht_matches_reference(golden, N):
    psi = golden[f"ket/{N}/psi"]
    assert abs(MO.renyi_entropy_wht(psi) - float(golden[f"ket/{N}/magic"])) < 1e-10
    assert abs(MO.renyi_entropy_literal(psi) - float(golden[f"ket/{N}/magic"])) < 1e-10
    assert abs(MO.gkp(psi) - float(golden[f"ket/{N}/gkp"])) < 1e-10
    assert abs(MO.single_Q(psi, N) - float(golden[f"ket/{N}/q"])) < 1e-12


def test_histogram_edges_and_reference_bins():
    # np.histogram keeps F == 1.0 in the last bin and drops values above 1 (measure.py:153)
    F = np.array([0.0, 1.0, 1.0 + 2e-16, 0.5, 1 / 75])
    _, _, counts, edges = MO.gen_histo(F, 75)
    assert counts.sum() == 4 and counts[-1] == 1
    assert MO.reference_nbins(5000) == 37 and MO.reference_nbins(20100) == 150


def test_training_golden_is_consistent_with_the_oracle(golden, golden_meta):
    # the reference's train() trajectories (tests/golden/make_golden.py section 8): the recorded final energy
    # is the oracle's energy of the recorded final angles, and every trajectory decreases overall
    import pyramaterised_gb300 as pq
    import recipes

    H = O.tfim_reference(4, 1.0)
    for tag in ("grad_fixed", "grad_random", "qng_fixed"):
        key = f"train/{tag}"
        c = recipes.he_ladder(pq, 4, golden_meta["meta"][key]["layers"])
        th = golden[f"{key}/final_theta"]
        E = O.expect(H, O.run(c.gates, 4, th), 4)
        assert abs(E - float(golden[f"{key}/energy"])) < 1e-10, tag
        traj = golden[f"{key}/traj"]
        assert traj[-1] < traj[1] and len(traj) - 1 == golden_meta["meta"][key]["iterations"]
        assert abs(traj[-1] - float(golden[f"{key}/energy"])) < 1e-12
