"""GPU parity at the configurations `bench.py` times, against the FP64 oracle.

Each test runs the CUDA path through the C ABI at the benchmark's own sizes and
checks it against the oracle (`oracle/`), evaluated row by row on the host
cores (`oracle_pool`):
  * batched sampling, HE ladder and TFIM-style ansatz, N = 20, L = 20: amplitudes;
  * the certified counts-only histogram of the first 201 states (20100 pairs,
    75 bins) against np.histogram of the oracle's fidelities of the same states;
  * the complex64 sampling mode's error against the oracle states;
  * differentiation, HE ladder N = 16, L = 8 (P = 256): <H> and dE/dtheta by
    the adjoint for TFIM h = 1 and XXZ Delta = 0.5, the derivative states, the
    256 x 256 QFIM and its effective quantum dimension;
  * magic, NPQC-style N = 12: Renyi-2 over all 4^N Pauli strings.
Tolerances: 1e-10 absolute on amplitudes, energies and gradient entries, 1e-8
relative on QFIM entries, histogram counts identical (no fidelity lies within
1e-12 of a bin edge).  The measured errors are printed (pytest -s).
"""
import numpy as np
import pytest

from oracle import measures_oracle as MO
from oracle import pqc_oracle as O
import pyramaterised_gb300 as pq
from pyramaterised_gb300 import engine

pytestmark = pytest.mark.gpu
AMP_TOL = 1e-10
QFIM_RTOL = 1e-8
N20, L20, S = 20, 20, 201


def _np(t):
    return t.detach().cpu().numpy()


def _theta(c, rows, seed):
    return np.random.default_rng(seed).random((rows, c.n_columns())) * 2 * np.pi


@pytest.fixture(scope="module")
def he20(cuda, oracle_pool):
    """The HE N = 20, L = 20 batch of the fidelity histogram (S rows on the device) and the oracle's first two."""
    c = pq.templates.hardware_efficient_ladder(N20, L20)
    th = _theta(c, S, 1234)
    psi = c.run_batch(th)
    ref = oracle_pool.states(("hardware_efficient_ladder", N20, L20), th[:2])
    return c, th, psi, ref


def test_he_n20_states_match_oracle(he20):
    c, th, psi, ref = he20
    err = float(np.abs(_np(psi[:2]) - ref).max())
    print(f"HE N=20 L=20 double-float: max |psi - oracle| = {err:.3e}")
    assert err < AMP_TOL
    assert c.program.status() == 0


def test_tfim_style_n20_states_match_oracle(cuda, oracle_pool):
    c = pq.templates.tfim_style(N20, L20)
    th = _theta(c, 2, 77)
    psi = _np(c.run_batch(th))
    ref = oracle_pool.states(("tfim_style", N20, L20), th)
    err = float(np.abs(psi - ref).max())
    print(f"TFIM-style N=20 L=20 double-float: max |psi - oracle| = {err:.3e}")
    assert err < AMP_TOL
    assert c.program.status() == 0


def test_certified_histogram_s201_n20_matches_numpy(he20):
    c, th, psi, ref = he20
    _, counts, _ = engine.allpairs_fidelity_hist(psi, 75, keep_samples=False)
    host = _np(psi)
    F = MO.pair_fidelities(host)
    assert len(F) == S * (S - 1) // 2
    edges = np.linspace(0, 1, 76)
    assert np.abs(F[:, None] - edges[None, :]).min() > 1e-12
    np.testing.assert_array_equal(_np(counts), np.histogram(F, bins=75, range=(0, 1))[0])
    # the fidelities of the oracle's own states agree with those of the device states
    f01 = abs(np.vdot(ref[0], ref[1])) ** 2
    assert abs(f01 - F[0]) < AMP_TOL


def test_complex64_mode_error_against_oracle(he20):
    c, th, psi, ref = he20
    s64 = _np(c.run_batch(th[:2], mode="c64")).astype(np.complex128)
    amp = float(np.abs(s64 - ref).max())
    norm = float(np.linalg.norm(s64 - ref, axis=1).max())
    f_err = abs(abs(np.vdot(s64[0], s64[1])) ** 2 - abs(np.vdot(ref[0], ref[1])) ** 2)
    print(f"complex64 HE N=20 L=20: max |psi - oracle| = {amp:.3e}, max ||psi - oracle||_2 = {norm:.3e}, "
          f"|F - F_oracle| = {f_err:.3e}")
    assert norm < 1e-4 and f_err < 1e-8


@pytest.fixture(scope="module")
def he16(cuda, oracle_pool):
    """HE N = 16, L = 8 (P = 256): two parameter rows, their oracle states and derivative states."""
    c = pq.templates.hardware_efficient_ladder(16, 8)
    th = _theta(c, 2, 16)
    spec = ("hardware_efficient_ladder", 16, 8)
    psi = oracle_pool.states(spec, th)
    grads = [oracle_pool.gradient_states(spec, t) for t in th]
    return c, th, psi, grads


@pytest.mark.parametrize("name", ["tfim_h1", "xxz_d0.5"])
def test_adjoint_energy_gradient_n16_p256_matches_oracle(he16, name):
    c, th, psi, grads = he16
    N = 16
    H, Ho = ((pq.hamiltonian.tfim_open(N, 1.0), O.tfim_open(N, 1.0)) if name == "tfim_h1"
             else (pq.hamiltonian.xxz_open(N, 0.5), O.xxz_open(N, 0.5)))
    E, g = c.program.energy_grad(th, H)
    E, g = _np(E), _np(g)
    assert g.shape == (2, 256)
    for r in range(2):
        Hpsi = O.apply_hamiltonian(Ho, psi[r], N)
        e_ref = float(np.real(np.vdot(psi[r], Hpsi)))
        # measure.py:461-471: dE/dtheta_i = 2 Re <psi|H|d_i psi> = 2 Re <H psi|d_i psi> (H Hermitian)
        g_ref = 2 * np.real(np.conj(Hpsi) @ grads[r].T)
        e_err, g_err = abs(E[r] - e_ref), float(np.abs(g[r] - g_ref).max())
        print(f"adjoint {name} N=16 P=256 row {r}: |E - oracle| = {e_err:.3e}, max |dE - oracle| = {g_err:.3e}")
        assert e_err < AMP_TOL and g_err < AMP_TOL


def test_derivative_states_and_qfim_n16_p256_match_oracle(he16):
    c, th, psi, grads = he16
    t0 = list(th[0])
    c.state = c.run(t0)
    err_state = float(np.abs(_np(c.state) - psi[0]).max())
    dpsi = _np(c.get_gradients())
    err_d = float(np.abs(dpsi - grads[0]).max())
    F = pq.measure.Measurements(c).get_QFI()
    Fr = O.get_QFI(psi[0], grads[0])
    rel = float(np.abs(F - Fr).max() / np.abs(Fr).max())
    print(f"QFIM N=16 P=256: max |psi - oracle| = {err_state:.3e}, max |d psi - oracle| = {err_d:.3e}, "
          f"max |F - F_oracle| / max |F_oracle| = {rel:.3e}")
    assert err_state < AMP_TOL and err_d < AMP_TOL
    assert F.shape == (256, 256)
    np.testing.assert_allclose(F, Fr, rtol=QFIM_RTOL, atol=QFIM_RTOL * np.abs(Fr).max())
    m = pq.measure.Measurements(c)
    assert m.get_effective_quantum_dimension(1e-12) == O.effective_quantum_dimension(Fr, 1e-12)
    # the same QFIM with the Gram in native FP64
    F64 = engine.qfim(c.state, c.get_gradients(), fp64=True).cpu().numpy()
    rel64 = float(np.abs(F64 - Fr).max() / np.abs(Fr).max())
    print(f"QFIM N=16 P=256, FP64 Gram: max |F - F_oracle| / max |F_oracle| = {rel64:.3e}")
    np.testing.assert_allclose(F64, Fr, rtol=QFIM_RTOL, atol=QFIM_RTOL * np.abs(Fr).max())


def test_magic_n12_matches_oracle(cuda, oracle_pool):
    c = pq.templates.npqc_style(12, 12)
    th = _theta(c, 2, 12)
    states = c.run_batch(th)
    got = _np(engine.magic(states, 2.0))
    ref = oracle_pool.magic(_np(states), 2.0)
    err = float(np.abs(got - ref).max())
    print(f"Renyi-2 magic NPQC-style N=12: max |M - oracle| = {err:.3e}")
    assert err < 1e-9
    # the states themselves against the oracle's
    ref_states = oracle_pool.states(("npqc_style", 12, 12), th)
    assert float(np.abs(_np(states) - ref_states).max()) < AMP_TOL


# ---------------------------------------------------------------- the other sizes of the batched-sampling config
@pytest.mark.parametrize("name,N,B", [("hardware_efficient_ladder", 12, 4096), ("tfim_style", 12, 4096),
                                      ("hardware_efficient_ladder", 16, 1024), ("tfim_style", 16, 1024)])
def test_batched_sampling_config_matches_oracle(cuda, oracle_pool, name, N, B):
    # L = N, B theta rows per launch: rows 0, 1 and B-1 against the oracle; the counts-only 20100-pair histogram of
    # the first 201 states against np.histogram of their FP64 fidelities; Meyer-Wallach of 8 rows against the
    # oracle's partial traces; the complex64 mode's fidelity error against the oracle states
    c = getattr(pq.templates, name)(N, N)
    th = _theta(c, B, 500 + N)
    psi = c.run_batch(th)
    rows = [0, 1, B - 1]
    ref = oracle_pool.states((name, N, N), th[rows])
    err = float(np.abs(_np(psi[rows]) - ref).max())
    print(f"{name} N={N} B={B}: max |psi - oracle| = {err:.3e}")
    assert err < AMP_TOL
    host = _np(psi[:S])
    F = MO.pair_fidelities(host)
    _, counts, _ = engine.allpairs_fidelity_hist(psi[:S], 75, keep_samples=False)
    np.testing.assert_array_equal(_np(counts), np.histogram(F, bins=75, range=(0, 1))[0])
    Q = _np(engine.mw(psi[:8]))
    want = np.array([MO.single_Q(s, N) for s in _np(psi[:8])])
    np.testing.assert_allclose(Q, want, atol=1e-11, rtol=0)
    s64 = _np(c.run_batch(th[:2], mode="c64")).astype(np.complex128)
    f_err = abs(abs(np.vdot(s64[0], s64[1])) ** 2 - abs(np.vdot(ref[0], ref[1])) ** 2)
    print(f"{name} N={N}: complex64 |F - F_oracle| = {f_err:.3e}")
    assert f_err < 1e-6
    assert c.program.status() == 0


def test_plain_small_config_matches_oracle(cuda):
    # N = 4, HE ladder L = 4 (P = 32), theta from seed 0: expressibility from S = 101 states (5050 pairs in
    # combinations order, 75 bins, d = 16), Meyer-Wallach averaged over 1000 states, the QFIM at 10 theta
    N, L = 4, 4
    c = pq.templates.hardware_efficient_ladder(N, L)
    rng = np.random.default_rng(0)
    th = rng.random((1000, c.n_columns())) * 2 * np.pi
    psi = c.run_batch(th)
    ref = O.run_batch(c.gates, N, th)
    np.testing.assert_allclose(_np(psi), ref, atol=AMP_TOL, rtol=0)
    _, counts, edges = engine.allpairs_fidelity_hist(psi[:101], 75, keep_samples=False)
    kl = float(engine.expr_kl(counts, edges, 16.0).item())
    want_kl = MO.expr(MO.pair_fidelities(ref[:101]), 16, 75)
    print(f"plain small: KL {kl:.12f} (oracle {want_kl:.12f})")
    assert abs(kl - want_kl) < 1e-10
    Q = float(_np(engine.mw(psi)).mean())
    assert abs(Q - np.mean([MO.single_Q(s, N) for s in ref])) < 1e-12
    m = pq.measure.Measurements(c)
    for t in th[:10]:
        c.state = c.run(list(t))  # get_QFI uses the circuit's current state (measure.py:33-71)
        F = m.get_QFI()
        want = O.get_QFI(O.run(c.gates, N, t), O.get_gradients(c.gates, N, t))
        np.testing.assert_allclose(F, want, atol=1e-10, rtol=0)
