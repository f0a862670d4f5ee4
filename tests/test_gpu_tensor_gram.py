"""The tensor-core (tcgen05, TF32) fidelity Gram and the counts-only histogram tier built on it.

`pqc_gram_tf32` must stay inside its stated bound |G - G_exact| <= delta_factor ||a|| ||b|| per component,
and `pqc_fidelity_hist` (counts only) must give the exact counts of np.histogram over the FP64 fidelities
(`_gen_f_samples` + `_gen_histo`, measure.py:123-159) whichever tier places a pair: the tensor-core bound,
the FP32 tier it hands over to when too many pairs are undecided, the exact recount of the listed pairs, or
the double-float recount of every pair.
"""
import numpy as np
import pytest
import torch

import recipes
import pyramaterised_gb300 as pq
from pyramaterised_gb300 import engine

pytestmark = pytest.mark.gpu


def _np(t):
    return t.detach().cpu().numpy()


def _mixed_states(N, S, seed):
    """HE circuit states, Haar-like random states, product states and repeated states."""
    rng = np.random.default_rng(seed)
    D = 2 ** N
    c = recipes.he_ladder(pq, N, 2)
    n_circ = S // 2
    th = rng.random((n_circ, c.n_columns())) * 2 * np.pi
    states = list(_np(c.run_batch(th)))
    while len(states) < S - 4:
        v = rng.standard_normal(D) + 1j * rng.standard_normal(D)
        states.append(v / np.linalg.norm(v))
    prod = np.zeros(D, complex)
    prod[0] = 1.0
    states.append(prod)
    prod2 = np.zeros(D, complex)
    prod2[D - 1] = 1j
    states.append(prod2)
    states.append(states[0].copy())
    states.append(states[1].copy())
    return np.array(states[:S])


@pytest.mark.parametrize("N,S", [(13, 2), (13, 100), (13, 129), (14, 201), (14, 256)])
def test_tensor_gram_is_within_its_bound(cuda, N, S):
    X = _mixed_states(N, S, seed=N + S)
    G, dfac = engine.gram_tf32(torch.from_numpy(X).cuda())
    G = _np(G)
    exact = X.conj() @ X.T
    norms = np.linalg.norm(X, axis=1)
    bound = dfac * np.outer(norms, norms)
    err_re = np.abs(G.real - exact.real)
    err_im = np.abs(G.imag - exact.imag)
    print(f"tensor-core Gram N={N} S={S}: delta_factor {dfac:.3e}, max component error / (|a||b|) "
          f"{max(err_re.max(), err_im.max()):.3e}")
    assert np.all(err_re <= bound) and np.all(err_im <= bound)
    # the TF32 rounding alone is a few 1e-4 of the norms: the products really come from the tensor cores
    assert max(err_re.max(), err_im.max()) > 1e-9


def _counts(psi, nbins, keep):
    F, counts, _ = engine.allpairs_fidelity_hist(psi, nbins, keep_samples=keep)
    return _np(counts), (None if F is None else _np(F))


@pytest.mark.parametrize("N,S", [(14, 201), (13, 100), (14, 256)])
def test_tensor_tier_counts_equal_exact_counts(cuda, N, S):
    c = recipes.he_ladder(pq, N, 4)
    th = np.random.default_rng(40 + S).random((S, c.n_columns())) * 2 * np.pi
    psi = c.run_batch(th)
    fast, _ = _counts(psi, 75, False)
    exact, F = _counts(psi, 75, True)
    np.testing.assert_array_equal(fast, exact)
    np.testing.assert_array_equal(fast, np.histogram(F, bins=75, range=(0, 1))[0])


def _edge_states(N, offsets, n_random, seed):
    D = 2 ** N
    base = np.zeros(D, complex)
    base[0] = 1.0
    states = [base]
    for edge in (0.2, 0.5, 0.7):
        for off in offsets:
            t = np.arccos(np.sqrt(edge + off))
            s = np.zeros(D, complex)
            s[0], s[5] = np.cos(t), np.sin(t)
            states.append(s)
    rng = np.random.default_rng(seed)
    for _ in range(n_random):
        v = rng.standard_normal(D) + 1j * rng.standard_normal(D)
        states.append(v / np.linalg.norm(v))
    return states


def test_tensor_tier_refines_pairs_near_bin_edges(cuda):
    # fidelities 1e-9 and 1e-4 from an edge: inside the tensor-core bound, so the pairs are listed and recomputed
    N, nbins = 13, 10
    states = _edge_states(N, (-1e-4, -1e-9, 1e-9, 1e-4), 40, seed=5)
    psi = torch.from_numpy(np.array(states))
    fast, _ = _counts(psi, nbins, False)
    exact, _ = _counts(psi, nbins, True)
    np.testing.assert_array_equal(fast, exact)
    ref = np.array([abs(np.vdot(states[a], states[b])) ** 2
                    for a in range(len(states)) for b in range(a + 1, len(states))])
    np.testing.assert_array_equal(fast, np.histogram(ref, bins=nbins, range=(0, 1))[0])


def test_tensor_tier_hands_over_to_the_fp32_tier(cuda):
    # 32640 pairs with fidelities spread over [0, 1]: about 30 % of them lie within the tensor-core bound of an
    # edge, more than the list holds, so the FP32 tier places them
    N, S = 13, 256
    D = 2 ** N
    phi = np.random.default_rng(6).random(S) * 2 * np.pi
    states = np.zeros((S, D), complex)
    states[:, 0] = 1 / np.sqrt(2)
    states[:, D // 2] = np.exp(1j * phi) / np.sqrt(2)
    psi = torch.from_numpy(states)
    fast, _ = _counts(psi, 75, False)
    exact, F = _counts(psi, 75, True)
    np.testing.assert_array_equal(fast, exact)
    ref = np.array([np.cos((phi[b] - phi[a]) / 2) ** 2 for a in range(S) for b in range(a + 1, S)])
    np.testing.assert_array_equal(fast, np.histogram(ref, bins=75, range=(0, 1))[0])


def test_tensor_tier_falls_back_to_the_double_float_recount(cuda):
    # every pair within 1e-9 of the last edge: neither low-precision tier can place them
    N, S = 13, 100
    D = 2 ** N
    rng = np.random.default_rng(7)
    v = rng.standard_normal(D) + 1j * rng.standard_normal(D)
    v /= np.linalg.norm(v)
    states = []
    for _ in range(S):
        w = v + 1e-6 * (rng.standard_normal(D) + 1j * rng.standard_normal(D)) / np.sqrt(D)
        states.append(w / np.linalg.norm(w))
    psi = torch.from_numpy(np.array(states))
    fast, _ = _counts(psi, 75, False)
    exact, _ = _counts(psi, 75, True)
    np.testing.assert_array_equal(fast, exact)
    assert fast.sum() == S * (S - 1) // 2


def test_tensor_tier_matches_the_fp32_tier(cuda, monkeypatch):
    c = recipes.he_ladder(pq, 14, 3)
    th = np.random.default_rng(8).random((150, c.n_columns())) * 2 * np.pi
    psi = c.run_batch(th)
    tc, _ = _counts(psi, 75, False)
    monkeypatch.setenv("PQC_NO_TENSOR_GRAM", "1")
    fp32, _ = _counts(psi, 75, False)
    np.testing.assert_array_equal(tc, fp32)


def test_tensor_gram_rejects_unsupported_sizes(cuda):
    small = torch.zeros((4, 2 ** 10), dtype=torch.complex128, device="cuda")
    small[:, 0] = 1
    with pytest.raises(pq._lib.EngineError, match="tensor-core Gram"):
        engine.gram_tf32(small)
