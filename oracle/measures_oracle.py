"""FP64 numpy restatement of the reference's capacity measures.

TEST INFRASTRUCTURE ONLY (see ``oracle/__init__.py``).
"""
from itertools import combinations

import numpy as np
import scipy.special


def pair_fidelities(states):
    """`measure.py:123-137`: |<psi_a|psi_b>|^2 over itertools.combinations(states, 2)."""
    states = np.asarray(states)
    G = np.conj(states) @ states.T
    a, b = np.triu_indices(len(states), 1)  # same (a<b, row-major) order as combinations
    return np.abs(G[a, b]) ** 2


def pair_fidelities_loop(states):
    """Literal pair loop (small S only), used to pin ``pair_fidelities``'s order."""
    return np.array([np.abs(np.vdot(p, q)) ** 2 for p, q in combinations(list(states), 2)])


def reference_nbins(m):
    """`measure.py:153-154`: int((75/10000) * len(F_samples))."""
    return int((75 / 10000) * m)


def gen_histo(F_samples, nbins=None):
    """`measure.py:139-159` (the ``filt`` argument is ignored there: it filters a copy
    but histograms the unfiltered list)."""
    if nbins is None:
        nbins = reference_nbins(len(F_samples))
    prob, edges = np.histogram(F_samples, bins=nbins, range=(0, 1))
    counts = prob.copy()
    prob = prob / sum(prob)
    F = np.array([(edges[i - 1] + edges[i]) / 2 for i in range(1, len(edges))])
    return prob, F, counts, edges


def expr_from_counts(counts, edges, d):
    """`measure.py:171-180`: sum kl_div(P_pqc, P_haar), P_haar ~ (d-1)(1-F)^(d-2)."""
    prob = counts / sum(counts)
    F = np.array([(edges[i - 1] + edges[i]) / 2 for i in range(1, len(edges))])
    haar = (d - 1) * ((1 - F) ** (d - 2))
    P_haar = haar / sum(haar)
    return float(np.sum(scipy.special.kl_div(prob, P_haar)))


def expr(F_samples, d, nbins=None):
    """`measure.py:161-180`."""
    if len(F_samples) == 0:
        return 0
    _, _, counts, edges = gen_histo(F_samples, nbins)
    return expr_from_counts(counts, edges, d)


def single_Q(psi, N):
    """`measure.py:226-237`: Q = 2 (1 - (1/N) sum_k tr rho_k^2)."""
    t = np.asarray(psi).reshape((2,) * N)
    s = 0.0
    for k in range(N):
        m = np.moveaxis(t, k, 0).reshape(2, -1)
        rho = m @ m.conj().T
        s += float(np.real(np.trace(rho @ rho)))
    return 2 * (1 - s / N)


def _conversion_matrices(N):
    """`measure.py:268-313`: (j XOR k) index matrix and (-1)^{popcount(i & j)} sign matrix."""
    idx = np.arange(2 ** N)
    mod_add = idx[:, None] ^ idx[None, :]
    par = np.zeros((2 ** N, 2 ** N), dtype=np.int64)
    x = idx[:, None] & idx[None, :]
    while np.any(x):
        par ^= x & 1
        x = x >> 1
    sign = (-1) ** par
    return mod_add, sign


def renyi_entropy_literal(psi, alpha=2.0):
    """`measure.py:318-349` with its dense O(8^N) product (N <= 8 or so)."""
    c = np.asarray(psi, dtype=np.complex128).reshape(-1)
    N = int(np.log2(len(c)))
    mod_add, sign = _conversion_matrices(N)
    r = np.dot(np.conjugate(c) * sign, c[mod_add])
    s = np.sum(np.abs(2 ** (-N / 2) * r) ** (2 * alpha))
    return float(1 / (1 - alpha) * np.log(s) - np.log(2 ** N))


def fwht(a, axis=-1):
    """Unnormalised Walsh-Hadamard transform along ``axis`` (any dtype)."""
    a = np.moveaxis(np.array(a), axis, -1).copy()
    n = a.shape[-1]
    h = 1
    while h < n:
        a = a.reshape(a.shape[:-1] + (n // (2 * h), 2, h))
        x = a[..., 0, :].copy()
        y = a[..., 1, :].copy()
        a[..., 0, :] = x + y
        a[..., 1, :] = x - y
        a = a.reshape(a.shape[:-3] + (n,))
        h *= 2
    return np.moveaxis(a, -1, axis)


def renyi_entropy_wht(psi, alpha=2.0):
    """Same quantity via r[:, k] = WHT_j(conj(c_j) c_{j XOR k}) -- O(N 4^N)."""
    c = np.asarray(psi, dtype=np.complex128).reshape(-1)
    D = len(c)
    N = int(np.log2(D))
    idx = np.arange(D)
    V = np.conj(c)[:, None] * c[idx[:, None] ^ idx[None, :]]  # V[j, k]
    r = fwht(V, axis=0)
    s = np.sum(np.abs(2 ** (-N / 2) * r) ** (2 * alpha))
    return float(1 / (1 - alpha) * np.log(s) - np.log(2 ** N))


def gkp(psi, renyi=renyi_entropy_wht):
    """`measure.py:361-368`: 1/(2 ln 2) * M_{1/2}."""
    return 1 / (2 * np.log(2)) * renyi(psi, alpha=1 / 2)


def efficient_measurements(states, N, measure_expr=True, measure_ent=True, measure_eom=True,
                           measure_GKP=True, full_data=False, renyi=renyi_entropy_wht):
    """`measure.py:370-459` on already generated states (sentinels -1, np.std)."""
    states = np.asarray(states)
    overlaps, magics, gkps, q_vals = [], [], [], []
    if len(states) == 0:
        measure_expr = measure_ent = measure_eom = measure_GKP = False
    if measure_expr and N < 12:
        overlaps = list(pair_fidelities(states))
        e = expr(overlaps, 2 ** N) if N < 7 else -1
    else:
        e = -1
    if measure_ent:
        q_vals = [single_Q(s, N) for s in states]
        q, qs = np.mean(q_vals), np.std(q_vals)
    else:
        q, qs = -1, -1
    if measure_eom:
        magics = [renyi(s) for s in states]
        m, ms = np.mean(magics), np.std(magics)
    else:
        m, ms = -1, -1
    if measure_GKP:
        gkps = [gkp(s, renyi) for s in states]
        g, gs = np.mean(gkps), np.std(gkps)
    else:
        g, gs = -1, -1
    if full_data:
        return {"Expr": overlaps, "Ent": q_vals, "Magic": magics, "GKP": gkps}
    return {"Expr": e, "Ent": [q, qs], "Magic": [m, ms], "GKP": [g, gs]}
