"""Adjoint energy gradients through pqc_energy_grad against the FP64 oracle.

Pauli-term generators take the fused double-float reverse sweeps; any other
generator kind takes the FP64 one-kernel-per-op path, so the two paths are
also checked against each other.  Tolerance: 1e-10 absolute on energies and
gradient entries (unit-norm states, |H| of order N).
"""
import numpy as np
import pytest
import torch

import recipes
from oracle import pqc_oracle as O
import pyramaterised_gb300 as pq
from pyramaterised_gb300 import _lib
from pyramaterised_gb300.engine import _p, _stream, _ws, check

pytestmark = pytest.mark.gpu
TOL = 1e-10

PAULI = {1: np.array([[0, 1], [1, 0]], complex), 2: np.array([[0, -1j], [1j, 0]]), 3: np.diag([1.0, -1.0]) + 0j}


def _np(t):
    return t.detach().cpu().numpy()


def pauli_mix(N, L):
    """Every Pauli-generated gate class (no fSim), L layers (N >= 4)."""
    c = pq.PQC(N)
    for _ in range(L):
        layer = [pq.H(0, N), pq.R_x(1, N), pq.R_y(2 % N, N), pq.R_z(0, N), pq.negative_R_z(1, N),
                 pq.offset_R_z(2 % N, N, 0.7), pq.fixed_R_y(0, N, 0.3), pq.S(1, N), pq.T(2 % N, N)]
        layer += [pq.R_y(i, N) for i in range(N)] + [pq.R_x(i, N) for i in range(0, N, 2)]
        layer += [pq.CNOT([i, (i + 1) % N], N) for i in range(N - 1)]
        layer += [pq.R_xx([0, N - 1], N), pq.R_yy([1, N - 2], N), pq.R_zz([2, N - 1], N), pq.CZ([0, N // 2], N),
                  pq.CPHASE([N - 1, 1], N), pq.sqrtiSWAP([N // 2, 0], N)]
        layer += [pq.shared_parameter([pq.R_z(i, N) for i in range(N)], N), pq.RR_block(pq.R_zz, N)]
        c.add_layer(layer)
    return c


def _egrad_abi(c, th, H, gens, after, n_cols, row_limit=None):
    prog = c.program
    lib = prog.lib
    th = torch.as_tensor(np.atleast_2d(th), dtype=torch.float64).cuda().contiguous()
    B = th.shape[0]
    terms = torch.from_numpy(H.device_terms().view(np.uint8)).cuda()
    E = torch.empty(B, dtype=torch.float64, device="cuda")
    grad = torch.full((B, n_cols), float("nan"), dtype=torch.float64, device="cuda")
    lim = None if row_limit is None else torch.as_tensor(row_limit, dtype=torch.int32).cuda()
    ws = _ws(lib.pqc_energy_grad_workspace_size(prog.handle, B, len(gens), n_cols), th.device)
    gens = np.ascontiguousarray(gens)
    after = np.ascontiguousarray(after, dtype=np.int32)
    check(lib.pqc_energy_grad(prog.handle, _p(th), th.shape[1], B, None, 0, _p(terms), len(H.terms),
                              gens.ctypes.data, after.ctypes.data, len(gens), n_cols, _p(E), _p(grad),
                              _p(lim) if lim is not None else None, _p(ws), ws.numel(), _stream()))
    return _np(E), _np(grad)


def _as_matrix_gen(g):
    """A single-qubit Pauli-term generator rewritten as a PQC_OP_MAT1 op (the same operator)."""
    letter = int(g["pauli"]) & 0xFF
    coef = complex(g["m"][0], g["m"][1])
    M = coef * PAULI[letter]
    out = np.zeros(1, dtype=_lib.OP_DTYPE)[0]
    out["kind"] = _lib.PQC_OP_MAT1
    out["q0"], out["q1"], out["param"], out["param2"] = g["q0"], -1, -1, -1
    out["sel"] = g["sel"]
    out["scale"], out["scale2"] = 1.0, 1.0
    m = np.zeros(32)
    m[0:8:2] = M.reshape(-1).real
    m[1:8:2] = M.reshape(-1).imag
    out["m"] = m
    return out


@pytest.mark.parametrize("N,L", [(4, 2), (6, 2), (9, 1), (13, 1), (15, 1)])
def test_fused_adjoint_matches_oracle(cuda, N, L):
    c = pauli_mix(N, L)
    for H, Hr in [(pq.hamiltonian.xxz_open(N, 0.5), O.xxz_open(N, 0.5)),
                  (pq.templates.TFIM_hamiltonian(N, 1.0, 0.3), O.tfim_reference(N, 1.0, 0.3))]:
        c.set_H(H)
        th = np.random.default_rng(N + L).random((2, c.n_columns())) * 2 * np.pi
        E, g = c.program.energy_grad(th, H)
        for b in range(2):
            psi = O.run(c.gates, N, th[b])
            np.testing.assert_allclose(float(E[b]), np.real(np.vdot(psi, O.apply_hamiltonian(Hr, psi, N))), atol=TOL)
            np.testing.assert_allclose(_np(g[b]), O.gradient_vector(c.gates, N, th[b], Hr), atol=TOL)


@pytest.mark.parametrize("N", [12, 14])
def test_adjoint_at_special_angles(cuda, N):
    # the reverse sweeps use the scaled rotation form; angles with cos(t/2) = 0 or tiny take the general form
    # past the growth bound, and measures divide out the pending factor
    c = recipes.he_ladder(pq, N, 3)
    H = pq.hamiltonian.tfim_open(N, 0.7)
    Hr = O.tfim_open(N, 0.7)
    P = c.n_columns()
    rng = np.random.default_rng(N)
    special = np.array([0.0, np.pi, -np.pi, 3 * np.pi, np.pi / 2, np.pi - 1e-9, np.pi + 1e-6])
    th = np.stack([rng.choice(special, P), np.full(P, np.pi), np.pi - 10.0 ** -rng.integers(1, 12, P),
                   np.where(rng.random(P) < 0.5, np.pi, rng.random(P) * 2 * np.pi)])
    E, g = c.program.energy_grad(th, H)
    for b in range(len(th)):
        psi = O.run(c.gates, N, th[b])
        np.testing.assert_allclose(float(E[b]), np.real(np.vdot(psi, O.apply_hamiltonian(Hr, psi, N))), atol=TOL)
        np.testing.assert_allclose(_np(g[b]), O.gradient_vector(c.gates, N, th[b], Hr), atol=TOL)


def test_fused_adjoint_agrees_with_fp64_op_path(cuda):
    N = 14
    c = recipes.he_ladder(pq, N, 3)
    H = pq.hamiltonian.tfim_open(N, 0.7)
    gens, after, n_cols = c.program.lowered.energy_gradient_runs()
    th = np.random.default_rng(5).random((3, c.n_columns())) * 2 * np.pi
    E1, g1 = _egrad_abi(c, th, H, gens, after, n_cols)
    mixed = gens.copy()
    single = [i for i in range(len(gens)) if int(gens[i]["kind"]) == _lib.PQC_OP_PAULI and int(gens[i]["q1"]) < 0]
    mixed[single[0]] = _as_matrix_gen(gens[single[0]])
    E2, g2 = _egrad_abi(c, th, H, mixed, after, n_cols)
    np.testing.assert_allclose(E1, E2, atol=TOL)
    np.testing.assert_allclose(g1, g2, atol=TOL)


def test_row_limits_give_the_prefix_circuit(cuda):
    N = 13
    c = pauli_mix(N, 2)
    H = pq.hamiltonian.xxz_open(N, 0.5)
    low = c.program.lowered
    P = c.n_columns()
    cut = [len(c.gates) // 3, len(c.gates) // 2, len(c.gates)]
    limits = [low.gate_last[g - 1] + 1 for g in cut]
    th = np.random.default_rng(2).random((3, P)) * 2 * np.pi
    E, g = c.program.energy_grad(th, H, row_limit=limits)
    for b, ng in enumerate(cut):
        gates = c.gates[:ng]
        Pb = sum(int(x.param_count) if x.is_param else 0 for x in gates)
        psi = O.run(gates, N, th[b, :Pb])
        Hr = O.xxz_open(N, 0.5)
        np.testing.assert_allclose(float(E[b]), np.real(np.vdot(psi, O.apply_hamiltonian(Hr, psi, N))), atol=TOL)
        np.testing.assert_allclose(_np(g[b, :Pb]), O.gradient_vector(gates, N, th[b, :Pb], Hr), atol=TOL)
        assert np.all(_np(g[b, Pb:]) == 0)


def test_energy_only_and_repeat_calls_reuse_the_plan(cuda):
    N = 12
    c = recipes.he_ladder(pq, N, 2)
    H = pq.hamiltonian.tfim_open(N, 1.0)
    th = np.random.default_rng(9).random((2, c.n_columns())) * 2 * np.pi
    E0, _ = c.program.energy_grad(th, H, want_grad=False)
    E1, g1 = c.program.energy_grad(th, H)
    E2, g2 = c.program.energy_grad(th, H)
    np.testing.assert_array_equal(_np(E1), _np(E2))
    np.testing.assert_array_equal(_np(g1), _np(g2))
    np.testing.assert_allclose(_np(E0), _np(E1), atol=TOL)


def test_autograd_function_uses_the_adjoint(cuda):
    from pyramaterised_gb300 import autograd
    N = 10
    c = recipes.he_ladder(pq, N, 2)
    c.set_H(pq.hamiltonian.xxz_open(N, 0.5))
    th = torch.tensor(np.random.default_rng(4).random(c.n_columns()) * 2 * np.pi, dtype=torch.float64,
                      device="cuda", requires_grad=True)
    E = autograd.energy(c, th)
    E.sum().backward()
    ref = O.gradient_vector(c.gates, N, th.detach().cpu().numpy(), O.xxz_open(N, 0.5))
    np.testing.assert_allclose(_np(th.grad).reshape(-1), ref, atol=TOL)
