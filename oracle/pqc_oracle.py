"""FP64 numpy restatement of the reference's statevector semantics.

TEST INFRASTRUCTURE ONLY (see ``oracle/__init__.py``).

Circuit descriptions are duck-typed gate objects read by class name and
attributes, exactly as the reference defines them in
``pyramaterised/gates.py`` (``q_on``; ``q1, q2``; fixed ``theta``;
``offset``; ``layer``/``commute`` of ``shared_parameter``; ``rotator`` of
``RR_block``; ``entangler`` of ``CHAIN``/``ALLTOALL``).  Both the product's
gate descriptors and the reference's own gate objects satisfy this.

Conventions restated from QuTiP 4.7.2 (the reference's arithmetic backend):
qubit 0 is the most significant tensor factor (``qt.tensor`` order), so
basis index ``i`` holds qubit ``q`` in bit ``N-1-q``; ``rx/ry/rz(a) =
exp(-i a sigma/2)``; a two-qubit gate's first tensor factor acts on
``control``/``targets[0]``.
"""
from itertools import permutations

import numpy as np
import scipy.linalg

SQ2 = 1.0 / np.sqrt(2.0)
PAULI = {
    "I": np.eye(2, dtype=np.complex128),
    "X": np.array([[0, 1], [1, 0]], dtype=np.complex128),
    "Y": np.array([[0, -1j], [1j, 0]], dtype=np.complex128),
    "Z": np.array([[1, 0], [0, -1]], dtype=np.complex128),
}


# --------------------------------------------------------------------------
# 2x2 / 4x4 gate matrices (qutip.qip.operations semantics)
# --------------------------------------------------------------------------
def rx(a):
    return np.array([[np.cos(a / 2), -1j * np.sin(a / 2)], [-1j * np.sin(a / 2), np.cos(a / 2)]], dtype=np.complex128)


def ry(a):
    return np.array([[np.cos(a / 2), -np.sin(a / 2)], [np.sin(a / 2), np.cos(a / 2)]], dtype=np.complex128)


def rz(a):
    return np.array([[np.exp(-1j * a / 2), 0], [0, np.exp(1j * a / 2)]], dtype=np.complex128)


def phasegate(t):
    return np.array([[1, 0], [0, np.exp(1.0j * t)]], dtype=np.complex128)


CNOT4 = np.array([[1, 0, 0, 0], [0, 1, 0, 0], [0, 0, 0, 1], [0, 0, 1, 0]], dtype=np.complex128)
CZ4 = np.diag([1, 1, 1, -1]).astype(np.complex128)
SQRTISWAP4 = np.array([[1, 0, 0, 0], [0, SQ2, 1j * SQ2, 0], [0, 1j * SQ2, SQ2, 0], [0, 0, 0, 1]], dtype=np.complex128)


def fsim(theta, phi):
    """`gates.py:588-606`."""
    c, s = np.cos(theta), np.sin(theta)
    return np.array([[1, 0, 0, 0], [0, c, -1j * s, 0], [0, -1j * s, c, 0], [0, 0, 0, np.exp(-1j * phi)]], dtype=np.complex128)


def fsim_d_theta(theta, phi):
    """`gates.py:609-627` (keeps the non-derivative diagonal entries, as the reference does)."""
    c, s = np.cos(theta), np.sin(theta)
    return np.array([[1, 0, 0, 0], [0, -s, -1j * c, 0], [0, -1j * c, -s, 0], [0, 0, 0, np.exp(-1j * phi)]], dtype=np.complex128)


def fsim_d_phi(theta, phi):
    """`gates.py:630-648`."""
    c, s = np.cos(theta), np.sin(theta)
    return np.array([[1, 0, 0, 0], [0, c, -1j * s, 0], [0, -1j * s, c, 0], [0, 0, 0, -1j * np.exp(-1j * phi)]], dtype=np.complex128)


def fixed_fsim(theta):
    """`gates.py:700-716`."""
    c, s = np.cos(theta), np.sin(theta)
    return np.array([[1, 0, 0, 0], [0, c, -1j * s, 0], [0, -1j * s, c, 0], [0, 0, 0, 1]], dtype=np.complex128)


def fixed_fsim_d_theta(theta):
    """`gates.py:719-737`."""
    c, s = np.cos(theta), np.sin(theta)
    return np.array([[1, 0, 0, 0], [0, -s, -1j * c, 0], [0, -1j * c, -s, 0], [0, 0, 0, 1]], dtype=np.complex128)


def hadamard():
    """`gates.py:226-232`: H = X . RY(pi/2) (kept literally: cos/sin(pi/4) differ in the last bit)."""
    return PAULI["X"] @ ry(np.pi / 2)


# --------------------------------------------------------------------------
# state helpers
# --------------------------------------------------------------------------
def basis_state(N, index=0):
    v = np.zeros(2 ** N, dtype=np.complex128)
    v[index] = 1.0
    return v


def product_state(bits):
    """|b_0 b_1 ... b_{N-1}> with qubit 0 most significant (`templates.py:373-377`)."""
    idx = 0
    for b in bits:
        idx = (idx << 1) | int(b)
    return basis_state(len(bits), idx)


def apply_local(psi, U, qubits, N):
    """Apply a 2^k x 2^k matrix on ``qubits`` (first qubit = most significant local bit).

    ``psi`` has shape (..., 2**N); the leading axes are a batch.
    """
    k = len(qubits)
    lead = psi.shape[:-1]
    t = psi.reshape(lead + (2,) * N)
    nl = len(lead)
    Ut = U.reshape((2,) * (2 * k))
    axes = [nl + q for q in qubits]
    out = np.tensordot(t, Ut, axes=(axes, list(range(k, 2 * k))))
    # tensordot puts the k new axes last, in the order of Ut's output axes
    out = np.moveaxis(out, list(range(out.ndim - k, out.ndim)), axes)
    return np.ascontiguousarray(out).reshape(lead + (2 ** N,))


def full_operator(local_ops, N):
    """Dense 2^N x 2^N operator of a list of (U, qubits), applied in list order."""
    M = np.eye(2 ** N, dtype=np.complex128)
    for U, qs in local_ops:
        M = apply_local(M.T, U, qs, N).T
    return M


def _pauli_string_local(pstr):
    """[(2x2, (q,))...] for a {qubit: 'X'|'Y'|'Z'} dict."""
    return [(PAULI[p], (q,)) for q, p in sorted(pstr.items())]


# --------------------------------------------------------------------------
# gate semantics (gates.py), keyed by the reference class names
# --------------------------------------------------------------------------
ROT1 = {"R_x": rx, "R_y": ry, "R_z": rz, "negative_R_z": rz, "offset_R_z": rz}
PAULI_OF = {"R_x": "X", "R_y": "Y", "R_z": "Z", "negative_R_z": "Z", "offset_R_z": "Z"}
RR_PAULI = {"R_zz": "Z", "R_xx": "X", "R_yy": "Y"}
ENT4 = {"CNOT": CNOT4, "CPHASE": CZ4, "CZ": CZ4, "sqrtiSWAP": SQRTISWAP4}


def gname(g):
    return type(g).__name__


def param_count(g):
    return int(getattr(g, "param_count", 0))


def member_angle(g, theta):
    """Angle a member gate stores after ``set_theta(theta)`` (`gates.py:129-131,181-183,203-205`)."""
    n = gname(g)
    if n == "negative_R_z":
        return -theta
    if n == "offset_R_z":
        return theta + g.offset
    return theta


def chain_pairs(N):
    """`gates.py:366-376`: brick order, top pairs then bottom pairs (applied in list order)."""
    top = [(2 * j, 2 * j + 1) for j in range(N // 2)]
    bot = [(2 * j + 1, 2 * j + 2) for j in range((N - 1) // 2)]
    return top + bot


def alltoall_pairs(N):
    """`gates.py:392-398`: every ordered pair, itertools.permutations order."""
    return list(permutations(range(N), 2))


def ring_pairs(N):
    """`gates.py:565-572`: periodic ring (i, (i+1) % N)."""
    return [(i, (i + 1) % N) for i in range(N)]


def gate_local_ops(g, N, params):
    """Forward action of one gate as a list of (matrix, qubits) in application order.

    ``params`` is the tuple of this gate's parameters in `set_params` order
    (`circuit.py:86-116`); empty for fixed gates.
    """
    n = gname(g)
    if n in ROT1:
        return [(ROT1[n](member_angle(g, params[0])), (g.q_on,))]
    if n == "I":
        return []
    if n == "H":
        return [(hadamard(), (g.q_on,))]
    if n == "X":
        return [(PAULI["X"], (g.q_on,))]
    if n == "S":
        return [(phasegate(np.pi / 2), (g.q_on,))]
    if n == "T":
        return [(phasegate(np.pi / 4), (g.q_on,))]
    if n == "fixed_R_y":
        return [(ry(g.theta), (g.q_on,))]
    if n == "fixed_R_z":
        return [(rz(g.theta), (g.q_on,))]
    if n in ENT4:
        return [(ENT4[n], (g.q1, g.q2))]
    if n == "CHAIN":
        M = ENT4[g.entangler.__name__]
        return [(M, p) for p in chain_pairs(N)]
    if n == "ALLTOALL":
        M = ENT4[g.entangler.__name__]
        return [(M, p) for p in alltoall_pairs(N)]
    if n in RR_PAULI:
        return [(rr_matrix(RR_PAULI[n], params[0]), (g.q1, g.q2))]
    if n == "shared_parameter" or n == "RR_block":
        ops = []
        for m in shared_members(g, N):
            ops += gate_local_ops(m, N, (params[0],))
        return ops
    if n == "fSim":
        return [(fsim(params[0], params[1]), (g.q1, g.q2))]
    if n == "fixed_fSim":
        return [(fixed_fsim(params[0]), (g.q1, g.q2))]
    if n == "ARBGATE":
        Hm = _dense(g._Ham)
        return [(scipy.linalg.expm(-1j * params[0] * Hm), tuple(range(N)))]
    raise NotImplementedError(f"oracle: unsupported gate {n}")


def shared_members(g, N):
    """Members of a shared-parameter block in application order (`gates.py:475-477, 565-582`)."""
    if gname(g) == "RR_block":
        rot = g.rotator
        return [_Desc(rot.__name__, q1=a, q2=b) for a, b in ring_pairs(N)]
    return list(g.layer)


class _Desc:
    """A tiny stand-in gate description (used for RR_block ring members)."""

    def __init__(self, name, **kw):
        self.__class__ = type(name, (_Desc,), {})
        self.__dict__.update(kw)
        self.param_count = 1


def rr_matrix(p, a):
    """`gates.py:509-517`: cos(a/2) I - i sin(a/2) P(x)P."""
    PP = np.kron(PAULI[p], PAULI[p])
    return np.cos(a / 2) * np.eye(4, dtype=np.complex128) - 1j * np.sin(a / 2) * PP


def _dense(H):
    if hasattr(H, "full"):
        return H.full()
    return np.asarray(H, dtype=np.complex128)


def assign_params(gates, theta):
    """Per-gate parameter tuples in `set_params` order (`circuit.py:86-116`)."""
    out = []
    k = 0
    for g in gates:
        pc = param_count(g) if getattr(g, "is_param", False) else 0
        out.append(tuple(float(theta[k + j]) for j in range(pc)))
        k += pc
    if k != len(theta):
        raise ValueError(f"expected {k} angles, got {len(theta)}")
    return out


def n_params(gates):
    return sum(param_count(g) for g in gates if getattr(g, "is_param", False))


# --------------------------------------------------------------------------
# PQC.run / cost / fidelity (circuit.py)
# --------------------------------------------------------------------------
def circuit_local_ops(gates, N, theta):
    ops = []
    for g, p in zip(gates, assign_params(gates, theta)):
        ops += gate_local_ops(g, N, p)
    return ops


def run(gates, N, theta, psi0=None):
    """`circuit.py:118-125`: psi = G_last ... G_1 psi0 (first gate in the list applied first)."""
    psi = basis_state(N) if psi0 is None else np.array(psi0, dtype=np.complex128).reshape(-1)
    for U, qs in circuit_local_ops(gates, N, theta):
        psi = apply_local(psi, U, qs, N)
    return psi


def run_batch(gates, N, thetas, psi0=None):
    return np.stack([run(gates, N, t, psi0) for t in np.asarray(thetas, dtype=np.float64)])


def fidelity(psi, phi):
    """`circuit.py:139-142`: |<psi|phi>|^2."""
    return float(np.abs(np.vdot(psi, phi)) ** 2)


# --------------------------------------------------------------------------
# Hamiltonians and energies
# --------------------------------------------------------------------------
def apply_hamiltonian(H, psi, N):
    """H|psi> for a dense matrix or a Pauli sum (object with ``terms``: [(coef, 'IXYZ..'), ...])."""
    if hasattr(H, "terms"):
        out = np.zeros_like(psi)
        for coef, s in H.terms:
            v = psi
            for q, p in enumerate(s):
                if p != "I":
                    v = apply_local(v, PAULI[p], (q,), N)
            out = out + coef * v
        return out
    return psi @ _dense(H).T


def zz_hamiltonian_terms(N):
    """`circuit.py:25-31`: default H = Z_0 Z_1."""
    s = ["I"] * N
    s[0] = s[1] = "Z"
    return [(1.0, "".join(s))]


def expect(H, psi, N):
    """`circuit.py:132-137` via ``qt.expect``: <psi|H|psi> (real for Hermitian H)."""
    return float(np.real(np.vdot(psi, apply_hamiltonian(H, psi, N))))


# --------------------------------------------------------------------------
# derivatives (circuit.py:149-192, gates.py derivative methods)
# --------------------------------------------------------------------------
def derivative_local_ops(g, N, params, which=0):
    """Operator ``deriv`` that `take_derivative` multiplies in after the gate.

    Returns a list of ("sum", [(coef, local_ops), ...]) terms or ("dense", M).
    ``which`` = 0 uses ``derivative()``; 1/2 use ``parameterised_derivative``.
    """
    n = gname(g)
    if which == 2 and n != "fSim":
        which = 0  # Gate.parameterised_derivative -> derivative() (gates.py:96-97)
    if which == 1 and n != "fSim":
        which = 0
    if n in PAULI_OF:
        c = 0.5j if n == "negative_R_z" else -0.5j
        return ("sum", [(c, [(PAULI[PAULI_OF[n]], (g.q_on,))])])
    if n == "I":
        return ("sum", [(-0.5j, [])])
    if n in RR_PAULI:
        p = PAULI[RR_PAULI[n]]
        return ("sum", [(-0.5j, [(p, (g.q1,)), (p, (g.q2,))])])
    if n == "RR_block" or (n == "shared_parameter" and getattr(g, "commute", True)):
        terms = []
        for m in shared_members(g, N):
            kind, t = derivative_local_ops(m, N, (params[0],))
            terms += t
        return ("sum", terms)
    if n == "shared_parameter":
        # gates.py:459-466: sum_k prod(layer with d_k g_k) times elementwise conj(U)
        members = shared_members(g, N)
        U = full_operator(gate_local_ops(g, N, params), N)
        acc = np.zeros_like(U)
        for k, m in enumerate(members):
            ops = []
            for j, mm in enumerate(members):
                ops += gate_local_ops(mm, N, (params[0],))
                if j == k:
                    _, dterms = derivative_local_ops(mm, N, (params[0],))
                    D = np.zeros_like(U)
                    for c, lops in dterms:
                        D = D + c * full_operator(lops, N)
                    ops_mat = full_operator(ops, N)
                    ops = [(D @ ops_mat, tuple(range(N)))]
            acc = acc + full_operator(ops, N)
        return ("dense", acc @ U.conj())
    if n == "fixed_fSim":
        return ("sum", [(1.0, [(fixed_fsim_d_theta(params[0]), (g.q1, g.q2))])])
    if n == "fSim":
        M = fsim_d_phi(params[0], params[1]) if which == 2 else fsim_d_theta(params[0], params[1])
        return ("sum", [(1.0, [(M, (g.q1, g.q2))])])
    if n == "ARBGATE":
        return ("dense", -0.5j * _dense(g._Ham))
    if n in ENT4 or n in ("CHAIN", "ALLTOALL"):
        return ("sum", [(1.0, [])])  # Gate.derivative -> identity (gates.py:93-94)
    raise NotImplementedError(f"oracle: no derivative for {n}")


def _apply_deriv(psi, d, N):
    kind, t = d
    if kind == "dense":
        return psi @ t.T
    out = np.zeros_like(psi)
    for c, lops in t:
        v = psi
        for U, qs in lops:
            v = apply_local(v, U, qs, N)
        out = out + c * v
    return out


def take_derivative(gates, N, theta, gate_index, which=0, psi0=None):
    """`circuit.py:149-172`: run with gate ``gate_index`` replaced by ``deriv * gate``."""
    params = assign_params(gates, theta)
    psi = basis_state(N) if psi0 is None else np.array(psi0, dtype=np.complex128).reshape(-1)
    for i, (g, p) in enumerate(zip(gates, params)):
        for U, qs in gate_local_ops(g, N, p):
            psi = apply_local(psi, U, qs, N)
        if i == gate_index:
            psi = _apply_deriv(psi, derivative_local_ops(g, N, p, which), N)
    return psi


def gradient_tasks(gates):
    """The (gate_index, which) arguments of `take_derivative` for each row of `get_gradients`, in row order.

    `circuit.py:174-192`, including its second-parameter lookup ``self.gates[count]`` (`circuit.py:188`),
    which indexes all gates with the position among parameterised gates."""
    tasks = []
    param_gates = [i for i, g in enumerate(gates) if param_count(g) > 0]
    for count, gi in enumerate(param_gates):
        g = gates[gi]
        if param_count(g) == 1:
            tasks.append((gi, 0))
        elif param_count(g) == 2:
            tasks.append((gi, 1))
            tasks.append((count, 2))
    return tasks


def get_gradients(gates, N, theta, psi0=None):
    """`circuit.py:174-192`: one `take_derivative` run per row of `gradient_tasks`."""
    out = [take_derivative(gates, N, theta, gi, which, psi0) for gi, which in gradient_tasks(gates)]
    return np.array(out).reshape(len(out), 2 ** N)


def get_QFI(state, grads):
    """`measure.py:33-71`: F_pq = 4 Re(<d_p|d_q> - <d_p|psi><psi|d_q>), symmetrised.

    ``state`` is the PQC's current ``state`` attribute (the reference reads
    ``self.QC.state``, not a fresh run).
    """
    grads = np.asarray(grads)
    single = np.array([np.vdot(state, g) for g in grads])  # state.overlap(d_p)
    G = np.conj(grads) @ grads.T  # <d_p|d_q>
    F = 4 * np.real(G - np.conj(single)[:, None] * single[None, :])
    Fs = np.triu(F) + np.triu(F, 1).T
    return Fs


def effective_quantum_dimension(F, cutoff):
    """`measure.py:77-87`."""
    w = scipy.linalg.eigh(F, eigvals_only=True)
    return int(np.sum(w > cutoff))


def new_measure(F):
    """`measure.py:89-99`."""
    w = scipy.linalg.eigh(F, eigvals_only=True)
    return float(sum(1 if v > 1 else v for v in w))


def gradient_vector(gates, N, theta, H, psi0=None):
    """`measure.py:461-471`: dE/dtheta_i = 2 Re <psi|H|d_i psi>."""
    psi = run(gates, N, theta, psi0)
    grads = get_gradients(gates, N, theta, psi0)
    return np.array([2 * np.real(np.vdot(psi, apply_hamiltonian(H, d, N))) for d in grads])


# --------------------------------------------------------------------------
# Hamiltonians used by the configs
# --------------------------------------------------------------------------
class PauliTerms:
    def __init__(self, terms):
        self.terms = list(terms)


def tfim_open(N, h=1.0):
    """H = -sum_i Z_i Z_{i+1} - h sum_i X_i on an open chain."""
    t = []
    for i in range(N - 1):
        s = ["I"] * N
        s[i] = s[i + 1] = "Z"
        t.append((-1.0, "".join(s)))
    for i in range(N):
        s = ["I"] * N
        s[i] = "X"
        t.append((-h, "".join(s)))
    return PauliTerms(t)


def tfim_reference(N, g, h=0.0):
    """`templates.py:220-227`: -sum_i (Z_i Z_{i+1 mod N} + g X_i + h Z_i)."""
    t = []
    for i in range(N):
        ip = (i + 1) % N
        s = ["I"] * N
        s[i] = "Z"
        s[ip] = "Z" if ip != i else "I"
        t.append((-1.0, "".join(s)))
        s = ["I"] * N
        s[i] = "X"
        t.append((-g, "".join(s)))
        if h:
            s = ["I"] * N
            s[i] = "Z"
            t.append((-h, "".join(s)))
    return PauliTerms(t)


def xxz_open(N, delta=0.5):
    """H = sum_i (X_i X_{i+1} + Y_i Y_{i+1} + delta Z_i Z_{i+1}) on an open chain."""
    t = []
    for i in range(N - 1):
        for p, c in (("X", 1.0), ("Y", 1.0), ("Z", delta)):
            s = ["I"] * N
            s[i] = s[i + 1] = p
            t.append((c, "".join(s)))
    return PauliTerms(t)
