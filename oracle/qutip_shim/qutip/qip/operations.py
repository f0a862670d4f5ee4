"""Gate constructors of qutip.qip.operations (QuTiP 4.7.2 semantics).

Each ``gate(..., N=None, ...)`` returns the 2x2 / 4x4 matrix when ``N`` is
None, otherwise the gate expanded to N qubits (qubit 0 is the most
significant tensor factor).  Two-qubit gates put their first tensor factor
on ``control`` (or ``targets[0]``) and their second on ``target``
(``targets[1]``).
"""
import numpy as np
import scipy.sparse as sp

from .. import Qobj, tensor, qeye, sigmax, sigmay, sigmaz


def gate_expand_1toN(U, N, target):
    if target >= N:
        raise ValueError("target must be integer < integer N")
    return tensor([qeye(2)] * target + [U] + [qeye(2)] * (N - target - 1))


def gate_expand_2toN(U, N, control=None, target=None, targets=None):
    if targets is not None:
        control, target = targets
    if control is None or target is None:
        raise ValueError("Specify value of control and target")
    if control >= N or target >= N or control == target:
        raise ValueError("control and target must be distinct integers < N")
    u = U.data.toarray()
    D = 2 ** N
    idx = np.arange(D, dtype=np.int64)
    pa = N - 1 - control
    pb = N - 1 - target
    ba = (idx >> pa) & 1
    bb = (idx >> pb) & 1
    base = idx & ~((1 << pa) | (1 << pb))
    rows, cols, vals = [], [], []
    col_local = 2 * ba + bb
    for r in range(4):
        ra, rb = r >> 1, r & 1
        row = base | (ra << pa) | (rb << pb)
        v = u[r, col_local]
        nz = v != 0
        rows.append(row[nz])
        cols.append(idx[nz])
        vals.append(v[nz])
    m = sp.csr_matrix((np.concatenate(vals), (np.concatenate(rows), np.concatenate(cols))), shape=(D, D), dtype=np.complex128)
    return Qobj(m, dims=[[2] * N, [2] * N])


def rx(phi, N=None, target=0):
    if N is not None:
        return gate_expand_1toN(rx(phi), N, target)
    return Qobj([[np.cos(phi / 2), -1j * np.sin(phi / 2)], [-1j * np.sin(phi / 2), np.cos(phi / 2)]])


def ry(phi, N=None, target=0):
    if N is not None:
        return gate_expand_1toN(ry(phi), N, target)
    return Qobj([[np.cos(phi / 2), -np.sin(phi / 2)], [np.sin(phi / 2), np.cos(phi / 2)]])


def rz(phi, N=None, target=0):
    if N is not None:
        return gate_expand_1toN(rz(phi), N, target)
    return Qobj([[np.exp(-1j * phi / 2), 0], [0, np.exp(1j * phi / 2)]])


def x_gate(N=None, target=0):
    if N is not None:
        return gate_expand_1toN(x_gate(), N, target)
    return sigmax()


def y_gate(N=None, target=0):
    if N is not None:
        return gate_expand_1toN(y_gate(), N, target)
    return sigmay()


def z_gate(N=None, target=0):
    if N is not None:
        return gate_expand_1toN(z_gate(), N, target)
    return sigmaz()


def phasegate(theta, N=None, target=0):
    if N is not None:
        return gate_expand_1toN(phasegate(theta), N, target)
    return Qobj([[1, 0], [0, np.exp(1.0j * theta)]], dims=[[2], [2]])


def t_gate(N=None, target=0):
    if N is not None:
        return gate_expand_1toN(t_gate(), N, target)
    return Qobj([[1, 0], [0, np.exp(1j * np.pi / 4)]])


def cnot(N=None, control=0, target=1):
    if (control == 1 and target == 0) and N is None:
        N = 2
    if N is not None:
        return gate_expand_2toN(cnot(), N, control, target)
    return Qobj([[1, 0, 0, 0], [0, 1, 0, 0], [0, 0, 0, 1], [0, 0, 1, 0]], dims=[[2, 2], [2, 2]])


def csign(N=None, control=0, target=1):
    if (control == 1 and target == 0) and N is None:
        N = 2
    if N is not None:
        return gate_expand_2toN(csign(), N, control, target)
    return Qobj([[1, 0, 0, 0], [0, 1, 0, 0], [0, 0, 1, 0], [0, 0, 0, -1]], dims=[[2, 2], [2, 2]])


cz_gate = csign


def sqrtiswap(N=None, targets=[0, 1]):
    if N is not None:
        return gate_expand_2toN(sqrtiswap(), N, targets=targets)
    s = 1 / np.sqrt(2)
    return Qobj(np.array([[1, 0, 0, 0], [0, s, 1j * s, 0], [0, 1j * s, s, 0], [0, 0, 0, 1]]), dims=[[2, 2], [2, 2]])
