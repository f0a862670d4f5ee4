"""A numpy interpreter of `pqc_op` records (test utility).

Independent of the CUDA kernels and of the oracle's gate semantics: it reads
the op table the lowering pass produced, so comparing it with the oracle
checks the lowering, and replaying it in the planner's order checks that the
sweep reordering preserves the result.
"""
import numpy as np

from oracle.pqc_oracle import apply_local

X = np.array([[0, 1], [1, 0]], dtype=np.complex128)
Y = np.array([[0, -1j], [1j, 0]], dtype=np.complex128)
Z = np.diag([1, -1]).astype(np.complex128)
I2 = np.eye(2, dtype=np.complex128)
LET = {0: I2, 1: X, 2: Y, 3: Z}


def op_matrix(op, theta):
    k = int(op["kind"])

    def ang(p, s, o):
        return s * theta[p] + o if p >= 0 else o

    a = ang(int(op["param"]), float(op["scale"]), float(op["offset"]))
    a2 = ang(int(op["param2"]), float(op["scale2"]), float(op["offset2"]))
    m = op["m"][0::2] + 1j * op["m"][1::2]
    c, s = np.cos(a / 2), np.sin(a / 2)
    if k == 1:
        return np.array([[c, -1j * s], [-1j * s, c]]), 1
    if k == 2:
        return np.array([[c, -s], [s, c]], dtype=np.complex128), 1
    if k == 3:
        return np.diag([np.exp(-1j * a / 2), np.exp(1j * a / 2)]), 1
    if k == 4:
        return m[:4].reshape(2, 2), 1
    if k == 5:
        return np.array([[1, 0, 0, 0], [0, 1, 0, 0], [0, 0, 0, 1], [0, 0, 1, 0]], dtype=np.complex128), 2
    if k == 6:
        return np.diag([1, 1, 1, -1]).astype(np.complex128), 2
    if k in (7, 8, 9):
        P = {7: X, 8: Y, 9: Z}[k]
        return c * np.eye(4) - 1j * s * np.kron(P, P), 2
    if k == 10:
        return m[:16].reshape(4, 4), 2
    if k in (11, 12, 14, 15, 16):
        ct, st = np.cos(a), np.sin(a)
        p11 = np.exp(-1j * a2)
        if k == 11:
            blk, d = (ct, st), p11
        elif k == 12:
            blk, d = (ct, st), 1.0
        elif k == 14:
            blk, d = (-st, ct), p11
        elif k == 15:
            blk, d = (ct, st), -1j * p11
        else:
            blk, d = (-st, ct), 1.0
        cc, ss = blk
        return np.array([[1, 0, 0, 0], [0, cc, -1j * ss, 0], [0, -1j * ss, cc, 0], [0, 0, 0, d]]), 2
    if k == 13:
        coef = m[0]
        l0, l1 = int(op["pauli"]) & 0xFF, (int(op["pauli"]) >> 8) & 0xFF
        if int(op["q1"]) >= 0:
            return coef * np.kron(LET[l0], LET[l1]), 2
        return coef * LET[l0], 1
    raise ValueError(k)


def apply_op(psi, op, theta, N):
    M, nq = op_matrix(op, theta)
    qs = (int(op["q0"]),) if nq == 1 else (int(op["q0"]), int(op["q1"]))
    return apply_local(psi, M, qs, N)


def run_ops(ops, theta, N, psi0, order=None):
    psi = np.array(psi0, dtype=np.complex128)
    idx = range(len(ops)) if order is None else order
    for i in idx:
        psi = apply_op(psi, ops[i], theta, N)
    return psi
