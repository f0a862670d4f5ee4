"""Pauli-sum Hamiltonians.

The reference passes Hamiltonians as dense/sparse QuTiP operators
(`circuit.py:25-33` `set_H`, `templates.py:220-227` `TFIM_hamiltonian`).  The
engine evaluates <psi|H|psi> matrix-free from a list of real-coefficient Pauli
strings; `PauliSum.from_matrix` converts a small dense operator.
"""
from itertools import product

import numpy as np
import torch

from . import _lib

_P = {
    "I": np.eye(2, dtype=np.complex128),
    "X": np.array([[0, 1], [1, 0]], dtype=np.complex128),
    "Y": np.array([[0, -1j], [1j, 0]], dtype=np.complex128),
    "Z": np.array([[1, 0], [0, -1]], dtype=np.complex128),
}


class PauliSum:
    """H = sum_t coef_t P_t, P_t a string over 'IXYZ' (character q acts on qubit q)."""

    def __init__(self, terms, n_qubits=None):
        terms = [(float(c), str(s)) for c, s in terms]
        if n_qubits is None:
            n_qubits = len(terms[0][1]) if terms else 0
        for c, s in terms:
            if len(s) != n_qubits or any(ch not in "IXYZ" for ch in s):
                raise ValueError(f"bad Pauli string {s!r} for {n_qubits} qubits")
        self.terms = terms
        self.n_qubits = n_qubits

    # ---------------------------------------------------------------- algebra
    def __add__(self, other):
        if not isinstance(other, PauliSum):
            return NotImplemented
        return PauliSum(self.terms + other.terms, self.n_qubits)

    def __mul__(self, c):
        return PauliSum([(c * a, s) for a, s in self.terms], self.n_qubits)

    __rmul__ = __mul__

    def __neg__(self):
        return self * -1.0

    # ---------------------------------------------------------------- device form
    def device_tensor(self, dev):
        """The `pqc_pauli_term` records as a uint8 tensor on `dev` (uploaded once per device and cached; the
        terms of a PauliSum are not changed after construction)."""
        cache = self.__dict__.setdefault("_dev_terms", {})
        t = cache.get(str(dev))
        if t is None:
            t = torch.from_numpy(self.device_terms().view(np.uint8)).to(dev)
            cache[str(dev)] = t
        return t

    def device_terms(self):
        """numpy array of `pqc_pauli_term` records."""
        N = self.n_qubits
        out = np.zeros(len(self.terms), dtype=_lib.TERM_DTYPE)
        for i, (c, s) in enumerate(self.terms):
            xm = zm = 0
            ny = 0
            for q, ch in enumerate(s):
                bit = 1 << (N - 1 - q)
                if ch in "XY":
                    xm |= bit
                if ch in "ZY":
                    zm |= bit
                ny += ch == "Y"
            out[i] = (xm, zm, c, ny, 0)
        return out

    # ---------------------------------------------------------------- small-N helpers
    def full(self):
        """Dense matrix (host, small N only)."""
        N = self.n_qubits
        if N > 14:
            raise ValueError("dense form limited to 14 qubits")
        M = np.zeros((2 ** N, 2 ** N), dtype=np.complex128)
        for c, s in self.terms:
            op = np.array([[1.0 + 0j]])
            for ch in s:
                op = np.kron(op, _P[ch])
            M += c * op
        return M

    def eigenenergies(self):
        return np.linalg.eigvalsh(self.full())

    def groundstate(self):
        w, v = np.linalg.eigh(self.full())
        return w[0], v[:, 0]

    @staticmethod
    def from_matrix(M, tol=1e-14):
        """Pauli decomposition c_P = tr(P M) / 2^N of a Hermitian matrix (N <= 8)."""
        M = np.asarray(M, dtype=np.complex128)
        D = M.shape[0]
        N = int(round(np.log2(D)))
        if 2 ** N != D or M.shape != (D, D):
            raise ValueError("matrix must be 2^N x 2^N")
        if N > 8:
            raise ValueError("dense Hamiltonians are accepted up to 8 qubits; pass a PauliSum")
        if not np.allclose(M, M.conj().T, atol=1e-12):
            raise ValueError("Hamiltonian must be Hermitian")
        terms = []
        for letters in product("IXYZ", repeat=N):
            op = np.array([[1.0 + 0j]])
            for ch in letters:
                op = np.kron(op, _P[ch])
            c = np.trace(op @ M) / D
            if abs(c) > tol:
                terms.append((float(np.real(c)), "".join(letters)))
        return PauliSum(terms, N)

    def __repr__(self):
        return f"PauliSum({len(self.terms)} terms on {self.n_qubits} qubits)"


def zz(N, a=0, b=1):
    """Z_a Z_b (the reference's default 'ZZ' Hamiltonian, circuit.py:28-31)."""
    s = ["I"] * N
    s[a] = "Z"
    s[b] = "Z"
    return PauliSum([(1.0, "".join(s))], N)


def _one(N, q, ch):
    s = ["I"] * N
    s[q] = ch
    return s


def tfim_periodic(N, g, h=0.0):
    """-sum_i (Z_i Z_{i+1 mod N} + g X_i + h Z_i) (templates.py:220-227)."""
    terms = []
    for i in range(N):
        ip = (i + 1) % N
        s = _one(N, i, "Z")
        if ip != i:
            s[ip] = "Z"
        else:
            s[i] = "I"
        terms.append((-1.0, "".join(s)))
        terms.append((-float(g), "".join(_one(N, i, "X"))))
        if h:
            terms.append((-float(h), "".join(_one(N, i, "Z"))))
    return PauliSum(terms, N)


def tfim_open(N, h=1.0):
    """-sum_i Z_i Z_{i+1} - h sum_i X_i on an open chain."""
    terms = []
    for i in range(N - 1):
        s = _one(N, i, "Z")
        s[i + 1] = "Z"
        terms.append((-1.0, "".join(s)))
    for i in range(N):
        terms.append((-float(h), "".join(_one(N, i, "X"))))
    return PauliSum(terms, N)


def xxz_open(N, delta=0.5):
    """sum_i (X_i X_{i+1} + Y_i Y_{i+1} + delta Z_i Z_{i+1}) on an open chain."""
    terms = []
    for i in range(N - 1):
        for ch, c in (("X", 1.0), ("Y", 1.0), ("Z", float(delta))):
            s = _one(N, i, ch)
            s[i + 1] = ch
            terms.append((c, "".join(s)))
    return PauliSum(terms, N)
