"""Minimal restatement of the QuTiP 4.7.2 API subset that pyramaterised calls.

TEST INFRASTRUCTURE ONLY.  This package is never imported by the product
(`pyramaterised_gb300`).  It exists so that the reference's own Python
(`pyramaterised/gates.py`, `circuit.py`, `measure.py`) can be executed in a
container where QuTiP 4.7.2 (`requirements.txt:15` of the reference) is not
installed, to generate golden vectors (`tests/golden/make_golden.py`).

What is restated, from QuTiP 4.7.2's documented semantics (not its source):

* ``Qobj``: a CSR matrix (``scipy.sparse.csr_matrix``, complex128) with
  ``dims``; ``*`` is the matrix product (or scaling by a number), ``+``
  adds (a number ``c`` adds ``c*I`` to an operator; ``0`` is a no-op),
  ``overlap`` is <self|other>, ``ptrace(k)`` keeps subsystem(s) ``k``,
  ``tr`` returns a real number for Hermitian operators, ``==`` compares to
  ``atol = 1e-12``, ``Qobj[i]`` returns the dense row ``i``.
* ``tensor`` is the Kronecker product with subsystem 0 most significant.
* ``qip.operations``: ``rx/ry/rz`` are ``exp(-i phi sigma/2)``;
  ``phasegate(t) = diag(1, e^{it})``; ``t_gate = phasegate(pi/4)``;
  ``cnot``, ``cz_gate``, ``sqrtiswap``; ``gate_expand_1toN`` /
  ``gate_expand_2toN`` place a 1-/2-qubit gate with its first tensor factor
  on ``control`` and its second on ``target``.
* ``expect(H, ket)`` is <ket|H|ket>, real when H is Hermitian.
* ``states.bell_state('11') = (|01> - |10>)/sqrt(2)``.
"""
import numbers

import numpy as np
import scipy.linalg
import scipy.sparse as sp

from . import settings  # noqa: F401


def _csr(a):
    if sp.issparse(a):
        return sp.csr_matrix(a, dtype=np.complex128)
    a = np.asarray(a, dtype=np.complex128)
    if a.ndim == 1:
        a = a.reshape(-1, 1)
    return sp.csr_matrix(a)


def _is_number(x):
    return isinstance(x, (numbers.Number, np.number))


class Qobj:
    __array_priority__ = 100
    __array_ufunc__ = None

    def __init__(self, inpt=None, dims=None):
        if isinstance(inpt, Qobj):
            self.data = inpt.data.copy()
            self.dims = [list(inpt.dims[0]), list(inpt.dims[1])] if dims is None else dims
            return
        if inpt is None:
            inpt = [[0]]
        self.data = _csr(inpt)
        if dims is None:
            r, c = self.data.shape
            dims = [[r], [c]]
        self.dims = [list(dims[0]), list(dims[1])]

    # ------------------------------------------------------------------ types
    @property
    def shape(self):
        return self.data.shape

    @property
    def isket(self):
        return self.data.shape[1] == 1 and all(d == 1 for d in self.dims[1])

    @property
    def isbra(self):
        return self.data.shape[0] == 1 and all(d == 1 for d in self.dims[0])

    @property
    def isoper(self):
        return not (self.isket or self.isbra)

    @property
    def type(self):
        return "ket" if self.isket else ("bra" if self.isbra else "oper")

    @property
    def isherm(self):
        if self.data.shape[0] != self.data.shape[1]:
            return False
        d = (self.data - self.data.getH()).tocsr()
        return not (d.nnz and np.any(np.abs(d.data) > settings.atol))

    # ------------------------------------------------------------ arithmetic
    def _new(self, data, dims):
        q = Qobj.__new__(Qobj)
        q.data = sp.csr_matrix(data, dtype=np.complex128)
        q.dims = [list(dims[0]), list(dims[1])]
        return q

    def __mul__(self, other):
        if isinstance(other, Qobj):
            if self.dims[1] != other.dims[0]:
                raise TypeError("Incompatible Qobj shapes")
            return self._new(self.data @ other.data, [self.dims[0], other.dims[1]])
        if _is_number(other):
            return self._new(self.data * other, self.dims)
        return NotImplemented

    def __rmul__(self, other):
        if _is_number(other):
            return self._new(self.data * other, self.dims)
        return NotImplemented

    def __truediv__(self, other):
        if _is_number(other):
            return self._new(self.data / other, self.dims)
        return NotImplemented

    def __neg__(self):
        return self._new(-self.data, self.dims)

    def __add__(self, other):
        if isinstance(other, Qobj):
            if self.dims != other.dims:
                raise TypeError("Incompatible quantum object dimensions")
            return self._new(self.data + other.data, self.dims)
        if _is_number(other):
            if other == 0:
                return Qobj(self)
            if self.data.shape[0] != self.data.shape[1]:
                raise TypeError("Can only add a number to a square operator")
            eye = sp.identity(self.data.shape[0], dtype=np.complex128, format="csr")
            return self._new(self.data + other * eye, self.dims)
        return NotImplemented

    __radd__ = __add__

    def __sub__(self, other):
        if isinstance(other, Qobj) or _is_number(other):
            return self.__add__(-other)
        return NotImplemented

    def __rsub__(self, other):
        return (-self).__add__(other)

    def __eq__(self, other):
        if not isinstance(other, Qobj) or self.dims != other.dims:
            return False
        d = (self.data - other.data).tocsr()
        return not (d.nnz and np.any(np.abs(d.data) > settings.atol))

    __hash__ = None

    def __getitem__(self, ind):
        out = self.data[ind]
        if sp.issparse(out):
            return np.asarray(out.todense())
        return out

    # ---------------------------------------------------------------- methods
    def copy(self):
        return Qobj(self)

    def full(self):
        return self.data.toarray()

    def dag(self):
        return self._new(self.data.getH(), [self.dims[1], self.dims[0]])

    def conj(self):
        return self._new(self.data.conj(), self.dims)

    def tr(self):
        t = complex(self.data.diagonal().sum())
        return t.real if self.isherm else t

    def overlap(self, other):
        a = self.data.toarray()
        b = other.data.toarray()
        if self.isket:
            a = a.conj().T
        if other.isbra:
            b = b.conj().T
        return complex((a @ b)[0, 0])

    def norm(self):
        return float(np.linalg.norm(self.data.toarray()))

    def expm(self):
        return self._new(scipy.linalg.expm(self.data.toarray()), self.dims)

    def ptrace(self, sel):
        if isinstance(sel, numbers.Integral):
            sel = [int(sel)]
        sel = sorted(sel)
        dims = self.dims[0]
        n = len(dims)
        if self.isket:
            psi = self.data.toarray().reshape(dims)
            rest = [i for i in range(n) if i not in sel]
            psi = np.transpose(psi, sel + rest).reshape(int(np.prod([dims[i] for i in sel])), -1)
            rho = psi @ psi.conj().T
        else:
            rho_full = self.data.toarray().reshape(dims + dims)
            rest = [i for i in range(n) if i not in sel]
            for count, i in enumerate(sorted(rest, reverse=True)):
                rho_full = np.trace(rho_full, axis1=i, axis2=i + rho_full.ndim // 2)
            k = int(np.prod([dims[i] for i in sel]))
            rho = rho_full.reshape(k, k)
        kd = [dims[i] for i in sel]
        return Qobj(rho, dims=[kd, kd])

    def permute(self, order):
        dims0 = self.dims[0]
        n = len(dims0)
        if self.isket:
            psi = self.data.toarray().reshape(dims0)
            psi = np.transpose(psi, order).reshape(-1, 1)
            return Qobj(psi, dims=[[dims0[i] for i in order], self.dims[1]])
        m = self.data.toarray().reshape(dims0 + self.dims[1])
        m = np.transpose(m, list(order) + [n + i for i in order])
        d = int(np.prod(dims0))
        return Qobj(m.reshape(d, d), dims=[[dims0[i] for i in order], [self.dims[1][i] for i in order]])

    def eigenenergies(self):
        return scipy.linalg.eigh(self.data.toarray(), eigvals_only=True)

    def eigenstates(self):
        w, v = scipy.linalg.eigh(self.data.toarray())
        kd = [self.dims[0], [1] * len(self.dims[0])]
        return w, [Qobj(v[:, i], dims=kd) for i in range(len(w))]

    def groundstate(self):
        w, vs = self.eigenstates()
        return w[0], vs[0]

    def __repr__(self):
        return f"Quantum object: dims = {self.dims}, shape = {self.shape}, type = {self.type}\n{self.data.toarray()}"


def tensor(*args):
    if len(args) == 1 and isinstance(args[0], (list, tuple)):
        args = args[0]
    out = args[0]
    data = out.data
    d0 = list(out.dims[0])
    d1 = list(out.dims[1])
    for q in args[1:]:
        data = sp.kron(data, q.data, format="csr")
        d0 += q.dims[0]
        d1 += q.dims[1]
    res = Qobj.__new__(Qobj)
    res.data = sp.csr_matrix(data, dtype=np.complex128)
    res.dims = [d0, d1]
    return res


def basis(N, n=0):
    v = np.zeros((N, 1), dtype=np.complex128)
    v[n, 0] = 1.0
    return Qobj(v, dims=[[N], [1]])


def qeye(N):
    if isinstance(N, (list, tuple)):
        return tensor([qeye(n) for n in N])
    return Qobj(sp.identity(N, dtype=np.complex128, format="csr"), dims=[[N], [N]])


identity = qeye


def sigmax():
    return Qobj([[0, 1], [1, 0]])


def sigmay():
    return Qobj([[0, -1j], [1j, 0]])


def sigmaz():
    return Qobj([[1, 0], [0, -1]])


def expect(oper, state):
    if isinstance(state, (list, tuple)):
        return np.array([expect(oper, s) for s in state])
    if state.isket:
        v = state.data.toarray()
        val = complex((v.conj().T @ (oper.data @ v))[0, 0])
    else:
        val = complex((oper.data @ state.data).diagonal().sum())
    return float(val.real) if oper.isherm else val


def ket2dm(psi):
    return psi * psi.dag()


from . import qip, states, random_objects  # noqa: E402,F401
