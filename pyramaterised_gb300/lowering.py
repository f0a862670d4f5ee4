"""Lower a gate list to the engine's op table and derivative generators.

Forward: every gate becomes one or more `pqc_op` records in application
order, with its angle(s) read from parameter columns assigned in the
reference's `set_params` order (`circuit.py:86-116`: a 2-parameter gate takes
two consecutive columns, theta then phi).

Derivatives: the reference's `get_gradients` (`circuit.py:174-192`) makes one
state per parameter by replacing the gate with `deriv * gate` and re-running
(`take_derivative`, `circuit.py:149-172`).  Here each derivative row is a
list of "runs"; a run inserts one generator op right after the gate's last
op.  A generator that is a sum of Pauli terms (`shared_parameter` with
`commute=True`, `RR_block`; gates.py:451-457) is one run per term and the
engine sums the runs of a row.  The reference's second-parameter lookup for
2-parameter gates, ``self.gates[count]`` with ``count`` the position among
parameterised gates (`circuit.py:188`), is reproduced as written.

`shared_parameter(commute=False)` over members that do not commute
(`gates.py:459-466`: sum_k prod(layer with d_k g_k) times conj(U), a matrix
product with the element-wise conjugate of the block's unitary U) has no
generator-run form; its rows are listed in `composite_rows` and
`engine.Program` builds them from sub-circuits (`composite_derivative`).
"""
from itertools import permutations

import numpy as np

from . import _lib
from . import gates as G

SQ2 = 1.0 / np.sqrt(2.0)


class UnsupportedGate(NotImplementedError):
    pass


def _op(kind, q0, q1=-1, param=-1, param2=-1, scale=1.0, offset=0.0, scale2=1.0, offset2=0.0, m=None, pauli=0,
        sel=-1):
    r = np.zeros((), dtype=_lib.OP_DTYPE)
    r["kind"], r["q0"], r["q1"] = kind, q0, q1
    r["param"], r["param2"], r["sel"], r["pauli"] = param, param2, sel, pauli
    r["scale"], r["offset"], r["scale2"], r["offset2"] = scale, offset, scale2, offset2
    if m is not None:
        flat = np.asarray(m, dtype=np.complex128).reshape(-1)
        r["m"][: 2 * len(flat)] = np.stack([flat.real, flat.imag], axis=1).reshape(-1)
    return r


def _ry(a):
    return np.array([[np.cos(a / 2), -np.sin(a / 2)], [np.sin(a / 2), np.cos(a / 2)]], dtype=np.complex128)


def _hadamard():
    """gates.py:226-232: X . RY(pi/2) (cos/sin(pi/4) differ in the last bit)."""
    return np.array([[0, 1], [1, 0]], dtype=np.complex128) @ _ry(np.pi / 2)


SQRTISWAP = np.array([[1, 0, 0, 0], [0, SQ2, 1j * SQ2, 0], [0, 1j * SQ2, SQ2, 0], [0, 0, 0, 1]], dtype=np.complex128)
ROT_KIND = {"X": _lib.PQC_OP_RX, "Y": _lib.PQC_OP_RY, "Z": _lib.PQC_OP_RZ}
RR_KIND = {"X": _lib.PQC_OP_RXX, "Y": _lib.PQC_OP_RYY, "Z": _lib.PQC_OP_RZZ}


def _ent_ops(ent_cls, q1, q2):
    if issubclass(ent_cls, G.CNOT):
        return [_op(_lib.PQC_OP_CNOT, q1, q2)]
    if issubclass(ent_cls, (G.CPHASE, G.CZ)):
        return [_op(_lib.PQC_OP_CZ, q1, q2)]
    if issubclass(ent_cls, G.sqrtiSWAP):
        return [_op(_lib.PQC_OP_MAT2, q1, q2, m=SQRTISWAP)]
    raise UnsupportedGate(f"entangler {ent_cls.__name__} is not supported")


def _member_ops(g, col):
    """Ops of a rotation that takes its angle from column `col` (shared-parameter members)."""
    if isinstance(g, G.RR):
        return [_op(RR_KIND[g.pauli_letter], g.q1, g.q2, param=col)]
    if isinstance(g, G.negative_R_z):
        return [_op(_lib.PQC_OP_RZ, g.q_on, param=col, scale=-1.0)]
    if isinstance(g, G.offset_R_z):
        return [_op(_lib.PQC_OP_RZ, g.q_on, param=col, offset=float(g.offset))]
    if type(g) is G.I:
        return []
    if isinstance(g, G.PRot) and g.pauli_letter in ROT_KIND and g.is_param:
        return [_op(ROT_KIND[g.pauli_letter], g.q_on, param=col)]
    raise UnsupportedGate(f"{type(g).__name__} cannot be a shared-parameter member")


def gate_ops(g, N, cols):
    """Forward ops of one gate; `cols` are its parameter columns."""
    t = type(g)
    if t is G.sqrtH:
        raise UnsupportedGate("sqrtH (element-wise sqrt of H, gates.py:235-242) is not a unitary gate")
    if t is G.ARBGATE:
        raise UnsupportedGate("ARBGATE (dense expm of an arbitrary operator) is not supported")
    if t is G.H:
        return [_op(_lib.PQC_OP_MAT1, g.q_on, m=_hadamard())]
    if t is G.X:
        return [_op(_lib.PQC_OP_MAT1, g.q_on, m=np.array([[0, 1], [1, 0]]))]
    if t is G.S:
        return [_op(_lib.PQC_OP_MAT1, g.q_on, m=np.diag([1, np.exp(1.0j * np.pi / 2)]))]
    if t is G.T:
        return [_op(_lib.PQC_OP_MAT1, g.q_on, m=np.diag([1, np.exp(1j * np.pi / 4)]))]
    if t is G.fixed_R_y:
        return [_op(_lib.PQC_OP_RY, g.q_on, offset=float(g.theta))]
    if t is G.fixed_R_z:
        return [_op(_lib.PQC_OP_RZ, g.q_on, offset=float(g.theta))]
    if isinstance(g, (G.shared_parameter,)):
        ops = []
        for m in g.layer:
            ops += _member_ops(m, cols[0])
        return ops
    if isinstance(g, G.fSim):
        return [_op(_lib.PQC_OP_FSIM, g.q1, g.q2, param=cols[0], param2=cols[1])]
    if isinstance(g, G.fixed_fSim):
        return [_op(_lib.PQC_OP_FIXED_FSIM, g.q1, g.q2, param=cols[0])]
    if isinstance(g, (G.RR, G.PRot)):
        return _member_ops(g, cols[0])
    if isinstance(g, G.CHAIN):
        return [o for a, b in g.pairs() for o in _ent_ops(g.entangler, a, b)]
    if isinstance(g, G.ALLTOALL):
        return [o for a, b in g.pairs() for o in _ent_ops(g.entangler, a, b)]
    if isinstance(g, G.EntGate):
        return _ent_ops(t, g.q1, g.q2)
    if t is G.Gate:
        return []
    raise UnsupportedGate(f"gate {t.__name__} is not supported")


def _pauli_gen(letters, qubits, coef):
    """Generator run: coef * P on up to two qubits."""
    code = 0
    for j, ch in enumerate(letters):
        code |= _lib.PAULI_LETTER[ch] << (8 * j)
    q0 = qubits[0]
    q1 = qubits[1] if len(qubits) > 1 else -1
    return _op(_lib.PQC_OP_PAULI, q0, q1, m=[complex(coef)], pauli=code)


def _prot_generators(g):
    """`derivative()` of a one-parameter gate as Pauli-term runs (gates.py:133-138, 185-187, 519-522)."""
    if isinstance(g, G.RR):
        return [_pauli_gen(g.pauli_letter * 2, (g.q1, g.q2), -0.5j)]
    if type(g) is G.I:
        return [_pauli_gen("I", (g.q_on,), -0.5j)]
    if type(g) in (G.fixed_R_y, G.fixed_R_z, G.H, G.X, G.S, G.T, G.sqrtH):
        raise UnsupportedGate(f"{type(g).__name__} has no derivative in the reference (it never builds `fock`)")
    if isinstance(g, G.negative_R_z):
        return [_pauli_gen("Z", (g.q_on,), 0.5j)]
    if isinstance(g, G.PRot) and g.pauli_letter in ROT_KIND:
        return [_pauli_gen(g.pauli_letter, (g.q_on,), -0.5j)]
    raise UnsupportedGate(f"no derivative for {type(g).__name__}")


def _commuting_symmetric_rr_layer(layer):
    """True when every member is an RR gate and any two act on identical or disjoint pairs.

    Then the members commute and their product U is symmetric, so the
    reference's non-commuting form sum_k prod(.. d_k g_k ..) * conj(U) * U
    (gates.py:459-466) equals sum_k d_k U, the commuting form.
    """
    if not all(isinstance(m, G.RR) for m in layer):
        return False
    sets = [frozenset((m.q1, m.q2)) for m in layer]
    return all(a == b or not (a & b) for i, a in enumerate(sets) for b in sets[i + 1:])


def is_composite_shared(g):
    """A shared_parameter(commute=False) whose members do not reduce to the commuting form."""
    return (isinstance(g, G.shared_parameter) and not getattr(g, "commute", True)
            and not _commuting_symmetric_rr_layer(g.layer))


def derivative_runs(g, which, cols):
    """Generator runs for `take_derivative(g, param=which)` (which 0: derivative(), 1/2: fSim params)."""
    if isinstance(g, G.fSim):
        kind = _lib.PQC_OP_FSIM_DPHI if which == 2 else _lib.PQC_OP_FSIM_DTHETA
        return [_op(kind, g.q1, g.q2, param=cols[0], param2=cols[1])]
    if isinstance(g, G.fixed_fSim):
        return [_op(_lib.PQC_OP_FIXED_FSIM_DTHETA, g.q1, g.q2, param=cols[0])]
    if isinstance(g, G.shared_parameter):
        if is_composite_shared(g):
            raise UnsupportedGate("shared_parameter(commute=False) over non-commuting members has no run form "
                                  "(Lowered.composite_rows lists it; engine.Program.composite_derivative builds it)")
        runs = []
        for m in g.layer:
            runs += _prot_generators(m)
        return runs
    if isinstance(g, (G.EntGate,)) or type(g) is G.Gate:
        return [_pauli_gen("I", (0,), 1.0)]  # Gate.derivative() = identity (gates.py:93-94)
    return _prot_generators(g)


class Lowered:
    """The op table of a gate list plus the bookkeeping for derivatives."""

    def __init__(self, gates, N):
        self.N = N
        ops = []
        self.gate_cols = []   # parameter columns of each gate
        self.gate_last = []   # index of each gate's last op (-1 before any op)
        col = 0
        for g in gates:
            pc = int(g.param_count) if g.is_param else 0
            cols = list(range(col, col + pc))
            col += pc
            ops += gate_ops(g, N, cols)
            self.gate_cols.append(cols)
            self.gate_last.append(len(ops) - 1)
        self.n_params = col
        self.ops = np.array(ops, dtype=_lib.OP_DTYPE) if ops else np.zeros(0, dtype=_lib.OP_DTYPE)
        self.gates = list(gates)
        self.composite_rows = []

    def gradient_runs(self):
        """(gens, after, n_rows) reproducing `PQC.get_gradients` row by row; the rows of non-commuting
        shared-parameter blocks get no runs and are listed in `self.composite_rows` as (row, gate index)."""
        gens, after = [], []
        self.composite_rows = []
        row = 0
        param_gates = [i for i, g in enumerate(self.gates) if int(g.param_count) > 0]
        for count, gi in enumerate(param_gates):
            g = self.gates[gi]
            if is_composite_shared(g):
                self.composite_rows.append((row, gi))
                row += 1
                continue
            if int(g.param_count) == 1:
                for r in derivative_runs(g, 0, self.gate_cols[gi]):
                    r["sel"] = row
                    gens.append(r)
                    after.append(self.gate_last[gi])
                row += 1
            elif int(g.param_count) == 2:
                for r in derivative_runs(g, 1, self.gate_cols[gi]):
                    r["sel"] = row
                    gens.append(r)
                    after.append(self.gate_last[gi])
                row += 1
                g2i = count  # circuit.py:188 indexes all gates with the parameterised-gate position
                g2 = self.gates[g2i]
                for r in derivative_runs(g2, 2, self.gate_cols[g2i]):
                    r["sel"] = row
                    gens.append(r)
                    after.append(self.gate_last[g2i])
                row += 1
        return self._pack(gens, after, row)

    def gate_runs(self, gate_index, which=0):
        """Runs of `take_derivative(gates[gate_index], param=which)` as row 0."""
        g = self.gates[gate_index]
        gens = derivative_runs(g, which, self.gate_cols[gate_index])
        for r in gens:
            r["sel"] = 0
        return self._pack(gens, [self.gate_last[gate_index]] * len(gens), 1)

    def energy_gradient_runs(self):
        """Generators for d<H>/d theta_j, one column per parameter column (true derivative)."""
        gens, after = [], []
        for gi, g in enumerate(self.gates):
            cols = self.gate_cols[gi]
            if not cols:
                continue
            if isinstance(g, (G.fSim,)):
                raise UnsupportedGate("adjoint gradients of fSim gates are not supported (their reference "
                                      "'derivatives' are not derivatives, gates.py:609-648)")
            if isinstance(g, G.fixed_fSim):
                raise UnsupportedGate("adjoint gradients of fixed_fSim are not supported (gates.py:719-737)")
            for r in derivative_runs(g, 0, cols):
                r["sel"] = cols[0]
                gens.append(r)
                after.append(self.gate_last[gi])
        return self._pack(gens, after, self.n_params)

    @staticmethod
    def _pack(gens, after, n_rows):
        g = np.array(gens, dtype=_lib.OP_DTYPE) if gens else np.zeros(0, dtype=_lib.OP_DTYPE)
        a = np.array(after, dtype=np.int32)
        return g, a, n_rows
