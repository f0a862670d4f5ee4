"""Gate descriptors with the reference's class names and constructor signatures.

Mirrors `pyramaterised/gates.py` (reference): the same classes, attributes
(`q_on`, `q1`/`q2`, `theta`, `phi`, `param_count`, `is_param`, `layer`,
`commute`, `rotator`, `entangler`, `offset`) and `set_theta`/`set_phi`
behaviour, so circuits built with the reference's API build unchanged.  The
difference is what a gate *is*: the reference materialises a full 2^N x 2^N
QuTiP operator per gate (rebuilt on every `set_theta`, gates.py:122-131);
here a gate is a description that `lowering.py` turns into device ops once,
and angles travel as a parameter matrix to the GB300 kernels.

`rng` is the module-global generator the reference draws "random" angles
from (`gates.py:10`), seeded identically so `run("random")` reproduces the
reference's angle stream.
"""
from typing import Literal, Tuple, Type, TypeAlias, Union  # noqa: F401

import numpy as np

rng = np.random.default_rng(1)

QubitIndex = int
QubitList = Union[list, tuple]
QubitNumber = int
Angle = Union[int, float]
Layer = list
RotationLayer = list
EntanglingLayer = list
Gradient: TypeAlias = object


def prod(factors):
    """Left fold with `*` (gates.py:30-31); kept for API compatibility."""
    out = 1
    for f in factors:
        out = out * f
    return out


def flatten(l):
    return [item for sublist in l for item in sublist]


class Gate:
    """Base descriptor (gates.py:49-100): no parameters, acts as identity."""

    def __init__(self, q_N: QubitNumber) -> None:
        self.q_N = q_N
        self.param_count = 0
        self.is_param = False
        self.theta: Angle = 0
        self.phi: Angle = 0

    def set_theta(self, theta: Angle) -> None:
        return

    def set_phi(self, phi: Angle) -> None:
        return

    def flip_pauli(self) -> None:
        pass

    @property
    def operation(self):
        raise NotImplementedError(
            "pyramaterised_gb300 gates are descriptions lowered to GPU ops; they hold no dense operator"
        )


# ------------------------------------------------------------------ rotations
class PRot(Gate):
    """Parameterised single-qubit rotation exp(-i theta sigma/2) (gates.py:106-147)."""

    pauli_letter = "I"

    def __init__(self, q_on: QubitIndex, q_N: QubitNumber) -> None:
        self.q_on = q_on
        self.q_N = q_N
        self.theta = 0
        self.phi = 0
        self.is_param = True
        self.param_count = 1
        self.pauli_sign = 1

    def set_theta(self, theta: Angle) -> None:
        self.theta = theta

    def flip_pauli(self) -> None:
        # gates.py:140-141 negates `pauli` but derivatives use the `fock`
        # operator built at construction, so the flip never reaches them.
        self.pauli_sign = -self.pauli_sign

    def __repr__(self) -> str:
        return f"{type(self).__name__}({self.theta:.2f})@q{self.q_on}"


class I(PRot):  # noqa: E742  (reference name)
    """Parameterised identity: consumes one angle, applies nothing (gates.py:150-156)."""


class R_x(PRot):
    pauli_letter = "X"


class R_y(PRot):
    pauli_letter = "Y"


class R_z(PRot):
    pauli_letter = "Z"


class negative_R_z(R_z):
    """rz(-theta); derivative +(i/2) Z (gates.py:180-187)."""

    def set_theta(self, theta: Angle) -> None:
        self.theta = -1 * theta


class offset_R_z(R_z):
    """rz(theta + offset) (gates.py:190-205)."""

    def __init__(self, q_on: QubitIndex, q_N: QubitNumber, offset: Angle) -> None:
        super().__init__(q_on, q_N)
        self.offset = offset

    def set_theta(self, theta: Angle) -> None:
        self.theta = theta + self.offset


class H(PRot):
    """Hadamard = X . RY(pi/2) (gates.py:211-232); not parameterised."""

    def __init__(self, q_on: QubitIndex, q_N: QubitNumber) -> None:
        self.q_on = q_on
        self.q_N = q_N
        self.theta = np.pi / 2
        self.phi = 0
        self.is_param = False
        self.param_count = 0
        self.pauli_sign = 1

    def set_theta(self, angle: Angle) -> None:
        return None


class sqrtH(H):
    """Element-wise sqrt of H (gates.py:235-242): not a unitary; unsupported by the engine."""


class X(H):
    """Pauli X (gates.py:245-249)."""


class S(H):
    """phasegate(pi/2) = diag(1, e^{i pi/2}) (gates.py:286-291)."""


class T(H):
    """T = diag(1, e^{i pi/4}) (gates.py:294-300)."""


class fixed_R_y(R_y):
    """Fixed, non-parameterised RY(theta) (gates.py:252-266)."""

    def __init__(self, q_on: QubitIndex, q_N: QubitNumber, theta: Angle) -> None:
        self.q_on = q_on
        self.q_N = q_N
        self.theta = theta
        self.phi = 0
        self.is_param = False
        self.param_count = 0
        self.pauli_sign = 1

    def set_theta(self, theta: Angle) -> None:
        return None


class fixed_R_z(R_z):
    """Fixed, non-parameterised RZ(theta) (gates.py:269-283)."""

    def __init__(self, q_on: QubitIndex, q_N: QubitNumber, theta: Angle) -> None:
        self.q_on = q_on
        self.q_N = q_N
        self.theta = theta
        self.phi = 0
        self.is_param = False
        self.param_count = 0
        self.pauli_sign = 1

    def set_theta(self, theta: Angle) -> None:
        return None


# ------------------------------------------------------------------ entanglers
class EntGate(Gate):
    """Two-qubit fixed gate on (q1, q2) (gates.py:306-324)."""

    def __init__(self, qs_on: QubitList, q_N: QubitNumber) -> None:
        self.q1, self.q2 = qs_on[0], qs_on[1]
        self.q_N = q_N
        self.is_param = False
        self.param_count = 0
        self.theta = 0
        self.phi = 0

    def __repr__(self) -> str:
        return f"{type(self).__name__}@q{self.q1},q{self.q2}"


class CNOT(EntGate):
    """Control q1, target q2 (gates.py:327-330)."""


class CPHASE(EntGate):
    """CZ, as in the reference (gates.py:333-337)."""


class sqrtiSWAP(EntGate):
    """sqrt(iSWAP) (gates.py:340-343)."""


class CZ(EntGate):
    """diag(1, 1, 1, -1) (gates.py:346-349)."""


class CHAIN(EntGate):
    """Entanglers on (2j, 2j+1) for all j, then on (2j+1, 2j+2) (gates.py:355-379)."""

    def __init__(self, entangler: Type[EntGate], q_N: QubitNumber) -> None:
        self.entangler = entangler
        self.q_N = q_N
        self.is_param = False
        self.param_count = 0
        self.theta = 0
        self.phi = 0

    def pairs(self):
        N = self.q_N
        top = [[2 * j, 2 * j + 1] for j in range(N // 2)]
        bottom = [[2 * j + 1, 2 * j + 2] for j in range((N - 1) // 2)]
        return top + bottom

    def __repr__(self) -> str:
        return f"CHAIN connected {self.entangler.__name__}s"


class ALLTOALL(EntGate):
    """Entanglers on every ordered pair, in permutations order (gates.py:382-401)."""

    def __init__(self, entangler: Type[EntGate], q_N: QubitNumber) -> None:
        self.entangler = entangler
        self.q_N = q_N
        self.is_param = False
        self.param_count = 0
        self.theta = 0
        self.phi = 0

    def pairs(self):
        from itertools import permutations

        return [list(p) for p in permutations(range(self.q_N), 2)]

    def __repr__(self):
        return f"ALL connected {self.entangler.__name__}s"


class ARBGATE(Gate):
    """exp(-i theta H) for an arbitrary H (gates.py:407-435): unsupported by the engine."""

    def __init__(self, Ham):
        self._Ham = Ham
        self.theta = 0
        self.phi = 0
        self.is_param = True
        self.param_count = 1

    def set_theta(self, theta):
        self.theta = theta

    def __repr__(self):
        return f"{type(self).__name__}({self.theta:.2f})"


# ------------------------------------------------------------------ shared parameters
class shared_parameter(PRot):
    """One angle shared by a list of rotations (gates.py:441-484)."""

    def __init__(self, layer: RotationLayer, q_N: QubitNumber, commute: bool = True):
        self.layer = layer
        self.theta = 0
        self.phi = 0
        self.q_N = q_N
        self.is_param = True
        self.param_count = 1
        self.commute = commute
        self.pauli_sign = 1

    def set_theta(self, theta: Angle) -> None:
        self.theta = theta
        for gate in self.layer:
            gate.set_theta(theta)

    def flip_pauli(self) -> None:
        for g in self.layer:
            g.flip_pauli()

    def __repr__(self) -> str:
        return f"Block of {self.layer}"


class RR(PRot):
    """cos(theta/2) I - i sin(theta/2) P_q1 P_q2 (gates.py:492-527)."""

    def __init__(self, qs_on: QubitList, q_N: QubitNumber) -> None:
        self.q1, self.q2 = qs_on[0], qs_on[1]
        self.q_N = q_N
        self.theta = 0
        self.phi = 0
        self.is_param = True
        self.param_count = 1
        self.pauli_sign = 1

    def __repr__(self) -> str:
        return f"{type(self).__name__}({self.theta:.2f})@q{self.q1},q{self.q2}"


class R_zz(RR):
    pauli_letter = "Z"


class R_xx(RR):
    pauli_letter = "X"


class R_yy(RR):
    pauli_letter = "Y"


class RR_block(shared_parameter):
    """Shared angle over `rotator` on the periodic ring (i, (i+1) % N) (gates.py:554-585)."""

    def __init__(self, rotator: Type[RR], q_N: QubitNumber):
        self.rotator = rotator
        self.theta = 0
        self.phi = 0
        self.q_N = q_N
        self.is_param = True
        self.param_count = 1
        self.pauli_sign = 1
        self.layer = self.gen_layer()
        self.commute = True

    def gen_layer(self):
        N = self.q_N
        return [self.rotator([i, (i + 1) % N], N) for i in range(N)]

    def __repr__(self) -> str:
        return f"RR block of {self.layer}"


class fSim(PRot):
    """Two-parameter fSim(theta, phi) on (q1, q2) (gates.py:651-697)."""

    def __init__(self, qs_on: QubitList, q_N: QubitNumber) -> None:
        self.q1, self.q2 = qs_on
        self.q_N = q_N
        self.theta = 0
        self.phi = 0
        self.is_param = True
        self.param_count = 2
        self.pauli_sign = 1

    def set_theta(self, theta: Angle) -> None:
        self.theta = theta

    def set_phi(self, phi: Angle) -> None:
        self.phi = phi

    def flip_pauli(self) -> None:
        pass

    def __repr__(self) -> str:
        return f"{type(self).__name__}({self.theta:.2f},{self.phi:.2f})@q{self.q1, self.q2}"


class fixed_fSim(PRot):
    """fSim with the |11> phase fixed to 1 (gates.py:740-759)."""

    def __init__(self, qs_on, q_N):
        self.q1, self.q2 = qs_on
        self.q_N = q_N
        self.theta = 0
        self.phi = 0
        self.is_param = True
        self.param_count = 1
        self.pauli_sign = 1

    def flip_pauli(self) -> None:
        pass
