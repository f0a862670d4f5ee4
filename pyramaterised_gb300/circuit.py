"""`PQC`: the reference's circuit container, evaluated on the GB300 engine.

Mirrors `pyramaterised/circuit.py` (reference) method by method: building
(`add_layer`, `set_layer`, `get_layer`, `set_gates` with its parameter
bookkeeping), angles (`get_params`, `set_params` drawing "random" angles
from the module-global `gates.rng` in the same order), and evaluation
(`run`, `update_state`, `cost`, `fidelity`, `take_derivative`,
`get_gradients`).  States are torch complex128 tensors on the GPU, shape
(2^N,); a batch API (`run_batch`, `cost_batch`) evaluates many parameter
rows in one launch.
"""
from copy import deepcopy

import numpy as np
import torch

from . import engine
from . import gates as _gates
from . import lowering as _lowering
from .gates import *  # noqa: F401,F403  (the reference re-exports gates from circuit)
from .hamiltonian import PauliSum, zz


class BasisState:
    """Computational basis state |index> of n qubits, kept symbolic."""

    def __init__(self, index, n_qubits):
        self.index = int(index)
        self.n_qubits = int(n_qubits)

    def full(self):
        v = np.zeros(2 ** self.n_qubits, dtype=np.complex128)
        v[self.index] = 1.0
        return v

    def __repr__(self):
        return f"BasisState(|{self.index:0{self.n_qubits}b}>)"


def basis_product(bits):
    """|b_0 ... b_{N-1}> with qubit 0 most significant (the reference's `qt.tensor` of basis kets)."""
    idx = 0
    for b in bits:
        idx = (idx << 1) | int(b)
    return BasisState(idx, len(bits))


class PQC:
    """An n qubit, p layer deep Parameterised Quantum Circuit (circuit.py:12-198)."""

    def __init__(self, n_qubits: QubitNumber) -> None:  # noqa: F405
        self.n_qubits = n_qubits
        self.n_layers = 0
        self.layers = []
        self.gates = []
        self.parameterised = []
        self.n_params = 0
        if n_qubits >= 2:
            self.set_H("ZZ")
        self._initial = BasisState(0, n_qubits)
        self._state = None  # None: the initial state
        self._program = None
        self._tile_qubits = 0
        self._ctas_per_sm = 0
        self._sweep_threads = 0
        self._theta_last = None

    # ------------------------------------------------------------------ Hamiltonian / states
    def set_H(self, H):
        """'ZZ' (default Z_0 Z_1, circuit.py:25-33), a PauliSum, or a small dense matrix."""
        if isinstance(H, str) and H == "ZZ":
            self.H = zz(self.n_qubits)
        elif isinstance(H, PauliSum):
            self.H = H
        else:
            self.H = PauliSum.from_matrix(H.full() if hasattr(H, "full") else H)

    @property
    def initial_state(self):
        return self._initial

    @initial_state.setter
    def initial_state(self, state):
        if isinstance(state, BasisState):
            self._initial = state
            return
        v = state.detach().cpu().numpy() if isinstance(state, torch.Tensor) else np.asarray(
            state.full() if hasattr(state, "full") else state)
        v = np.asarray(v, dtype=np.complex128).reshape(-1)
        nz = np.flatnonzero(v)
        if len(nz) == 1 and v[nz[0]] == 1:
            self._initial = BasisState(int(nz[0]), self.n_qubits)
        else:
            self._initial = v

    def set_initial_state(self, state) -> None:
        """Tensor power of a single-qubit state (circuit.py:35-36)."""
        s = np.asarray(state.full() if hasattr(state, "full") else state, dtype=np.complex128).reshape(-1)
        v = np.array([1.0 + 0j])
        for _ in range(self.n_qubits):
            v = np.kron(v, s)
        self.initial_state = v

    def _psi0(self):
        init = self._initial
        if isinstance(init, BasisState):
            return init.index
        return init

    @property
    def state(self):
        if self._state is None:
            init = self._initial
            v = init.full() if isinstance(init, BasisState) else init
            self._state = engine._c128(v, engine.device())
        return self._state

    @state.setter
    def state(self, value):
        self._state = value if isinstance(value, torch.Tensor) else engine._c128(
            value.full() if hasattr(value, "full") else value, engine.device())

    # ------------------------------------------------------------------ building
    def add_layer(self, layer, n: int = 1) -> None:
        for i in range(n):
            self.layers.append(deepcopy(layer))
        self.n_layers += n
        self.set_gates()

    def set_layer(self, layer, pos: int) -> None:
        self.layers[pos] = deepcopy(layer)
        self.set_gates()

    def get_layer(self, pos: int):
        return self.layers[pos]

    def set_gates(self) -> None:
        """Flatten layers; `parameterised`/`n_params` keep the reference's bookkeeping
        (circuit.py:53-72: the inner for-else appends -1 after every gate and
        `n_params` counts each parameter twice)."""
        layers = []
        for i in self.layers:
            layers = layers + i
        self.gates = layers
        self.parameterised = []
        total = 0
        for gate in self.gates:
            c = gate.param_count
            total += c
            for j in range(c):
                total += 1
                self.parameterised.append(total)
            self.parameterised.append(-1)
        self.n_params = total
        self._program = None
        self._theta_last = None

    def set_tile_qubits(self, k: int) -> None:
        """Shared-memory tile size of the sweep planner (0 = automatic)."""
        self._tile_qubits = int(k)
        self._program = None

    def autotune(self, batch: int):
        """Choose the tile size and CTAs per SM that run this circuit fastest for `batch` parameter rows
        (timed on the device, cached per circuit and batch size); returns the timings."""
        (tile, occ, threads), timings = engine.autotune(self.gates, self.n_qubits, batch)
        self._tile_qubits, self._ctas_per_sm, self._sweep_threads = tile, occ, threads
        self._program = None
        return timings

    @property
    def program(self):
        if self._program is None:
            self._program = engine.Program(self.gates, self.n_qubits, self._tile_qubits)
            if self._ctas_per_sm in (2, 3):
                self._program.set_launch(self._ctas_per_sm, self._sweep_threads if self._ctas_per_sm == 3 else 0)
        return self._program

    # ------------------------------------------------------------------ angles
    def get_params(self):
        angles = []
        for g in self.gates:
            if g.param_count == 2:
                angles.append(g.theta)
                angles.append(g.phi)
            elif g.param_count == 1:
                angles.append(g.theta)
        return angles

    def set_params(self, angles) -> np.ndarray:
        """Assign angles in gate order (circuit.py:86-116); returns the parameter vector."""
        parameterised = [g for g in self.gates if g.is_param]
        out = []
        k = 0
        for g in parameterised:
            if g.param_count == 2:
                if not isinstance(angles, str):
                    a1, a2 = angles[k], angles[k + 1]
                elif angles == "random":
                    a1 = _gates.rng.random(1)[0] * 2 * np.pi
                    a2 = _gates.rng.random(1)[0] * 2 * np.pi
                else:
                    raise Exception("No parameters supplied!")
                g.set_theta(a1)
                g.set_phi(a2)
                out += [a1, a2]
                k += 2
            elif g.param_count == 1:
                if not isinstance(angles, str):
                    a1 = angles[k]
                elif angles == "random":
                    a1 = _gates.rng.random(1)[0] * 2 * np.pi
                else:
                    raise Exception("No parameters supplied!")
                g.set_theta(a1)
                out.append(a1)
                k += 1
        theta = np.asarray([float(a) for a in out], dtype=np.float64)
        self._theta_last = theta
        return theta

    def n_columns(self) -> int:
        """Number of angles `set_params` consumes (the true parameter count)."""
        return sum(int(g.param_count) for g in self.gates if g.is_param)

    def random_params(self, batch: int) -> np.ndarray:
        """`batch` rows drawn from `gates.rng` exactly as `batch` successive run("random") calls."""
        P = self.n_columns()
        th = _gates.rng.random((batch, P)) * 2 * np.pi
        if batch:
            self.set_params(list(th[-1]))
        return th

    # ------------------------------------------------------------------ evaluation
    def run(self, angles):
        """|psi> for `angles` (a list or "random"): a device tensor of shape (2^N,)."""
        theta = self.set_params(angles)
        return self.program.run(theta[None, :], self._psi0())[0]

    def run_batch(self, thetas, mode="c128"):
        """States [B, 2^N] for parameter rows `thetas` [B, P]; mode c128 | c64 | plain."""
        return self.program.run(thetas, self._psi0(), mode=mode)

    def update_state(self, angles):
        self.state = self.run(angles)
        return self.state

    def cost(self, angles) -> float:
        """<psi|H|psi> (circuit.py:132-137)."""
        self.state = self.run(angles=angles)
        return float(engine.expect(self.state, self.H)[0])

    def cost_batch(self, thetas):
        """Energies [B] for parameter rows `thetas` [B, P] (device tensor)."""
        return self.program.energy_grad(thetas, self.H, self._psi0(), want_grad=False)[0]

    def fidelity(self, target_state) -> float:
        """|<psi|phi>|^2 with psi the current state (circuit.py:139-142)."""
        t = target_state
        if hasattr(t, "full") and not isinstance(t, torch.Tensor):
            t = t.full()
        return float(engine.fidelity_pairs(self.state, t)[0])

    def flip_deriv(self) -> None:
        for g in [g for g in self.gates if g.is_param]:
            g.flip_pauli()

    def _current_theta(self):
        last = getattr(self, "_theta_last", None)
        if last is not None and len(last) == self.n_columns():
            return last
        return np.asarray([float(a) for a in self._raw_params()], dtype=np.float64)

    def _raw_params(self):
        """The angles last passed to set_params, in column order (undoing stored offsets)."""
        out = []
        for g in self.gates:
            if not g.is_param:
                continue
            if g.param_count == 2:
                out += [g.theta, g.phi]
            elif g.param_count == 1:
                out.append(_stored_to_angle(g))
        return out

    def take_derivative(self, g_on, param=0):
        """State of the circuit with `g_on` replaced by `deriv * g_on` (circuit.py:149-172)."""
        gi = next(i for i, g in enumerate(self.gates) if g is g_on)
        prog = self.program
        if _lowering.is_composite_shared(g_on):
            return prog.composite_derivative(gi, self._current_theta()[None, :], self._psi0())
        gens, after, n_rows = prog.lowered.gate_runs(gi, param)
        return prog.derivative_states(self._current_theta()[None, :], self._psi0(), gens, after, n_rows)[0]

    def get_gradients(self):
        """Derivative states [P, 2^N] in the reference's order (circuit.py:174-192)."""
        return self.program.gradient_states(self._current_theta()[None, :], self._psi0())

    def __repr__(self) -> str:
        line = f"A {self.n_qubits} qubit, {self.n_layers} layer deep PQC. \n"
        for count, l in enumerate(self.layers):
            line += f"Layer {count}: {l} \n"
        return line


def _stored_to_angle(g):
    """Invert the per-class `set_theta` transform to recover the column angle."""
    if isinstance(g, _gates.negative_R_z):
        return -g.theta
    if isinstance(g, _gates.offset_R_z):
        return g.theta - g.offset
    return g.theta
