"""Circuit recipes written against the API both packages share.

Each recipe takes the package module (the reference `pyramaterised`, run on
the QuTiP shim when generating golden vectors, or `pyramaterised_gb300`) and
builds the same circuit with it, so a golden vector produced by the
reference can be compared with the engine's result for the same circuit.
"""
import random

import numpy as np


def qg_test_circuit(pkg):
    """The circuit of the reference's `test_qg_circuit` (tests.py:158-190)."""
    c = pkg.PQC(4)
    c.add_layer([pkg.fixed_R_y(i, 4, np.pi / 4) for i in range(4)])
    c.add_layer([pkg.R_z(0, 4), pkg.R_x(1, 4), pkg.R_y(2, 4), pkg.R_z(3, 4), pkg.CHAIN(pkg.CNOT, 4)])
    c.add_layer([pkg.R_x(0, 4), pkg.R_x(1, 4), pkg.R_x(2, 4), pkg.R_y(3, 4), pkg.CHAIN(pkg.CNOT, 4)])
    c.add_layer([pkg.R_z(0, 4), pkg.R_x(1, 4), pkg.R_y(2, 4), pkg.R_y(3, 4), pkg.CHAIN(pkg.CNOT, 4)], n=1)
    return c


QG_DEFAULT_ANGLES = [3.21587011, 5.97193953, 0.90578156, 5.96054027, 1.9592948, 2.65983852, 5.20060878, 2.571074,
                     3.45319898, 0.17315902, 4.73446249, 3.38125416]  # tests.py:192-205


def he_ladder(pkg, N, L):
    """Hardware-efficient ansatz: RY, RZ on every qubit, then CNOT(i, i+1) for i = 0..N-2."""
    c = pkg.PQC(N)
    layer = [pkg.R_y(i, N) for i in range(N)] + [pkg.R_z(i, N) for i in range(N)]
    layer += [pkg.CNOT([i, i + 1], N) for i in range(N - 1)]
    c.add_layer(layer, n=L)
    return c


def tfim_style(pkg, N, L):
    """RX on every qubit, then CNOT-RZ-CNOT on nearest neighbours (open chain)."""
    c = pkg.PQC(N)
    layer = [pkg.R_x(i, N) for i in range(N)]
    for i in range(N - 1):
        layer += [pkg.CNOT([i, i + 1], N), pkg.R_z(i + 1, N), pkg.CNOT([i, i + 1], N)]
    c.add_layer(layer, n=L)
    return c


def npqc_style(pkg, N, L):
    """RY, RZ on every qubit; CPHASE on (2k, 2k+1), then (2k+1, 2k+2) on alternate layers."""
    c = pkg.PQC(N)
    for l in range(L):
        layer = [pkg.R_y(i, N) for i in range(N)] + [pkg.R_z(i, N) for i in range(N)]
        if l % 2 == 0:
            layer += [pkg.CPHASE([2 * k, 2 * k + 1], N) for k in range(N // 2)]
        else:
            layer += [pkg.CPHASE([2 * k + 1, 2 * k + 2], N) for k in range((N - 1) // 2)]
        c.add_layer(layer)
    return c


def every_gate(pkg, N):
    """One circuit touching every gate class the engine lowers (N >= 4)."""
    c = pkg.PQC(N)
    layer = [pkg.H(0, N), pkg.X(1, N), pkg.S(2, N), pkg.T(3, N), pkg.fixed_R_y(0, N, 0.3), pkg.fixed_R_z(1, N, 1.1),
             pkg.R_x(2, N), pkg.R_y(3, N), pkg.R_z(0, N), pkg.negative_R_z(1, N), pkg.offset_R_z(2, N, 0.7),
             pkg.CNOT([0, 2], N), pkg.CZ([1, 3], N), pkg.CPHASE([3, 0], N), pkg.sqrtiSWAP([2, 1], N),
             pkg.R_xx([0, 1], N), pkg.R_yy([1, 3], N), pkg.R_zz([3, 2], N), pkg.CHAIN(pkg.CNOT, N),
             pkg.shared_parameter([pkg.R_x(i, N) for i in range(N)], N), pkg.RR_block(pkg.R_zz, N),
             pkg.fixed_fSim([0, 3], N), pkg.ALLTOALL(pkg.CZ, N)]
    c.add_layer(layer)
    return c


def fsim_mix(pkg, N):
    """fSim circuit whose get_gradients exercises the reference's second-parameter lookup."""
    c = pkg.PQC(N)
    # the fixed gates in front shift `self.gates[count]` (circuit.py:188) onto RY gates
    c.add_layer([pkg.H(0, N), pkg.CZ([1, 2], N)] + [pkg.R_y(i, N) for i in range(N)]
                + [pkg.fSim([0, 1], N), pkg.fSim([2, 3], N)])
    c.add_layer([pkg.R_z(i, N) for i in range(N)] + [pkg.fSim([1, 2], N)])
    return c


TEMPLATES = [
    ("NPQC", 4, 3), ("NPQC", 6, 4), ("TFIM", 4, 2), ("TFIM_modified", 4, 2), ("XXZ", 4, 2), ("XXZ", 6, 1),
    ("Circuit_1", 4, 2), ("Circuit_2", 4, 2), ("Circuit_2", 5, 2), ("Circuit_9", 4, 2), ("qg_circuit", 4, 1),
    ("generic_HE", 4, 2), ("generic_HE", 5, 2), ("clifford", 4, 2), ("y_CPHASE", 4, 2), ("double_y_CPHASE", 4, 2),
    ("fermionic", 4, 1), ("fermionic", 6, 1), ("zfsim", 4, 2), ("zfsim", 5, 3), ("fsim", 4, 2), ("fixed_fsim", 4, 2),
]


def template_circuit(pkg, name, N, p, seed=7):
    """generate_circuit with Python's `random` seeded (shuffled initial states)."""
    random.seed(seed)
    return pkg.templates.generate_circuit(name, N, p)


def gate_signature(circuit):
    """A comparable description of a circuit's gate list."""
    sig = []
    for g in circuit.gates:
        name = type(g).__name__
        if hasattr(g, "q_on"):
            sig.append((name, int(g.q_on)))
        elif hasattr(g, "q1"):
            sig.append((name, int(g.q1), int(g.q2)))
        elif hasattr(g, "layer"):
            sig.append((name, tuple(gate_signature_list(g.layer))))
        elif hasattr(g, "entangler"):
            sig.append((name, g.entangler.__name__))
        else:
            sig.append((name,))
    return sig


def gate_signature_list(gs):
    class _C:
        pass

    c = _C()
    c.gates = gs
    return gate_signature(c)


def shared_noncommuting(m, N):
    """A shared_parameter(commute=False) block whose members do not commute (gates.py:459-466), between a
    rotation layer and a CNOT ladder + RZ layer."""
    c = m.PQC(N)
    c.add_layer([m.R_y(q, N) for q in range(N)])
    c.add_layer([m.shared_parameter([m.R_x(0, N), m.R_y(0, N), m.R_zz([0, 1], N), m.R_x(1, N),
                                     m.R_xx([1, 2], N)], N, commute=False)])
    c.add_layer([m.CNOT([q, q + 1], N) for q in range(N - 1)] + [m.R_z(q, N) for q in range(N)])
    return c
