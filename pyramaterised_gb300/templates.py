"""Circuit library with the reference's template names and gate sequences.

Mirrors `pyramaterised/templates.py` (reference): each builder returns the
same gates in the same order as the reference's (the gate lists are the
engine's input, so their order is part of parity).  Templates that start
from a half-filled product state draw the shuffle from Python's `random`
module, like the reference (templates.py:373-377).  `TFIM_hamiltonian`
returns a `PauliSum` instead of a QuTiP operator.
"""
import random

import numpy as np

from .circuit import PQC, basis_product
from .gates import (CHAIN, CNOT, CPHASE, CZ, H, R_x, R_xx, R_y, R_yy, R_z, R_zz, RR_block, S, X, fSim, fixed_fSim,
                    fixed_R_y, fixed_R_z, negative_R_z, offset_R_z, shared_parameter, sqrtiSWAP)
from .hamiltonian import PauliSum, tfim_periodic

LEN_CLIFF_STRING = 3


def clifford_circuit_layers(p, N, method="random"):
    """Random Clifford layers from {H, S, CZ, CNOT} (templates.py:17-48)."""
    pool = [H, S, CZ, CNOT]
    qs = list(range(N))
    layers = []
    if method.lower() == "random":
        for _ in range(p):
            layer = []
            for _n in range(N):
                gate = random.choice(pool)
                if gate in (H, S):
                    layer.append(gate(random.randint(0, N - 1), N))
                else:
                    a, b = random.sample(qs, k=2)
                    layer.append(gate([a, b], N))
            layers.append(layer)
    else:
        singles = pool[:2]
        for _ in range(p):
            qs_on = random.sample(qs, k=N // 2)
            strings = [random.choices(singles, k=LEN_CLIFF_STRING) for _q in qs_on]
            layer = [g(q, N) for q, string in zip(qs_on, strings) for g in string]
            layer.append(CHAIN(CNOT, N))
            layers.append(layer)
    return layers


def gen_shift_list(p, N):
    """Shift sequence a_s of the NPQC construction (templates.py:51-63)."""
    pending = list(range(N // 2))
    shifts = np.zeros(2 ** (N // 2), dtype=np.int32)
    s = 1
    while pending:
        shifts[s - 1] = pending.pop(0)
        for q in range(1, s):
            shifts[s + q - 1] = shifts[q - 1]
        s *= 2
    return shifts


def NPQC_layers(p, N):
    """NPQC layers and their reference angles (templates.py:66-95)."""
    layers = [[R_y(i, N) for i in range(N)] + [R_z(i, N) for i in range(N)]]
    angles = [np.pi / 2] * N + [0] * N
    shifts = gen_shift_list(p, N)
    for i in range(p - 1):
        a_l = shifts[i]
        evens = [2 * k - 2 for k in range(1, 1 + N // 2)]
        fixed = [fixed_R_y(q, N, np.pi / 2) for q in evens]
        ents = [CPHASE([q, ((q + 1) + 2 * a_l) % N], N) for q in evens]
        layer = fixed + ents
        for q in evens:
            layer = layer + [R_y(q, N), R_z(q, N)]
            angles.append(np.pi / 2)
            angles.append(0)
        layers.append(layer)
    return layers, angles


def string_to_entangler(string):
    """templates.py:98-111."""
    table = {"cnot": CNOT, "cphase": CPHASE, "cz": CZ, "sqrtiswap": sqrtiSWAP}
    try:
        return table[string.lower()]
    except KeyError:
        raise Exception("Must supply a valid entangler!")


def _repeat(layer, p):
    return [layer for _ in range(p)]


def circuit_1_layers(p, N):
    """arXiv:1905.10876 circuit 1 (templates.py:114-119)."""
    return _repeat([R_x(i, N) for i in range(N)] + [R_y(i, N) for i in range(N)], p)


def circuit_2_layers(p, N, ent_str="cnot"):
    """Circuit 2 (templates.py:122-128)."""
    e = string_to_entangler(ent_str)
    return _repeat([R_x(i, N) for i in range(N)] + [R_z(i, N) for i in range(N)] + [CHAIN(e, N)], p)


def circuit_9_layers(p, N, ent_str="cphase"):
    """Circuit 9 (templates.py:131-137)."""
    e = string_to_entangler(ent_str)
    return _repeat([H(i, N) for i in range(N)] + [CHAIN(e, N)] + [R_x(i, N) for i in range(N)], p)


def qg_circuit_layers(p, N, ent_str="cnot"):
    """arXiv:2102.01659 circuit (templates.py:140-151)."""
    e = string_to_entangler(ent_str)
    init = [fixed_R_y(i, N, np.pi / 4) for i in range(N)]
    layer = []
    for rot in (R_z, R_x, R_z):
        layer += [rot(i, N) for i in range(N)] + [CHAIN(e, N)]
    return [init] + _repeat(layer, p)


def generic_HE_layers(p, N, ent_str="cnot"):
    """Generic hardware-efficient circuit (templates.py:154-162)."""
    e = string_to_entangler(ent_str)
    init = [fixed_R_y(i, N, np.pi / 4) for i in range(N)]
    layer = [R_y(i, N) for i in range(N)] + [R_z(i, N) for i in range(N)] + [CHAIN(e, N)]
    return [init] + _repeat(layer, p)


def clifford_HE_layers(p, N, ent_str="cnot"):
    """templates.py:164-171."""
    e = string_to_entangler(ent_str)
    return _repeat([R_y(i, N) for i in range(N)] + [R_z(i, N) for i in range(N)] + [CHAIN(e, N)], p)


def y_CPHASE_layers(p, N):
    """templates.py:173-180."""
    return _repeat([R_y(i, N) for i in range(N)] + [CHAIN(CPHASE, N)], p)


def double_y_CPHASE_layers(p, N):
    """templates.py:182-189."""
    return _repeat([R_y(i, N) for i in range(N)] + [R_y(i, N) for i in range(N)] + [CHAIN(CPHASE, N)], p)


def TFIM_layers(p, N):
    """TFIM circuit (templates.py:194-204): H layer, then [RR_block(R_zz), shared RX] x p."""
    layers = [[H(i, N) for i in range(N)]]
    for _ in range(p):
        layers.append([RR_block(R_zz, N), shared_parameter([R_x(i, N) for i in range(N)], N)])
    return layers


def modified_TFIM_layers(p, N):
    """templates.py:207-217."""
    layers = []
    for _ in range(p):
        layers.append([RR_block(R_zz, N), shared_parameter([R_x(i, N) for i in range(N)], N),
                       shared_parameter([R_z(i, N) for i in range(N)], N)])
    return layers


def TFIM_hamiltonian(N, g, h=0):
    """-sum_i (Z_i Z_{i+1 mod N} + g X_i + h Z_i) (templates.py:220-227), as a PauliSum."""
    return tfim_periodic(N, g, h)


def XXZ_layers(p, N, commute=False):
    """XXZ circuit (templates.py:230-257)."""
    even = [(2 * i - 2, 2 * i - 1) for i in range(1, N // 2 + 1)]
    odd = [(2 * i - 1, (2 * i) % N) for i in range(1, N // 2 + 1)]
    layers = []
    for _ in range(p):
        layers.append([
            shared_parameter([R_zz((i, j), N) for i, j in odd], N),
            shared_parameter([R_yy((i, j), N) for i, j in odd] + [R_xx((i, j), N) for i, j in odd], N,
                             commute=commute),
            shared_parameter([R_zz((i, j), N) for i, j in even], N),
            shared_parameter([R_yy((i, j), N) for i, j in even] + [R_xx((i, j), N) for i, j in even], N,
                             commute=commute),
        ])
    return layers


def gen_theta_block(q1, q2, N):
    """Fermionic theta block (templates.py:260-274)."""
    return [
        sqrtiSWAP([q1, q2], N),
        shared_parameter([negative_R_z(q1, N), offset_R_z(q2, N, np.pi)], N),
        sqrtiSWAP([q1, q2], N),
        fixed_R_z(q2, N, np.pi),
    ]


def list_to_pairs(x):
    return [(x[i], x[i + 1]) for i in range(0, len(x) - 1, 2)]


def fermionic_circuit_layers(p, N):
    """Diamond of theta blocks (templates.py:282-304)."""
    layers = []
    for _ in range(p):
        blocks = []
        for n in range(1, 1 + N // 2):
            first = list(range(N // 2 - n + 1, N // 2 + 1))
            second = list(range(1 + N // 2, 1 + N // 2 + n))
            blocks.append(list_to_pairs(first + second))
        blocks = blocks + list(reversed(blocks))[1:]
        for b in blocks:
            layer = []
            for a, c in b:
                layer += gen_theta_block(a - 1, c - 1, N)
            layers.append(layer)
    return layers


def fSim_circuit_layers(p, N, rotator="y", fixed=False):
    """fSim circuits with periodic connections (templates.py:307-353)."""
    rots = {"y": R_y, "x": R_x, "z": R_z}
    r = rotator.lower()
    if r not in rots:
        raise Exception("Please supply a valid single qubit rotator")
    rot = rots[r]
    make = fixed_fSim if fixed is True else fSim
    layers = []
    for l in range(p):
        layer = [rot(i, N) for i in range(N)]
        if N % 2 == 0:
            for i in range(l % 2, N, 2):
                layer.append(make([i, (i + 1) % N], N))
        else:
            offset = l % N
            idx = [i for i in range(N) if i != offset]
            pairs = []
            if offset % 2 == 1:
                pairs.append((idx.pop(0), idx.pop(-1)))
            pairs += [(idx[i], idx[i + 1]) for i in range(0, len(idx), 2)]
            for a, b in pairs:
                layer.append(make([a, b], N))
            layer.append(rot(offset, N))
        layers.append(layer)
    return layers


def add_layers(circuit, layers):
    for l in layers:
        circuit.add_layer(l)
    return circuit


def _half_filled(N, shuffle):
    bits = [1] * (N // 2) + [0] * (N - N // 2)
    if shuffle:
        random.shuffle(bits)
    return basis_product(bits)


def generate_circuit(circuit_type, N, p, hamiltonian="ZZ", rotator="", shuffle=True):
    """Build an N qubit, p layer circuit from its name (templates.py:361-429)."""
    circuit = PQC(N)
    if circuit_type == "NPQC":
        layers, theta_ref = NPQC_layers(p, N)
    elif circuit_type == "TFIM":
        layers = TFIM_layers(p, N)
    elif circuit_type == "TFIM_modified":
        layers = modified_TFIM_layers(p, N)
    elif circuit_type == "XXZ":
        layers = XXZ_layers(p, N)
        circuit.initial_state = _half_filled(N, shuffle)
    elif circuit_type == "Circuit_1":
        layers = circuit_1_layers(p, N)
    elif circuit_type == "Circuit_2":
        layers = circuit_2_layers(p, N)
    elif circuit_type == "Circuit_9":
        layers = circuit_9_layers(p, N)
    elif circuit_type == "qg_circuit":
        layers = qg_circuit_layers(p, N)
    elif circuit_type == "generic_HE":
        layers = generic_HE_layers(p, N)
    elif circuit_type == "clifford":
        layers = clifford_HE_layers(p, N)
    elif circuit_type == "y_CPHASE":
        layers = y_CPHASE_layers(p, N)
    elif circuit_type == "double_y_CPHASE":
        layers = double_y_CPHASE_layers(p, N)
    elif circuit_type == "fermionic":
        layers = fermionic_circuit_layers(p, N)
        circuit.initial_state = _half_filled(N, shuffle)
    elif circuit_type == "zfsim":
        layers = fSim_circuit_layers(p, N, rotator="z")
        circuit.initial_state = _half_filled(N, shuffle)
    elif circuit_type == "fsim":
        layers = fSim_circuit_layers(p, N, rotator=rotator) if rotator in ["x", "y", "z"] else fSim_circuit_layers(p, N)
        circuit.initial_state = _half_filled(N, shuffle)
    elif circuit_type == "fixed_fsim":
        layers = fSim_circuit_layers(p, N, rotator="z", fixed=True)
        circuit.initial_state = _half_filled(N, shuffle)
    for l in layers:
        circuit.add_layer(l)
    return circuit


# ---------------------------------------------------------------------- benchmark ansaetze
def hardware_efficient_ladder(N, L):
    """L layers of RY then RZ on every qubit followed by a CNOT ladder 0->1->...->N-1."""
    c = PQC(N)
    layer = [R_y(i, N) for i in range(N)] + [R_z(i, N) for i in range(N)] + [CNOT([i, i + 1], N) for i in range(N - 1)]
    c.add_layer(layer, n=L)
    return c


def tfim_style(N, L):
    """L layers of RX on every qubit, then ZZ(theta) as CNOT-RZ-CNOT on nearest neighbours (open chain)."""
    c = PQC(N)
    layer = [R_x(i, N) for i in range(N)]
    for i in range(N - 1):
        layer += [CNOT([i, i + 1], N), R_z(i + 1, N), CNOT([i, i + 1], N)]
    c.add_layer(layer, n=L)
    return c


def npqc_style(N, L):
    """L layers of RY and RZ on every qubit with CPHASE on (2k, 2k+1), then (2k+1, 2k+2) on alternate layers."""
    c = PQC(N)
    for l in range(L):
        layer = [R_y(i, N) for i in range(N)] + [R_z(i, N) for i in range(N)]
        if l % 2 == 0:
            layer += [CPHASE([2 * k, 2 * k + 1], N) for k in range(N // 2)]
        else:
            layer += [CPHASE([2 * k + 1, 2 * k + 2], N) for k in range((N - 1) // 2)]
        c.add_layer(layer)
    return c
