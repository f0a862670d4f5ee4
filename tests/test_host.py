"""Host-side logic, no GPU: templates, lowering, the sweep planner, the C ABI surface."""
import itertools
import os
import re
import subprocess

import numpy as np
import pytest

import op_interp
import recipes
from oracle import pqc_oracle as O
import pyramaterised_gb300 as pq
from pyramaterised_gb300 import _lib, engine, gates
from pyramaterised_gb300.lowering import Lowered, UnsupportedGate

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "pyramaterised_gb300.h")


def _norm(x):
    if isinstance(x, (list, tuple)):
        return [_norm(y) for y in x]
    return x


def test_template_gate_sequences_match_reference(golden_meta):
    for key, sig in golden_meta["signatures"].items():
        _, name, N, p = key.split("/")
        c = recipes.template_circuit(pq, name, int(N), int(p))
        mine = _norm(recipes.gate_signature(c))
        assert mine == _norm(sig), key


def test_set_gates_bookkeeping_quirks():
    # circuit.py:53-72: the for-else appends -1 after every gate and n_params double counts
    c = pq.PQC(3)
    c.add_layer([pq.R_x(0, 3), pq.CNOT([0, 1], 3), pq.fSim([1, 2], 3)])
    assert c.parameterised == [2, -1, -1, 5, 6, -1]
    assert c.n_params == 6 and c.n_columns() == 3


def test_random_angles_follow_reference_stream():
    # run("random") draws rng.random(1)[0]*2*pi per parameter from default_rng(1) (gates.py:10, circuit.py:99-112)
    gates.rng = np.random.default_rng(1)
    c = recipes.he_ladder(pq, 3, 2)
    th = c.random_params(5)
    ref = np.random.default_rng(1)
    seq = np.array([[ref.random(1)[0] * 2 * np.pi for _ in range(12)] for _ in range(5)])
    assert np.array_equal(th, seq)
    assert np.array_equal(np.array(c.get_params()), seq[-1])
    gates.rng = np.random.default_rng(1)


def _cases(golden):
    keys = sorted({k.rsplit("/", 1)[0] for k in golden.files if k.endswith("/state")})
    from test_oracle import _build

    return [(k, _build(k)) for k in keys]


def test_lowering_reproduces_reference_states(golden):
    # op table interpreted in numpy == the reference's states (checks the lowering, not the kernels)
    for key, c in _cases(golden):
        N = c.n_qubits
        L = Lowered(c.gates, N)
        psi = op_interp.run_ops(L.ops, golden[f"{key}/theta"], N, golden[f"{key}/init"])
        np.testing.assert_allclose(psi, golden[f"{key}/state"], atol=1e-12, err_msg=key)


def test_lowered_derivative_runs_reproduce_reference_gradients(golden):
    for key, c in _cases(golden):
        if f"{key}/grads" not in golden.files:
            continue
        N = c.n_qubits
        L = Lowered(c.gates, N)
        th = golden[f"{key}/theta"]
        gens, after, n_rows = L.gradient_runs()
        rows = np.zeros((n_rows, 2 ** N), dtype=np.complex128)
        for g, a in zip(gens, after):
            order = list(range(a + 1))
            psi = op_interp.run_ops(L.ops, th, N, golden[f"{key}/init"], order)
            psi = op_interp.apply_op(psi, g, th, N)
            psi = op_interp.run_ops(L.ops, th, N, psi, list(range(a + 1, len(L.ops))))
            rows[int(g["sel"])] += psi
        for row, gi in L.composite_rows:  # the engine's composite_derivative, restated on the op interpreter
            g = c.gates[gi]
            col, last = L.gate_cols[gi][0], int(L.gate_last[gi])
            psi_g = op_interp.run_ops(L.ops, th, N, golden[f"{key}/init"], list(range(last + 1)))
            LL = Lowered(list(g.layer), N)
            tl = np.full(LL.n_params, th[col])
            phi = np.conj(op_interp.run_ops(LL.ops, tl, N, np.conj(psi_g)))
            lg, la, _ = LL.gradient_runs()
            chi = np.zeros_like(phi)
            for gg, a in zip(lg, la):
                v = op_interp.run_ops(LL.ops, tl, N, phi, list(range(a + 1)))
                v = op_interp.apply_op(v, gg, tl, N)
                chi += op_interp.run_ops(LL.ops, tl, N, v, list(range(a + 1, len(LL.ops))))
            rows[row] = op_interp.run_ops(L.ops, th, N, chi, list(range(last + 1, len(L.ops))))
        np.testing.assert_allclose(rows, golden[f"{key}/grads"], atol=1e-12, err_msg=key)


@pytest.mark.parametrize("N,k", [(8, 5), (10, 6), (11, 7), (12, 8)])
def test_planner_reordering_preserves_the_state(engine_lib, N, k):
    rs = np.random.default_rng(N)
    for build in (recipes.he_ladder, recipes.tfim_style, recipes.npqc_style):
        c = build(pq, N, 3)
        L = Lowered(c.gates, N)
        th = rs.random(L.n_params) * 2 * np.pi
        order, sweep, ns = engine.plan_order(L.ops, N, k)
        assert sorted(order) == list(range(len(L.ops)))
        assert ns > 1
        psi0 = O.basis_state(N)
        a = op_interp.run_ops(L.ops, th, N, psi0)
        b = op_interp.run_ops(L.ops, th, N, psi0, order)
        np.testing.assert_allclose(a, b, atol=1e-12)


@pytest.mark.parametrize("N,p", [(8, 4), (10, 5), (12, 6)])
def test_fusion_schedule_groups_npqc_rotations(engine_lib, N, p):
    # NPQC layers (templates.py:66-95) interleave RY and RZ on each even qubit; the planner reorders commuting
    # ops so that the RYs pair and the RZs share phase-block passes.  The order must give the same state.
    layers, theta_ref = pq.templates.NPQC_layers(p, N)
    c = pq.PQC(N)
    for layer in layers:
        c.add_layer(layer)
    L = Lowered(c.gates, N)
    order, _, _ = engine.plan_order(L.ops, N)
    assert sorted(order) == list(range(len(L.ops)))
    th = np.random.default_rng(N).random(L.n_params) * 2 * np.pi
    psi0 = O.basis_state(N)
    np.testing.assert_allclose(op_interp.run_ops(L.ops, th, N, psi0, order), op_interp.run_ops(L.ops, th, N, psi0),
                               atol=1e-12)
    kinds = L.ops["kind"][order]
    # every layer after the first: its even-qubit RYs now sit in one run (interleaved with RZ they formed none)
    runs = [len(list(g)) for k, g in itertools.groupby(kinds) if k == _lib.PQC_OP_RY]
    assert max(runs) >= N // 2
    assert not np.array_equal(order, np.arange(len(L.ops)))


def _derivative_circuits():
    yield "he_ladder", recipes.he_ladder(pq, 7, 3), 0
    yield "every_gate", recipes.every_gate(pq, 6), 4
    yield "fsim_mix", recipes.fsim_mix(pq, 6), 0
    for name, N, p in (("Circuit_9", 7, 3), ("generic_HE", 7, 2), ("qg_circuit", 6, 2), ("TFIM", 6, 3),
                       ("XXZ", 6, 2)):
        yield name, pq.templates.generate_circuit(name, N, p), 0
    layers, _ = pq.templates.NPQC_layers(4, 8)
    c = pq.PQC(8)
    for layer in layers:
        c.add_layer(layer)
    yield "NPQC", c, 5


@pytest.mark.parametrize("case", list(range(9)))
def test_derivative_plan_order_gives_every_run_its_state(engine_lib, case):
    # The derivative plan may reorder commuting forward ops (rotation pairs, phase blocks) and move each generator
    # later past the ops it commutes with.  Replaying each run in the plan's order on the op interpreter must give
    # the run of the reference's take_derivative: the ops before the generator's op, the generator, the rest.
    name, c, k = list(_derivative_circuits())[case]
    N = c.n_qubits
    L = Lowered(c.gates, N)
    gens, after, n_rows = L.gradient_runs()
    order, ns = engine.derivative_plan_order(L.ops, gens, after, N, k)
    assert sorted(order) == sorted(list(range(len(L.ops))) + [-(r + 1) for r in range(len(gens))]), name
    th = np.random.default_rng(case).random(L.n_params) * 2 * np.pi
    psi0 = O.basis_state(N)
    for r in range(len(gens)):
        a = int(after[r])
        want = op_interp.run_ops(L.ops, th, N, psi0, list(range(a + 1)))
        want = op_interp.apply_op(want, gens[r], th, N)
        want = op_interp.run_ops(L.ops, th, N, want, list(range(a + 1, len(L.ops))))
        psi = psi0
        for v in order:
            if v >= 0:
                psi = op_interp.apply_op(psi, L.ops[v], th, N)
            elif v == -(r + 1):
                psi = op_interp.apply_op(psi, gens[r], th, N)
        np.testing.assert_allclose(psi, want, atol=1e-12, err_msg=f"{name} run {r}")


def _random_circuit(rng, N, n_gates):
    """A random gate list over the classes the engine lowers, weighted towards rotations and diagonal gates so
    that the planner's reordering and generator moves have runs to work on."""
    one = [pq.R_x, pq.R_y, pq.R_z, pq.negative_R_z]  # H, X, S, T have no derivative in the reference
    two = [pq.CNOT, pq.CZ, pq.CPHASE, pq.R_zz, pq.R_xx, pq.R_yy, pq.fSim, pq.sqrtiSWAP]
    gates_ = []
    for _ in range(n_gates):
        if rng.random() < 0.7:
            g = one[rng.integers(len(one))]
            gates_.append(g(int(rng.integers(N)), N))
        else:
            a, b = rng.choice(N, 2, replace=False)
            g = two[rng.integers(len(two))]
            gates_.append(g([int(a), int(b)], N))
    c = pq.PQC(N)
    c.add_layer(gates_)
    return c


@pytest.mark.parametrize("seed", list(range(12)))
def test_planner_random_circuits_keep_states_and_derivative_runs(engine_lib, seed):
    # Random circuits, tiles of 4 to N qubits: the forward order (with the fusion schedule) gives the circuit's
    # state, and every derivative run replayed in the derivative plan's order gives take_derivative's state.
    rng = np.random.default_rng(100 + seed)
    N = int(rng.integers(5, 8))
    c = _random_circuit(rng, N, int(rng.integers(20, 60)))
    L = Lowered(c.gates, N)
    th = rng.random(L.n_params) * 2 * np.pi
    psi0 = O.basis_state(N)
    k = int(rng.integers(4, N + 1))
    order, _, _ = engine.plan_order(L.ops, N, k)
    np.testing.assert_allclose(op_interp.run_ops(L.ops, th, N, psi0, order), op_interp.run_ops(L.ops, th, N, psi0),
                               atol=1e-12)
    gens, after, _ = L.gradient_runs()
    dorder, _ = engine.derivative_plan_order(L.ops, gens, after, N, k)
    for r in range(len(gens)):
        a = int(after[r])
        want = op_interp.run_ops(L.ops, th, N, psi0, list(range(a + 1)))
        want = op_interp.apply_op(want, gens[r], th, N)
        want = op_interp.run_ops(L.ops, th, N, want, list(range(a + 1, len(L.ops))))
        psi = psi0
        for v in dorder:
            if v >= 0:
                psi = op_interp.apply_op(psi, L.ops[v], th, N)
            elif v == -(r + 1):
                psi = op_interp.apply_op(psi, gens[r], th, N)
        np.testing.assert_allclose(psi, want, atol=1e-12, err_msg=f"seed {seed} run {r}")


def test_planner_every_gate_and_generators(engine_lib):
    c = recipes.every_gate(pq, 6)
    L = Lowered(c.gates, 6)
    th = np.random.default_rng(0).random(L.n_params)
    for k in (4, 5):
        order, sweep, ns = engine.plan_order(L.ops, 6, k)
        a = op_interp.run_ops(L.ops, th, 6, O.basis_state(6))
        b = op_interp.run_ops(L.ops, th, 6, O.basis_state(6), order)
        np.testing.assert_allclose(a, b, atol=1e-12)


def test_sweep_counts_at_benchmark_sizes(engine_lib):
    # N <= 13 is one sweep; at N = 20 the commutation-aware planner needs fewer sweeps per layer than a
    # naive plan, which takes ceil(N / k) sweeps per layer (2 with 2^13-amplitude tiles, 2 with 2^12)
    for N, L in ((12, 12), (20, 20)):
        c = pq.templates.hardware_efficient_ladder(N, L)
        ops = Lowered(c.gates, N).ops
        _, _, ns = engine.plan_order(ops, N)
        if N <= 13:
            assert ns == 1
        else:
            assert ns < 2 * L
            _, _, ns13 = engine.plan_order(ops, N, 13)
            assert ns13 <= 1.5 * L


def test_abi_exports_every_declared_symbol(engine_lib):
    with open(HEADER) as f:
        text = f.read()
    declared = set(re.findall(r"\b(pqc_[a-z0-9_]+)\s*\(", text))
    lib_path = pq.build.lib_path()
    out = subprocess.run(["nm", "-D", "--defined-only", lib_path], capture_output=True, text=True).stdout
    exported = set(re.findall(r" T (pqc_[a-z0-9_]+)", out))
    assert declared and declared <= exported, declared - exported
    assert set(_lib.EXPORTS) <= exported


def test_header_struct_layout_matches_python(tmp_path):
    src = tmp_path / "sz.c"
    src.write_text('#include <stdio.h>\n#include <stddef.h>\n#include "pyramaterised_gb300.h"\n'
                   'int main(void){printf("%zu %zu %zu %zu\\n", sizeof(pqc_op), sizeof(pqc_pauli_term),'
                   ' offsetof(pqc_op, m), offsetof(pqc_op, scale)); return 0;}\n')
    exe = tmp_path / "sz"
    subprocess.run(["gcc", "-std=c99", "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe)], check=True)
    sizes = subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.split()
    assert [int(s) for s in sizes] == [_lib.OP_DTYPE.itemsize, _lib.TERM_DTYPE.itemsize,
                                        _lib.OP_DTYPE.fields["m"][1], _lib.OP_DTYPE.fields["scale"][1]]


def test_invalid_programs_fail_with_messages(engine_lib):
    ops = np.zeros(1, dtype=_lib.OP_DTYPE)
    ops[0]["kind"], ops[0]["q0"], ops[0]["q1"] = _lib.PQC_OP_CNOT, 0, 0  # same qubit twice
    with pytest.raises(_lib.EngineError, match="second qubit"):
        engine.plan_order(ops, 3)
    ops[0]["kind"] = 99
    ops[0]["q1"] = 1
    with pytest.raises(_lib.EngineError, match="unsupported kind"):
        engine.plan_order(ops, 3)
    ops[0]["kind"], ops[0]["q0"] = _lib.PQC_OP_RX, 7
    with pytest.raises(_lib.EngineError, match="out of range"):
        engine.plan_order(ops, 3)
    # derivative plans: generator positions must name an op (or -1, before the first)
    L = Lowered(recipes.he_ladder(pq, 4, 2).gates, 4)
    gens, after, _ = L.gradient_runs()
    bad = np.array(after, dtype=np.int32)
    bad[0] = len(L.ops)
    with pytest.raises(_lib.EngineError, match="gen_after out of range"):
        engine.derivative_plan_order(L.ops, gens, bad, 4)
    bad[0] = -2
    with pytest.raises(_lib.EngineError, match="gen_after out of range"):
        engine.derivative_plan_order(L.ops, gens, bad, 4)
    order, ns = engine.derivative_plan_order(L.ops, gens[:0], bad[:0], 4)  # no generators: the forward ops only
    assert sorted(order) == list(range(len(L.ops))) and ns >= 1


def test_unsupported_gates_are_rejected():
    c = pq.PQC(2)
    c.add_layer([pq.gates.sqrtH(0, 2)])
    with pytest.raises(UnsupportedGate):
        Lowered(c.gates, 2)
    c = pq.PQC(2)
    c.add_layer([pq.gates.ARBGATE(np.eye(4))])
    with pytest.raises(UnsupportedGate):
        Lowered(c.gates, 2)


def test_engine_fails_loudly_without_gpu():
    import torch

    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    c = recipes.he_ladder(pq, 3, 1)
    with pytest.raises(_lib.EngineError, match="CUDA device"):
        c.run([0.1] * 6)


def test_pauli_sum_from_matrix_roundtrip():
    H = pq.templates.TFIM_hamiltonian(3, 0.7, 0.2)
    H2 = pq.PauliSum.from_matrix(H.full())
    np.testing.assert_allclose(H2.full(), H.full(), atol=1e-13)
    ref = O.tfim_reference(3, 0.7, 0.2)
    psi = np.random.default_rng(0).standard_normal(8) + 0j
    psi /= np.linalg.norm(psi)
    assert abs(np.vdot(psi, H.full() @ psi).real - O.expect(ref, psi, 3)) < 1e-12
