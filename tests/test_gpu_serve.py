"""The serving loop on the GPU: every request gets the same result alone and in a mixed stream, the
batched fused path agrees with the plain op-by-op FP64 path, and admission under a tight HBM budget
completes every request."""
from dataclasses import replace

import numpy as np
import pytest

from oracle import pqc_oracle as O
from pyramaterised_gb300 import serve

pytestmark = pytest.mark.gpu
TOL = 1e-10       # fidelities, Meyer-Wallach Q, energies and gradient entries
QFIM_RTOL = 1e-8


def _close(a, b, kind, atol=TOL):
    if kind == "energy":
        assert abs(a[0] - b[0]) <= atol
        np.testing.assert_allclose(a[1], b[1], atol=atol)
    elif kind == "qfim":
        np.testing.assert_allclose(a, b, rtol=QFIM_RTOL, atol=QFIM_RTOL * max(1.0, np.abs(b).max()))
    else:
        assert abs(a - b) <= atol


@pytest.fixture(scope="module")
def stream():
    return serve.synthetic_stream(60, rate=300.0, seed=11, n_range=(6, 13))


def test_results_are_the_same_alone_and_in_the_mix(cuda, stream):
    srv = serve.Server(hbm_budget=8 << 30, n_streams=3, max_rows=64)
    srv.prepare(stream)
    mixed = srv.run(stream, realtime=True)
    assert sorted(mixed) == [r.rid for r in stream]
    for r in stream[::2]:
        alone = srv.run([replace(r, arrival=0.0)], realtime=False)[r.rid]
        _close(mixed[r.rid].value, alone.value, r.kind, atol=1e-12)
    assert all(res.latency >= 0 for res in mixed.values())
    s = serve.latency_summary(mixed)
    assert s["requests"] == len(stream) and s["p99_ms"] >= s["p50_ms"] > 0


def test_batched_path_matches_plain_path_and_oracle(cuda, stream):
    srv = serve.Server(hbm_budget=8 << 30, n_streams=2, max_rows=128)
    srv.prepare(stream)
    fused = srv.run(stream, realtime=False)
    plain = serve.PlainServer()
    plain.prepare(stream)
    ref = plain.run(stream, realtime=False)
    for r in stream:
        _close(fused[r.rid].value, ref[r.rid].value, r.kind)
    # the oracle on the small fidelity requests
    for r in [q for q in stream if q.kind == "fidelity" and q.n_qubits <= 9][:4]:
        gates = serve.build_ansatz(r.ansatz, r.n_qubits, r.layers).gates
        a = O.run(gates, r.n_qubits, r.theta[0])
        b = O.run(gates, r.n_qubits, r.theta[1])
        assert abs(fused[r.rid].value - abs(np.vdot(a, b)) ** 2) <= TOL


def test_tight_budget_admits_requests_as_memory_frees(cuda, stream):
    big = max(serve.request_bytes(r) for r in stream)
    srv = serve.Server(hbm_budget=2 * big, n_streams=4, max_rows=16)
    srv.prepare(stream)
    res = srv.run(stream, realtime=False)
    assert sorted(res) == [r.rid for r in stream]
    base = serve.Server(hbm_budget=8 << 30, n_streams=1, max_rows=256)
    base.prepare(stream)
    ref = base.run(stream, realtime=False)
    for r in stream:
        _close(res[r.rid].value, ref[r.rid].value, r.kind, atol=1e-12)


def test_cross_family_batches_give_the_single_family_results(cuda, stream):
    # fidelity / MW requests of small families share MultiBatch launches (pqc_run_multi); every result equals
    # the one of the per-family batches
    mixed = serve.Server(hbm_budget=8 << 30, n_streams=2, max_rows=128, multi_max_qubits=13)
    single = serve.Server(hbm_budget=8 << 30, n_streams=2, max_rows=128, multi_max_qubits=0)
    for srv in (mixed, single):
        srv.prepare(stream)
    a = mixed.run(stream, realtime=False)
    b = single.run(stream, realtime=False)
    assert sorted(a) == sorted(b) == [r.rid for r in stream]
    for r in stream:
        _close(a[r.rid].value, b[r.rid].value, r.kind, atol=1e-12)
