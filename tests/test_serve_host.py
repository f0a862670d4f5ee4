"""Host-side logic of the serving loop: the synthetic request stream and batch admission."""
import time
from collections import deque

import numpy as np

from pyramaterised_gb300 import serve


def test_stream_is_seeded_and_respects_its_ranges():
    a = serve.synthetic_stream(400, rate=100.0, seed=3)
    b = serve.synthetic_stream(400, rate=100.0, seed=3)
    assert [(r.kind, r.n_qubits, r.layers, r.ansatz) for r in a] == [(r.kind, r.n_qubits, r.layers, r.ansatz) for r in b]
    assert all(np.array_equal(x.theta, y.theta) for x, y in zip(a, b))
    t = np.array([r.arrival for r in a])
    assert np.all(np.diff(t) >= 0) and 2.0 < t[-1] < 6.0  # 400 arrivals at 100/s
    for r in a:
        assert 6 <= r.n_qubits <= 22 and r.ansatz in serve.ANSATZE and r.kind in serve.KINDS
        ppl = serve.params_per_layer(r.ansatz, r.n_qubits)
        assert r.theta.shape[-1] == r.layers * ppl
        assert 1 <= r.layers <= 2 * r.n_qubits
        if r.kind == "qfim":
            assert r.theta.shape[-1] <= 128
        if r.kind == "fidelity":
            assert r.theta.shape[0] == 2
        assert np.all((r.theta >= 0) & (r.theta < 2 * np.pi))
    kinds = [r.kind for r in a]
    for k, p in zip(serve.KINDS, (0.4, 0.3, 0.2, 0.1)):
        assert abs(kinds.count(k) / len(kinds) - p) < 0.08


def _req(rid, kind, N, ansatz="he", L=2, t=0.0):
    ppl = serve.params_per_layer(ansatz, N)
    th = np.zeros((2, L * ppl)) if kind == "fidelity" else np.zeros(L * ppl)
    return serve.Request(rid, kind, N, ansatz, L, th, t)


def test_take_batch_groups_one_family_in_arrival_order():
    q = deque([_req(0, "mw", 8), _req(1, "mw", 10), _req(2, "fidelity", 8), _req(3, "energy", 8, "tfim"),
               _req(4, "energy", 8)])
    take = serve.take_batch(q, 1 << 40, 256, 1 << 40)
    assert [r.rid for r in take] == [0, 2, 4]
    assert [r.rid for r in q] == [1, 3]
    take = serve.take_batch(q, 1 << 40, 256, 1 << 40)
    assert [r.rid for r in take] == [1] and [r.rid for r in q] == [3]


def test_take_batch_respects_rows_and_memory():
    q = deque([_req(i, "fidelity", 10) for i in range(10)])
    take = serve.take_batch(q, 1 << 40, 7, 1 << 40)  # 2 rows per fidelity request
    assert len(take) == 3 and len(q) == 7
    one = serve.request_bytes(q[0])
    take = serve.take_batch(q, 2 * one, 256, 1 << 40)
    assert len(take) == 2
    # a head that does not fit the free memory is not taken (it waits for memory)
    take = serve.take_batch(q, one - 1, 256, 1 << 40)
    assert take == [] and len(q) == 5


def test_request_bytes_cover_the_states():
    for kind in serve.KINDS:
        r = _req(0, kind, 20, L=1)
        S = 16 << 20
        need = {"fidelity": 2 * S, "mw": S, "energy": 2 * S, "qfim": (r.theta.shape[-1] + 1) * S}[kind]
        assert serve.request_bytes(r) >= need


class _StubEvent:
    def __init__(self, ready_at):
        self.ready_at = ready_at

    def query(self):
        return time.perf_counter() >= self.ready_at


class _StubBatch:
    """Device work replaced by a fixed service time per batch (no CUDA)."""

    cost_s = 1e-3

    def __init__(self, fam, reqs, slot):
        self.reqs, self.slot = reqs, slot
        self.bytes = sum(serve.request_bytes(r) for r in reqs)

    def launch(self):
        self.event = _StubEvent(time.perf_counter() + self.cost_s)

    def results(self):
        return {r.rid: 0.0 for r in self.reqs}


class _StubMulti(_StubBatch):
    def __init__(self, families, reqs, slot):
        super().__init__(None, reqs, slot)


class _StubFamilies:
    def get(self, ansatz, N):
        return (ansatz, N)


def test_admission_keeps_up_with_the_arrival_rate_when_device_work_is_stubbed():
    # the host loop alone (polling, admission, batching, result hand-off) at 4000 requests/s: every request is
    # served and the queue does not grow
    rate, n = 4000.0, 2000
    reqs = serve.synthetic_stream(n, rate, seed=5)
    srv = serve.Server(hbm_budget=1 << 40, max_rows=256, slots=[(i, None) for i in range(4)], batch_cls=_StubBatch,
                       families=_StubFamilies(), multi_cls=_StubMulti)
    t0 = time.perf_counter()
    res = srv.run(reqs, realtime=True)
    s = serve.latency_summary(res, time.perf_counter() - t0)
    assert sorted(res) == [r.rid for r in reqs]
    assert s["requests_per_s"] > 0.8 * rate
    assert s["p50_ms"] < 10.0 and s["p99_ms"] < 50.0


def test_take_small_batch_mixes_small_families_and_leaves_the_rest():
    q = deque([_req(0, "mw", 8), _req(1, "fidelity", 10, "tfim"), _req(2, "energy", 8), _req(3, "mw", 16),
               _req(4, "fidelity", 13), _req(5, "qfim", 6)])
    take = serve.take_small_batch(q, 1 << 40, 256, 1 << 40, 13)
    assert [r.rid for r in take] == [0, 1, 4]
    assert [r.rid for r in q] == [2, 3, 5]
    q = deque([_req(i, "fidelity", 9) for i in range(6)])
    assert len(serve.take_small_batch(q, 1 << 40, 5, 1 << 40, 13)) == 2 and len(q) == 4  # 2 rows each
