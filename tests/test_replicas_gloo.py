"""Replica sharding and result combination with two gloo ranks on CPU.

Each rank evaluates its shard of parameter rows with the oracle (the compute
stands in for the GPU kernels; the logic under test is the sharding and the
reductions), then the combined results must equal a single-process run.
"""
import os
import socket

import numpy as np
import torch
import torch.distributed as dist
import torch.multiprocessing as mp

from pyramaterised_gb300.replicas import gather_rows, max_over_ranks, mean_std, shard_rows, sum_counts


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, total, q):
    import sys

    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    from oracle import measures_oracle as MO
    from oracle import pqc_oracle as O
    import pyramaterised_gb300 as pq

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        c = pq.templates.hardware_efficient_ladder(4, 2)
        th = np.random.default_rng(0).random((total, c.n_columns())) * 2 * np.pi
        start, count = shard_rows(total, world, rank)
        states = O.run_batch(c.gates, 4, th[start:start + count])
        Q = torch.tensor([MO.single_Q(s, 4) for s in states], dtype=torch.float64)
        F = MO.pair_fidelities(states)
        counts = torch.from_numpy(np.histogram(F, bins=10, range=(0, 1))[0].astype(np.int64))
        allQ = gather_rows(Q, total)
        m, s = mean_std(Q)
        tot = sum_counts(counts)
        mx = max_over_ranks(float(rank + 1))
        q.put((rank, allQ.numpy(), m, s, tot.numpy(), mx))
    finally:
        dist.destroy_process_group()


def test_shard_rows_partitions_exactly():
    for total in (0, 1, 7, 256, 1001):
        for world in (1, 2, 3, 8):
            spans = [shard_rows(total, world, r) for r in range(world)]
            assert sum(c for _, c in spans) == total
            assert all(spans[r][0] + spans[r][1] == spans[r + 1][0] for r in range(world - 1))


def test_two_gloo_ranks_combine_like_one_process():
    from oracle import measures_oracle as MO
    from oracle import pqc_oracle as O
    import pyramaterised_gb300 as pq

    total, world = 9, 2
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, world, port, total, q)) for r in range(world)]
    for p in procs:
        p.start()
    res = [q.get(timeout=120) for _ in range(world)]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    c = pq.templates.hardware_efficient_ladder(4, 2)
    th = np.random.default_rng(0).random((total, c.n_columns())) * 2 * np.pi
    states = O.run_batch(c.gates, 4, th)
    Q = np.array([MO.single_Q(s, 4) for s in states])
    counts = np.zeros(10, dtype=np.int64)
    for r in range(world):
        start, cnt = shard_rows(total, world, r)
        counts += np.histogram(MO.pair_fidelities(states[start:start + cnt]), bins=10, range=(0, 1))[0]
    for rank, allQ, m, s, tot, mx in res:
        np.testing.assert_allclose(allQ, Q, atol=1e-14)
        assert abs(m - Q.mean()) < 1e-14 and abs(s - Q.std()) < 1e-12
        np.testing.assert_array_equal(tot, counts)
        assert mx == 2.0
