"""Replica parallelism across GPUs: one process per GPU, independent batches.

The path shards naturally (parameter rows, states, QFIM instances and
requests are independent), so N GPUs run N independent batches and only the
small results are combined: histogram counts are summed, Meyer-Wallach
statistics are combined from per-rank sums, and per-row results are
gathered.  There is no data-path collective.  Works with any
torch.distributed backend (nccl on GPUs, gloo in CPU tests).
"""
import torch
import torch.distributed as dist


def shard_rows(total, world, rank):
    """Contiguous [start, start + count) block of `total` rows for `rank` (sizes differ by at most one)."""
    base, extra = divmod(int(total), int(world))
    start = rank * base + min(rank, extra)
    return start, base + (1 if rank < extra else 0)


def _world():
    return dist.get_world_size() if dist.is_available() and dist.is_initialized() else 1


def sum_counts(counts):
    """Element-wise sum of int64 histogram counts over ranks."""
    c = counts.clone()
    if _world() > 1:
        dist.all_reduce(c, op=dist.ReduceOp.SUM)
    return c


def mean_std(values):
    """Population mean and std (np.std semantics) of per-row values spread over ranks."""
    v = values.to(torch.float64)
    s = torch.stack([torch.tensor(float(v.numel()), dtype=torch.float64, device=v.device), v.sum(),
                     (v * v).sum()])
    if _world() > 1:
        dist.all_reduce(s, op=dist.ReduceOp.SUM)
    n, a, b = s[0], s[1], s[2]
    mean = a / n
    var = torch.clamp(b / n - mean * mean, min=0.0)
    return float(mean), float(torch.sqrt(var))


def gather_rows(values, total):
    """All ranks' row results in global row order (rows sharded with `shard_rows`)."""
    world = _world()
    if world == 1:
        return values
    counts = [shard_rows(total, world, r)[1] for r in range(world)]
    width = max(counts)
    pad = torch.zeros((width,) + tuple(values.shape[1:]), dtype=values.dtype, device=values.device)
    pad[: values.shape[0]] = values
    out = [torch.empty_like(pad) for _ in range(world)]
    dist.all_gather(out, pad)
    return torch.cat([o[:c] for o, c in zip(out, counts)])


def max_over_ranks(x):
    t = torch.tensor([float(x)], dtype=torch.float64)
    if _world() > 1:
        if dist.get_backend() == "nccl":
            t = t.cuda()
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())
