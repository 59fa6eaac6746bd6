"""Replica sharding of a closure batch across ranks (one GPU per rank).

Every cell and lookup is independent and the tables are read-only, so N
GPUs take contiguous, disjoint ranges of the cells with no data exchange;
the only collective is the reduction of the timing (the slowest rank's
time) that a benchmark reports.
"""


def shard_range(n, rank, world):
    """[begin, end) of rank's share of n cells: contiguous, disjoint,
    covering [0, n), sizes differing by at most one."""
    if world < 1 or not 0 <= rank < world:
        raise ValueError(f"rank {rank} outside world of size {world}")
    base, extra = divmod(n, world)
    begin = rank * base + min(rank, extra)
    return begin, begin + base + (1 if rank < extra else 0)


def max_over_ranks(x, world, device=None):
    """The maximum of a float over the ranks of the default process group
    (x itself when world == 1)."""
    if world == 1:
        return float(x)
    import torch
    import torch.distributed as dist
    t = torch.tensor([float(x)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())
