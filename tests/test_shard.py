"""Replica sharding across ranks (sgx/shard.py), on CPU: the ranges of a
world partition the cells, and the timing reduction returns the slowest
rank's value on every rank, checked with two gloo ranks."""
import os
import socket

import pytest

from sgx.shard import max_over_ranks, shard_range


@pytest.mark.parametrize("n,world", [(0, 1), (10, 1), (10, 3), (7, 8), (2**22 + 5, 4)])
def test_shard_ranges_partition_the_cells(n, world):
    ranges = [shard_range(n, r, world) for r in range(world)]
    assert ranges[0][0] == 0 and ranges[-1][1] == n
    for (b0, e0), (b1, e1) in zip(ranges, ranges[1:]):
        assert e0 == b1
    sizes = [e - b for b, e in ranges]
    assert max(sizes) - min(sizes) <= 1


def test_shard_range_rejects_bad_rank():
    with pytest.raises(ValueError):
        shard_range(10, 2, 2)


def _worker(rank, world, port, out):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        b, e = shard_range(1000, rank, world)
        slowest = max_over_ranks(float(rank + 1) * 0.5, world)
        out.put((rank, b, e, slowest))
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks_reduce_the_slowest_time():
    torch = pytest.importorskip("torch")
    mp = torch.multiprocessing.get_context("spawn")
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        port = s.getsockname()[1]
    q = mp.Queue()
    procs = [mp.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [r[1:3] for r in res] == [(0, 500), (500, 1000)]
    assert all(r[3] == 1.0 for r in res)
