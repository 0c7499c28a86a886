"""Replica sharding (pxdock_gb300.shard) on CPU: a cost-balanced split that every rank
computes identically, covering each unit once; checked with world_size-2 gloo ranks
that compare their splits and the total work with collectives."""
import os

import pytest

from pxdock_gb300 import shard


def test_partition_covers_and_balances():
    costs = [shard.unit_cost(n, 256) for n in (20, 45, 60, 33, 12, 58, 41, 27, 50, 19)]
    parts = shard.partition(costs, 3)
    flat = sorted(u for p in parts for u in p)
    assert flat == list(range(len(costs)))
    loads = [sum(costs[u] for u in p) for p in parts]
    assert max(loads) - min(loads) <= max(costs)
    assert shard.partition(costs, 1) == [list(range(len(costs)))]
    assert shard.partition([], 2) == [[], []]
    with pytest.raises(ValueError):
        shard.partition(costs, 0)


def _worker(rank, world, port, costs, q):
    import torch
    import torch.distributed as dist

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    mine = shard.rank_share(costs, rank, world)
    # every rank computes the same split: gather all ranks' shares and compare
    shares = [None] * world
    dist.all_gather_object(shares, mine)
    total = torch.tensor([sum(costs[u] for u in mine)], dtype=torch.float64)
    dist.all_reduce(total)
    q.put((rank, shares, float(total.item())))
    dist.destroy_process_group()


def test_two_rank_split_gloo():
    import socket

    import torch.multiprocessing as mp

    costs = [shard.unit_cost(n, 64, 150.0) for n in range(10, 60, 3)]
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        port = s.getsockname()[1]
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, costs, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = [q.get(timeout=120) for _ in procs]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    out.sort()
    assert out[0][1] == out[1][1] == shard.partition(costs, 2)
    assert sorted(u for part in out[0][1] for u in part) == list(range(len(costs)))
    assert abs(out[0][2] - sum(costs)) < 1e-6 * sum(costs)
