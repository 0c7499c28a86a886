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


def test_rank_index_splits_an_index_file(tmp_path):
    """Each rank's index lists its share; together they list every ligand once, and a
    world of one is the whole index in order."""
    import json

    paths = []
    for k, n in enumerate((12, 40, 25, 33, 8, 51)):
        p = tmp_path / ("lig%d.json" % k)
        json.dump({"xyz": [[[0.0, 0.0, 0.0]] * n] * (1 + k % 3)}, open(p, "w"))
        paths.append(str(p))
    index = tmp_path / "index.txt"
    index.write_text("\n".join(paths[:3] + ["", str(tmp_path / "missing.json")] + paths[3:]) + "\n")
    assert shard.index_lines(str(index)) == paths
    got = []
    for rank in range(2):
        out = tmp_path / ("rank%d.txt" % rank)
        n = shard.rank_index(str(index), rank, 2, str(out))
        lines = [l for l in out.read_text().split("\n") if l]
        assert len(lines) == n and lines == sorted(lines, key=paths.index)
        got += lines
    assert sorted(got) == sorted(paths)
    one = tmp_path / "one.txt"
    assert shard.rank_index(str(index), 0, 1, str(one)) == len(paths)
    assert [l for l in one.read_text().split("\n") if l] == paths


def _optimise_worker(rank, world, port, q):
    """One rank: builds the FP64 port's systems, optimises its share of the ligands'
    poses, and gathers every rank's results."""
    import numpy as np
    import torch.distributed as dist

    import oracle as O
    from pxdock_gb300 import abi, model, synth

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        units, costs = _optimise_units()
        rec = model.Receptor.from_json(synth.make_receptor(seed=0, n_heavy=200, cube=14.0, cavity=5.0))
        p = abi.lbfgs_params(max_iter=30, history=8)

        def work(u):
            lig, poses = units[u]
            port = O.PortSystem(rec, lig)
            r = port.lbfgs_batch(p, np.zeros((len(poses), 0)), poses, 1)
            port.close()
            return (r["energy"].tolist(), r["nevals"].tolist())

        local = shard.run_share(costs, rank, world, work)
        q.put((rank, sorted(local), shard.gather_results(local)))
    finally:
        dist.destroy_process_group()


def _optimise_units():
    import numpy as np

    from pxdock_gb300 import model, synth

    units = []
    for k, (h, r) in enumerate(((8, 1), (14, 3), (10, 2), (18, 4), (12, 2))):
        lig = model.Ligand.from_json(synth.make_ligand(seed=40 + k, n_heavy=h, n_rot=r, n_n=1, n_o=1))
        rng = np.random.default_rng(k)
        poses = lig.poses[0][None] + rng.normal(scale=0.3, size=(3 + k,) + lig.poses[0].shape)
        units.append((lig, poses))
    costs = [shard.unit_cost(l.n_atoms, len(p), 30.0) for l, p in units]
    return units, costs


def test_two_rank_sharded_optimisation_gloo():
    """Two gloo ranks optimise their shares of five ligands' poses on the FP64 port; the
    gathered union covers every ligand once and equals a single-rank run."""
    import socket

    import numpy as np
    import torch.multiprocessing as mp

    import oracle as O
    from pxdock_gb300 import abi, model, synth

    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        port = s.getsockname()[1]
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=_optimise_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = sorted(q.get(timeout=300) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    units, costs = _optimise_units()
    assert sorted(out[0][1] + out[1][1]) == list(range(len(units)))
    assert out[0][2] == out[1][2] and sorted(out[0][2]) == list(range(len(units)))
    rec = model.Receptor.from_json(synth.make_receptor(seed=0, n_heavy=200, cube=14.0, cavity=5.0))
    p = abi.lbfgs_params(max_iter=30, history=8)
    for u, (lig, poses) in enumerate(units):
        port = O.PortSystem(rec, lig)
        r = port.lbfgs_batch(p, np.zeros((len(poses), 0)), poses, 1)
        port.close()
        assert out[0][2][u] == (r["energy"].tolist(), r["nevals"].tolist())
