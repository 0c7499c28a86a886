"""Replica sharding: one process per GPU, each with its own receptor maps, takes a
share of the independent units (ligands of an index file, or pose blocks). There is
no data-path collective; results are files or host arrays per rank.

The cost model is the evaluation cost of a unit: atoms^2 (the force-field pair terms
dominate) times the expected evaluations (poses or walkers x steps).
"""
import heapq


def unit_cost(n_atoms, n_items, evals_per_item=1.0):
    return float(n_atoms) * float(n_atoms) * float(n_items) * float(evals_per_item)


def partition(costs, world):
    """Longest-processing-time assignment of units to `world` ranks. Returns one
    ordered list of unit indices per rank; every unit appears exactly once, and the
    result depends only on the costs (every rank computes the same split)."""
    if world < 1:
        raise ValueError("world size must be >= 1")
    heap = [(0.0, r) for r in range(world)]
    out = [[] for _ in range(world)]
    for u in sorted(range(len(costs)), key=lambda i: (-costs[i], i)):
        load, r = heapq.heappop(heap)
        out[r].append(u)
        heapq.heappush(heap, (load + costs[u], r))
    return [sorted(v) for v in out]


def rank_share(costs, rank, world):
    """The units of `rank` (partition(costs, world)[rank])."""
    return partition(costs, world)[rank]


def env_rank_world():
    """(rank, world) from the torchrun environment, (0, 1) without one."""
    import os

    return int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1"))


# ------------------------------------------------------------ ligand index files
def index_lines(index_file):
    """The ligand paths an index file lists, as index_file_source::fill (source.cpp:26-44)
    takes them: every non-empty line that names an existing file, in order."""
    import os

    out = []
    with open(index_file) as f:
        for line in f.read().split("\n"):
            if line and os.path.isfile(line):
                out.append(line)
    return out


def ligand_cost(path, evals_per_pose=1.0):
    """unit_cost of one ligand file: atoms^2 x poses (the reference's ligand JSON keeps one
    [atoms][3] list per pose under "xyz")."""
    import json

    with open(path) as f:
        xyz = json.load(f).get("xyz", [[]])
    poses = max(1, len(xyz))
    atoms = len(xyz[0]) if xyz and xyz[0] else 1
    return unit_cost(atoms, poses, evals_per_pose)


def rank_index(index_file, rank, world, out_path, walkers=None):
    """Writes the ligands of `rank`'s cost-balanced share of index_file to out_path, one
    per line in index order, and returns how many there are. With `walkers` (a search),
    every ligand runs the same number of walkers, so its cost is atoms^2 x walkers."""
    paths = index_lines(index_file)
    if walkers is None:
        costs = [ligand_cost(p) for p in paths]
    else:
        costs = [ligand_cost(p) / max(1.0, _poses_of(p)) * walkers for p in paths]
    mine = rank_share(costs, rank, world)
    with open(out_path, "w") as f:
        for u in mine:
            f.write(paths[u] + "\n")
    return len(mine)


def _poses_of(path):
    import json

    with open(path) as f:
        return float(max(1, len(json.load(f).get("xyz", [[]]))))


def run_share(costs, rank, world, work):
    """Runs work(unit) for every unit of `rank`'s share and returns {unit: result}."""
    return {u: work(u) for u in rank_share(costs, rank, world)}


def gather_results(local, group=None):
    """Every rank's {unit: result} merged into one dict on every rank, over an initialised
    torch.distributed group (host objects only: no device collective). Without a group
    (world of one) the local results are returned."""
    import torch.distributed as dist

    if not dist.is_available() or not dist.is_initialized():
        return dict(local)
    parts = [None] * dist.get_world_size(group)
    dist.all_gather_object(parts, local, group=group)
    out = {}
    for p in parts:
        for k, v in p.items():
            if k in out:
                raise RuntimeError("unit %r computed by two ranks" % (k,))
            out[k] = v
    return out

