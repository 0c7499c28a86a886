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
