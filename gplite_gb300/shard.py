"""Data-parallel sharding of independent GP problems over ranks (one GPU each).

Batched problems and served requests are independent, so a job of many of
them shards with no data-path collective: every rank solves its own part on
its own GPU and the results are gathered on the host. The partition balances
the O(n^3) work of the fits greedily (largest first onto the least loaded
rank), so ranks finish at about the same time.
"""
from __future__ import annotations

import heapq

import numpy as np


def partition(sizes, world, cost=lambda n: float(n) ** 3):
    """Indices of the problems each rank solves: longest-processing-time greedy
    on cost(n). Deterministic (ties go to the lower rank / lower index)."""
    order = sorted(range(len(sizes)), key=lambda i: (-cost(sizes[i]), i))
    heap = [(0.0, r) for r in range(world)]
    parts = [[] for _ in range(world)]
    for i in order:
        load, r = heapq.heappop(heap)
        parts[r].append(i)
        heapq.heappush(heap, (load + cost(sizes[i]), r))
    return [sorted(p) for p in parts]


def solve_sharded(problems, solve, rank=None, world=None, group=None):
    """Solve `problems` (dicts with at least "y") across the ranks of the default
    process group: rank r runs solve(its problems) -> list of per-problem results,
    then the results are gathered in the original order on every rank (a host
    gather of Python objects; no collective touches the device data path)."""
    import torch.distributed as dist
    if world is None:
        world = dist.get_world_size(group) if dist.is_initialized() else 1
    if rank is None:
        rank = dist.get_rank(group) if dist.is_initialized() else 0
    parts = partition([len(p["y"]) for p in problems], world)
    mine = parts[rank]
    local = solve([problems[i] for i in mine]) if mine else []
    if world == 1:
        return list(local)
    gathered = [None] * world
    dist.all_gather_object(gathered, (mine, list(local)), group=group)
    out = [None] * len(problems)
    for idx, res in gathered:
        for i, r in zip(idx, res):
            out[i] = r
    return out


def balance(parts, sizes, cost=lambda n: float(n) ** 3):
    """Largest / mean per-rank cost of a partition (1.0 = perfectly balanced)."""
    loads = np.array([sum(cost(sizes[i]) for i in p) for p in parts])
    return float(loads.max() / max(loads.mean(), 1e-300))
