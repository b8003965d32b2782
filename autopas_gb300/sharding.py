"""Distribution of independent systems over ranks, and the rank helpers bench.py uses.

An ensemble of independent systems shards with no data-path collective: every rank steps its own systems in
its own engine on its own GPU.  Systems are assigned by longest-processing-time-first bin packing on an
estimate of their pair work (particles x density x interaction volume), which keeps the slowest rank within
4/3 of the optimum.  Only the per-rank totals (time, pair counts) are combined, on the host.
"""
from __future__ import annotations

import heapq
import math


def pair_work(num_particles: int, density: float, interaction_length: float) -> float:
    """Estimated interacting-pair evaluations of one system per force call (full lists)."""
    return num_particles * density * 4.0 / 3.0 * math.pi * interaction_length ** 3


def lpt_assign(costs, world_size: int):
    """Longest-processing-time-first assignment.  Returns (systems per rank, load per rank)."""
    ranks = [[] for _ in range(world_size)]
    heap = [(0.0, r) for r in range(world_size)]
    heapq.heapify(heap)
    for idx in sorted(range(len(costs)), key=lambda k: (-costs[k], k)):
        load, r = heapq.heappop(heap)
        ranks[r].append(idx)
        heapq.heappush(heap, (load + costs[idx], r))
    loads = [0.0] * world_size
    for r, idxs in enumerate(ranks):
        loads[r] = sum(costs[k] for k in idxs)
        idxs.sort()
    return ranks, loads


def barrier(pg):
    if pg is not None:
        pg.barrier()


def max_over_ranks(pg, value: float) -> float:
    if pg is None:
        return value
    import torch
    t = torch.tensor([value], dtype=torch.float64)
    pg.all_reduce(t, op=pg.ReduceOp.MAX)
    return float(t.item())


def sum_over_ranks(pg, value: float) -> float:
    if pg is None:
        return value
    import torch
    t = torch.tensor([value], dtype=torch.float64)
    pg.all_reduce(t, op=pg.ReduceOp.SUM)
    return float(t.item())
