"""Sharding of independent hole-filling problems across ranks (one GPU each).

Every image (and every channel of it) is an independent problem, so N GPUs
need no collective on the data path: each rank solves its own shard and the
results stay where they were computed.  The only communication is host-side
bookkeeping: the max-over-ranks step time, and gathering per-rank reports.

``partition`` balances shards by the number of unknown samples (the work of a
converged solve is close to linear in it): longest-processing-time first, each
problem to the currently lightest rank, ties to the lowest rank, so every rank
computes the same assignment without exchanging anything.
"""
from __future__ import annotations

import heapq


def partition(weights, world: int):
    """Indices of `weights` for each of `world` ranks (deterministic LPT)."""
    if world < 1:
        raise ValueError("world must be >= 1")
    order = sorted(range(len(weights)), key=lambda k: (-weights[k], k))
    heap = [(0.0, r) for r in range(world)]
    heapq.heapify(heap)
    shards = [[] for _ in range(world)]
    for k in order:
        load, r = heapq.heappop(heap)
        shards[r].append(k)
        heapq.heappush(heap, (load + float(weights[k]), r))
    return [sorted(s) for s in shards]


def shard(items, weights, rank: int, world: int):
    """The items of `rank`."""
    return [items[k] for k in partition(weights, world)[rank]]


def imbalance(weights, shards) -> float:
    """max shard load / mean shard load (1.0 = perfect)."""
    loads = [sum(weights[k] for k in s) for s in shards]
    mean = sum(loads) / max(1, len(loads))
    return max(loads) / mean if mean > 0 else 1.0


def max_over_ranks(value: float, device=None) -> float:
    """Max of a per-rank float over the default process group (identity when
    torch.distributed is not initialised)."""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()):
        return float(value)
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def sum_over_ranks(value: float, device=None) -> float:
    """Sum of a per-rank float over the default process group."""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()):
        return float(value)
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.SUM)
    return float(t.item())


def gather_to_root(obj, root: int = 0):
    """Per-rank Python objects, as a list on `root` (None elsewhere)."""
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()):
        return [obj]
    out = [None] * dist.get_world_size() if dist.get_rank() == root else None
    dist.gather_object(obj, out, dst=root)
    return out
