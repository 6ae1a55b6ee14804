"""Partitioning independent t-SNE systems over ranks (one process per GPU).

A batch of embeddings has no exchange step: every system's P matrix, tree and
embedding live on one GPU, so ranks split the systems and never talk during a
step.  The split balances particle counts (longest-processing-time greedy:
largest system first, each to the least-loaded rank; ties to the lower rank),
which is deterministic, so every rank computes the same assignment without a
collective.  The only collectives are outside the data path: a barrier before
timing and a MAX of the ranks' elapsed times after it.
"""
from __future__ import annotations

import heapq

import numpy as np


def assign(sizes, world: int) -> list[list[int]]:
    """Per rank, the indices (ascending) of the systems it owns."""
    if world < 1:
        raise ValueError("world must be >= 1")
    sizes = np.asarray(sizes, dtype=np.int64)
    if sizes.ndim != 1 or (sizes < 0).any():
        raise ValueError("sizes must be a 1-D array of non-negative counts")
    order = sorted(range(len(sizes)), key=lambda i: (-int(sizes[i]), i))
    heap = [(0, r) for r in range(world)]
    owned: list[list[int]] = [[] for _ in range(world)]
    for i in order:
        load, r = heapq.heappop(heap)
        owned[r].append(i)
        heapq.heappush(heap, (load + int(sizes[i]), r))
    return [sorted(o) for o in owned]


def shard(sizes, rank: int, world: int) -> list[int]:
    """The indices of the systems rank `rank` of `world` owns."""
    if not 0 <= rank < world:
        raise ValueError("rank out of range")
    return assign(sizes, world)[rank]


def max_over_ranks(seconds: float, device=None) -> float:
    """The largest of the ranks' elapsed times (the job's time); the value
    itself when torch.distributed is not initialised."""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return float(seconds)
    t = torch.tensor([float(seconds)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def sum_over_ranks(count: int, device=None) -> int:
    """The sum of a per-rank count (particles processed by the whole job)."""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return int(count)
    t = torch.tensor([int(count)], dtype=torch.int64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.SUM)
    return int(t.item())
