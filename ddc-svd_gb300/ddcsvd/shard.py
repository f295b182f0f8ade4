"""Replicas across GPUs: cost-balanced partition of a batch and the job-level
timing reduction used under torchrun (one process per GPU).

The single-matrix SVD does not shard (every column step of the
bidiagonalisation needs the whole trailing block), so several GPUs run
independent replicas.  A batch of independent problems partitions with no
exchange: problems go to ranks by longest-processing-time assignment on
their cost m n^2 (the flop count of the SVD up to a constant), so that every
rank gets about the same work.
"""
from __future__ import annotations

import heapq

import numpy as np


def problem_cost(m: int, n: int) -> float:
    """Relative cost of one SVD: 8 m n^2 - 4/3 n^3 for m >= n (either orientation)."""
    a, b = (m, n) if m >= n else (n, m)
    return 8.0 * a * b * b - 4.0 / 3.0 * b ** 3


def shard_batch(shapes, world: int, rank: int) -> list[int]:
    """Indices of the problems (in their original order) that rank `rank` of
    `world` processes.  Deterministic: every rank computes the same partition."""
    if world <= 1:
        return list(range(len(shapes)))
    costs = np.array([problem_cost(int(m), int(n)) for m, n in shapes])
    order = np.argsort(-costs, kind="stable")
    heap = [(0.0, r) for r in range(world)]
    owner = np.empty(len(shapes), dtype=np.int64)
    for i in order:
        load, r = heapq.heappop(heap)
        owner[i] = r
        heapq.heappush(heap, (load + costs[i], r))
    return [int(i) for i in np.nonzero(owner == rank)[0]]


def job_time_ms(local_ms: float, dist=None, device=None) -> float:
    """Job-level time of a step run on every rank: the maximum over ranks
    (all_reduce MAX); the local time when not distributed."""
    if dist is None or not dist.is_available() or not dist.is_initialized() or dist.get_world_size() == 1:
        return float(local_ms)
    import torch
    t = torch.tensor([float(local_ms)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())
