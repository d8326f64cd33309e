"""Instance sharding of the batched workloads across ranks (one GPU each).

Independent cavity instances need no exchange: every rank solves its own
share, and only per-instance statistics are gathered at the end. Shares are
balanced by estimated cost (nodes per instance) with the longest-processing-
time rule: instances in decreasing cost order, each to the currently lightest
rank (ties to the lowest rank), so every rank computes the same partition.
"""
from __future__ import annotations

import numpy as np


def shard_instances(costs, world: int) -> list[np.ndarray]:
    """Per-rank sorted instance indices of a cost-balanced partition."""
    costs = np.asarray(costs, dtype=np.float64)
    if world < 1:
        raise ValueError("world size must be >= 1")
    order = np.argsort(-costs, kind="stable")
    load = np.zeros(world)
    parts = [[] for _ in range(world)]
    for i in order:
        r = int(np.argmin(load))
        parts[r].append(int(i))
        load[r] += costs[i]
    return [np.array(sorted(p), dtype=np.int64) for p in parts]


def gather_results(results: list[dict], indices: np.ndarray, n_total: int, group=None) -> list[dict]:
    """All ranks' per-instance results in global instance order (torch.distributed
    all_gather_object over the default or given group)."""
    import torch.distributed as dist

    mine = list(zip(indices.tolist(), results))
    world = dist.get_world_size(group)
    parts = [None] * world
    dist.all_gather_object(parts, mine, group=group)
    out = [None] * n_total
    for part in parts:
        for i, r in part:
            out[i] = r
    return out
