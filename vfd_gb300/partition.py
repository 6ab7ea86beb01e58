"""Batches of independent scenes across GPUs: one rank per GPU, no exchange in the step.

Scenes of a batch share nothing, so a batch shards across ranks by scene: each rank
advances its own sub-batch (vfd_create_batch) and the ranks meet only to gather the
per-scene statistics on the host. The scenes are assigned by cost, largest first, each
to the rank with the smallest total so far (LPT greedy); the cost of a scene is its
particle count, optionally weighted by its expected solver work.
"""
from __future__ import annotations

import heapq


def assign(costs, ranks: int) -> list[list[int]]:
    """Scene indices per rank: LPT greedy on `costs`, deterministic (ties by index)."""
    if ranks < 1:
        raise ValueError("ranks must be positive")
    order = sorted(range(len(costs)), key=lambda i: (-float(costs[i]), i))
    heap = [(0.0, r) for r in range(ranks)]
    heapq.heapify(heap)
    out: list[list[int]] = [[] for _ in range(ranks)]
    for i in order:
        load, r = heapq.heappop(heap)
        out[r].append(i)
        heapq.heappush(heap, (load + float(costs[i]), r))
    for lst in out:
        lst.sort()
    return out


def imbalance(costs, parts) -> float:
    """max rank load / mean rank load (1.0 = perfect balance)."""
    loads = [sum(float(costs[i]) for i in p) for p in parts]
    mean = sum(loads) / len(loads)
    return max(loads) / mean if mean > 0 else 1.0


def local_scenes(scene_list, rank: int, world: int, costs=None):
    """(indices, scenes) of this rank's share of `scene_list`."""
    if costs is None:
        costs = [len(s["x"]) for s in scene_list]
    idx = assign(costs, world)[rank]
    return idx, [scene_list[i] for i in idx]


def gather_scene_stats(local_idx, local_stats, world: int, group=None) -> dict:
    """{scene index: stats} of every rank, on every rank (torch.distributed object gather;
    the host-side exchange of the batch, no device collective)."""
    mine = dict(zip(local_idx, local_stats))
    if world == 1:
        return mine
    import torch.distributed as dist
    parts = [None] * world
    dist.all_gather_object(parts, mine, group=group)
    out = {}
    for p in parts:
        out.update(p)
    return out
