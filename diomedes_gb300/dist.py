"""Multi-rank helpers: one process per GPU, scenes sharded across ranks.

Scenes are independent, so ranks share no data while stepping; the only
communication is the timing frame (a barrier, the max of the ranks'
elapsed times) and the totals of the work done.  A single large scene is
not split across GPUs.
"""
import heapq

import numpy as np


def shard_scenes(costs, world_size):
    """Longest-processing-time assignment of scenes to ranks.

    `costs` are per-scene work estimates (bodies + rows); returns, per rank,
    the sorted list of scene indices it owns.  Deterministic: ties go to the
    lowest rank and, within equal costs, to the lowest scene index."""
    order = sorted(range(len(costs)), key=lambda s: (-float(costs[s]), s))
    heap = [(0.0, r) for r in range(world_size)]
    heapq.heapify(heap)
    owned = [[] for _ in range(world_size)]
    for s in order:
        load, r = heapq.heappop(heap)
        owned[r].append(s)
        heapq.heappush(heap, (load + float(costs[s]), r))
    return [sorted(o) for o in owned]


def scene_costs(scene_offsets, constraints=None):
    """Per-scene cost estimate: bodies plus joints."""
    off = np.asarray(scene_offsets, np.int64)
    cost = np.diff(off).astype(np.float64)
    if constraints is not None and len(constraints):
        s = np.searchsorted(off, np.asarray(constraints["a"], np.int64), side="right") - 1
        cost += np.bincount(s, minlength=len(cost))[: len(cost)]
    return cost


def frame(dist, elapsed_ms, units, device=None):
    """Max elapsed time and summed units over ranks (torch.distributed)."""
    import torch

    t = torch.tensor([float(elapsed_ms)], dtype=torch.float64, device=device)
    u = torch.tensor([float(units)], dtype=torch.float64, device=device)
    if dist is not None and dist.is_initialized():
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        dist.all_reduce(u, op=dist.ReduceOp.SUM)
    return float(t.item()), float(u.item())
