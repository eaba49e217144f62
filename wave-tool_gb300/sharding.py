"""Multi-rank layout of the path (one process per GPU).

Patches are independent, so the forward shards with no collective on the
data path: `shard_patches` assigns patches to ranks by longest-processing-time
on their term counts (vertices x waves) and rebases each rank's output offsets.
When ranks share one wave set, the adjoint's per-rank wave gradients are
summed with `allreduce_grads_fixed_order` — gathered and added in rank order,
so every rank gets the same bits whatever the arrival order.
No reference counterpart: the reference renders one grid on one GPU.
"""
from __future__ import annotations

import heapq

import numpy as np

from .abi import PATCH_DTYPE, patch_vertices


def shard_patches(patches: np.ndarray, world_size: int, rank: int) -> tuple[np.ndarray, np.ndarray]:
    """Patches of `rank` (LPT on vertices x waves, ties by index) with
    out_offset rebased to a dense per-rank output; also returns their indices
    in the input table."""
    assert patches.dtype == PATCH_DTYPE and 0 <= rank < world_size
    cost = patch_vertices(patches) * np.maximum(patches["wave_count"].astype(np.uint64), 1)
    order = sorted(range(len(patches)), key=lambda i: (-int(cost[i]), i))
    heap = [(0, r) for r in range(world_size)]
    owner = np.empty(len(patches), np.int64)
    for i in order:
        load, r = heapq.heappop(heap)
        owner[i] = r
        heapq.heappush(heap, (load + int(cost[i]), r))
    idx = np.flatnonzero(owner == rank)
    mine = patches[idx].copy()
    off = 0
    for p in mine:
        p["out_offset"] = off
        off += int(p["cols"]) * int(p["rows"])
    return mine, idx


def allreduce_grads_fixed_order(grad, group=None):
    """Sum a per-rank gradient tensor over ranks in rank order (deterministic).
    Works on any torch.distributed backend (gloo on CPU, NCCL on GPU)."""
    import torch
    import torch.distributed as dist
    world = dist.get_world_size(group)
    parts = [torch.empty_like(grad) for _ in range(world)]
    dist.all_gather(parts, grad.contiguous(), group=group)
    out = parts[0].clone()
    for t in parts[1:]:
        out += t
    return out
