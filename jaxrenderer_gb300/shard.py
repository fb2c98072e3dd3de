"""Scene sharding across GPUs (one process per GPU).

Scenes are independent, so a batch shards into contiguous scene ranges with
no exchange step: each rank renders its range and nothing crosses GPUs (an
optional host gather of canvases is the caller's).  Ranges are balanced by
an estimate of each scene's cost, `width * height + faces` per pass (the
tiled form's work grows with both).
"""
from __future__ import annotations

from typing import List, Sequence, Tuple

import numpy as np


def scene_costs(n_faces: Sequence[int], width: Sequence[int], height: Sequence[int],
                shadow_pixels: Sequence[int] | int = 0) -> np.ndarray:
    """Cost estimate per scene: pixels of every pass plus faces per pass."""
    f = np.asarray(n_faces, dtype=np.float64)
    px = np.asarray(width, dtype=np.float64) * np.asarray(height, dtype=np.float64)
    sp = np.broadcast_to(np.asarray(shadow_pixels, dtype=np.float64), f.shape)
    passes = np.where(sp > 0, 2.0, 1.0)
    return px + sp + passes * f


def partition(costs: Sequence[float], world: int) -> List[Tuple[int, int]]:
    """Contiguous [begin, end) ranges, one per rank, covering every scene,
    each as close as possible to total/world by cost (prefix-sum split)."""
    c = np.asarray(costs, dtype=np.float64)
    n = c.size
    if world < 1:
        raise ValueError("world must be >= 1")
    if n == 0:
        return [(0, 0)] * world
    prefix = np.concatenate([[0.0], np.cumsum(c)])
    total = prefix[-1]
    cuts = [0]
    for r in range(1, world):
        target = total * r / world
        k = int(np.searchsorted(prefix, target, side="left"))
        # pick the boundary nearer the target, keep ranges ordered
        if k > 0 and abs(prefix[k - 1] - target) <= abs(prefix[min(k, n)] - target):
            k -= 1
        cuts.append(min(max(k, cuts[-1]), n))
    cuts.append(n)
    return [(cuts[r], cuts[r + 1]) for r in range(world)]


def shard_for_rank(costs: Sequence[float], rank: int, world: int) -> Tuple[int, int]:
    return partition(costs, world)[rank]


__all__ = ["scene_costs", "partition", "shard_for_rank"]
