"""Scene sharding across ranks for batches and serving pools.

Scenes are independent (no coupling between their systems), so a batch or a
serving pool splits across processes -- one per GPU -- with no exchange at
all: every rank steps its own shard and no collective runs on the data path.
The partition is deterministic and needs no communication either: every rank
computes the same assignment from the scenes' work estimates (tet counts).

Greedy longest-processing-time assignment: scenes in decreasing order of
work (ties by scene index), each to the rank with the least work so far
(ties by rank).  The most loaded rank carries at most 4/3 of the optimum
(Graham's bound), and in practice a few percent above the mean for hundreds
of uneven scenes.  A scene's result does not depend on the rank or on the
other scenes of its shard: a batch advances each scene by exactly its own
step sequence.
"""
from __future__ import annotations

import heapq

import numpy as np


def shard_scenes(work, world: int) -> list[list[int]]:
    """Scene indices per rank (each list ascending) for `world` ranks."""
    work = np.asarray(work, dtype=np.float64)
    if world < 1:
        raise ValueError("world must be >= 1")
    order = sorted(range(len(work)), key=lambda i: (-work[i], i))
    heap = [(0.0, r) for r in range(world)]
    shards: list[list[int]] = [[] for _ in range(world)]
    for i in order:
        load, r = heapq.heappop(heap)
        shards[r].append(i)
        heapq.heappush(heap, (load + float(work[i]), r))
    return [sorted(s) for s in shards]


def my_shard(work, rank: int, world: int) -> list[int]:
    """The scenes rank `rank` steps."""
    if not 0 <= rank < world:
        raise ValueError("rank out of range")
    return shard_scenes(work, world)[rank]


def imbalance(work, world: int) -> float:
    """Most loaded rank's work / the mean work per rank."""
    work = np.asarray(work, dtype=np.float64)
    loads = [work[s].sum() for s in shard_scenes(work, world)]
    return float(max(loads) / max(1e-300, work.sum() / world))
