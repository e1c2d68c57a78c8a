"""Sharding the independent systems of a batch over ranks (one process per GPU).

Independent triangles shard with no exchange during the solve: each rank
analyses its own subset as one batch (one persistent launch per solve) and
solves it alone. Systems are assigned by greedy longest-first bin packing on a
per-system cost (stored entries by default), which is deterministic, so every
rank derives the same map without communicating. The only collective is the
host-side gather of per-rank solutions at the end (``gather_solutions``).

A single system does not shard: its dependency chain would need fine-grained
cross-GPU synchronisation. Those runs are replicas. Its right-hand sides do:
with many columns, every rank holds the same triangle and analysis and solves a
contiguous slice of the columns (``rhs_columns``); ``gather_columns`` joins the
slices afterwards.
"""
from __future__ import annotations

import heapq

import numpy as np


def assign(weights, world: int) -> list[list[int]]:
    """Greedy longest-processing-time assignment of systems to ``world`` ranks.

    Systems are taken by decreasing weight (ties: lower index first) and each
    goes to the currently lightest rank (ties: lower rank). Returns, per rank,
    the ascending list of system indices it owns. The heaviest rank carries at
    most mean load + the largest single weight."""
    if world < 1:
        raise ValueError("world must be >= 1")
    w = np.asarray(weights, dtype=np.int64)
    if w.ndim != 1 or (w.size and w.min() < 0):
        raise ValueError("weights must be a 1-D array of non-negative costs")
    order = sorted(range(w.size), key=lambda i: (-int(w[i]), i))
    heap = [(0, r) for r in range(world)]
    owned: list[list[int]] = [[] for _ in range(world)]
    for i in order:
        load, r = heapq.heappop(heap)
        owned[r].append(i)
        heapq.heappush(heap, (load + int(w[i]), r))
    return [sorted(o) for o in owned]


def shard_of(weights, world: int, rank: int) -> list[int]:
    """System indices owned by ``rank`` under ``assign``."""
    if not 0 <= rank < world:
        raise ValueError("rank out of range")
    return assign(weights, world)[rank]


def loads(weights, world: int) -> list[int]:
    """Total weight per rank under ``assign``."""
    w = np.asarray(weights, dtype=np.int64)
    return [int(w[o].sum()) if o else 0 for o in assign(w, world)]


def gather_solutions(local: dict[int, np.ndarray], count: int, group=None) -> list[np.ndarray] | None:
    """Collects every rank's {system index: solution} on all ranks
    (``torch.distributed.all_gather_object``; host memory, after the timed
    region). Returns the solutions ordered by system index, and checks that
    every system was solved by exactly one rank."""
    import torch.distributed as dist
    world = dist.get_world_size(group)
    parts: list = [None] * world
    dist.all_gather_object(parts, {int(k): np.asarray(v) for k, v in local.items()}, group=group)
    out: list = [None] * count
    for part in parts:
        for k, v in part.items():
            if not 0 <= k < count or out[k] is not None:
                raise RuntimeError(f"system {k} solved by more than one rank or out of range")
            out[k] = v
    missing = [k for k, v in enumerate(out) if v is None]
    if missing:
        raise RuntimeError(f"systems not solved by any rank: {missing[:8]}")
    return out


def rhs_columns(rhs: int, world: int, rank: int) -> tuple[int, int]:
    """Contiguous slice [start, stop) of ``rhs`` right-hand-side columns owned
    by ``rank``: the first ``rhs % world`` ranks take one column more, so slice
    widths differ by at most one. A rank may own no column (start == stop)."""
    if world < 1 or not 0 <= rank < world:
        raise ValueError("rank out of range")
    if rhs < 0:
        raise ValueError("rhs must be >= 0")
    base, extra = divmod(rhs, world)
    start = rank * base + min(rank, extra)
    return start, start + base + (1 if rank < extra else 0)


def gather_columns(local: np.ndarray, rhs: int, group=None) -> np.ndarray:
    """Joins every rank's n x (its ``rhs_columns`` width) block into the
    n x rhs solution on all ranks (host memory, after the timed region).
    Checks that each rank's block has the width its slice asks for."""
    import torch.distributed as dist
    world = dist.get_world_size(group)
    rank = dist.get_rank(group)
    local = np.asarray(local)
    if local.ndim != 2:
        raise ValueError("local block must be n x width")
    parts: list = [None] * world
    dist.all_gather_object(parts, (rank, local), group=group)
    n = local.shape[0]
    out = np.empty((n, rhs), dtype=local.dtype)
    for r, blk in parts:
        a, b = rhs_columns(rhs, world, r)
        if blk.shape != (n, b - a):
            raise RuntimeError(f"rank {r} returned a block of shape {blk.shape}, expected {(n, b - a)}")
        out[:, a:b] = blk
    return out
