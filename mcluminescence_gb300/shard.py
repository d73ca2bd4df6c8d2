"""Sharding of a batch of parameter sets over ranks (one process per GPU).

Parameter sets are independent and every random draw is keyed by the set's
``set_id`` (Philox counter word 2), so splitting a batch over ranks changes
nothing in the results: each rank simulates its share with the ordinary
single-GPU call and the per-set curves are concatenated on the host.  There
is no collective on the data path; the only exchange is the host-side gather
of finished per-set results (``torch.distributed`` object collectives, which
run over gloo or NCCL alike).

The reference runs parameter sets one after another in one process
(src/class/simulate.py:36-48) and parallelises the optimizer's population over
processes (src/class/optimizer.py:104-111); this module is the multi-GPU
counterpart of both.
"""
from __future__ import annotations

import heapq
from typing import Callable, List, Optional, Sequence

import numpy as np

from .batch import BatchResult
from .schedule import SetSpec


def shard_indices(weights: Sequence[float], world: int) -> List[List[int]]:
    """Split items with the given costs into ``world`` shards, longest first
    onto the least-loaded shard (LPT).  Deterministic: ties go to the lower
    rank, and each shard lists its items in ascending index order."""
    if world < 1:
        raise ValueError("world must be >= 1")
    order = sorted(range(len(weights)), key=lambda i: (-float(weights[i]), i))
    heap = [(0.0, r) for r in range(world)]
    heapq.heapify(heap)
    shards: List[List[int]] = [[] for _ in range(world)]
    for i in order:
        load, r = heapq.heappop(heap)
        shards[r].append(i)
        heapq.heappush(heap, (load + float(weights[i]), r))
    return [sorted(s) for s in shards]


def shard_for_rank(specs: Sequence[SetSpec], rank: int, world: int) -> List[int]:
    """Indices of the sets rank ``rank`` simulates (balanced by trials)."""
    if not 0 <= rank < world:
        raise ValueError(f"rank {rank} outside world of {world}")
    return shard_indices([max(s.trials, 1) for s in specs], world)[rank]


def assemble(specs: Sequence[SetSpec], parts) -> BatchResult:
    """Rebuild one BatchResult in the original set order from per-rank parts;
    ``parts`` is a list of ``(indices, lum_list, alive_list, fates_list)``
    with one array per set (alive/fates lists may be None)."""
    n = len(specs)
    lum = [None] * n
    alive = [None] * n
    fates = [None] * n
    have_alive = have_fates = True
    for idx, l, a, f in parts:
        for k, i in enumerate(idx):
            if lum[i] is not None:
                raise ValueError(f"set {i} simulated by two ranks")
            lum[i] = np.asarray(l[k])
            alive[i] = None if a is None else np.asarray(a[k])
            fates[i] = None if f is None else np.asarray(f[k])
        if len(idx):
            have_alive &= a is not None
            have_fates &= f is not None
    missing = [i for i in range(n) if lum[i] is None]
    if missing:
        raise ValueError(f"sets {missing[:5]} not simulated by any rank")
    for i, s in enumerate(specs):
        if lum[i].size != s.n_bins:
            raise ValueError(f"set {i}: {lum[i].size} bins, expected {s.n_bins}")
    b_off = np.concatenate([[0], np.cumsum([s.n_bins for s in specs])]).astype(np.int64)
    s_off = np.concatenate([[0], np.cumsum([s.n_slots for s in specs])]).astype(np.int64)
    cat = lambda xs, dt: np.concatenate(xs).astype(dt) if xs else np.zeros(0, dt)
    return BatchResult(cat(lum, np.uint32),
                       cat(alive, np.uint32) if have_alive else None,
                       cat(fates, np.int32) if have_fates else None,
                       b_off, s_off)


def _split(res: BatchResult, k: int):
    lum = [res.lum_of(i).copy() for i in range(k)]
    alive = [res.alive_of(i).copy() for i in range(k)] if res.alive is not None else None
    fates = [res.fates_of(i).copy() for i in range(k)] if res.fates is not None else None
    return lum, alive, fates


def run_sharded(specs: Sequence[SetSpec], runner: Callable[[List[SetSpec]], BatchResult],
                group=None, rank: Optional[int] = None, world: Optional[int] = None) -> BatchResult:
    """Simulate ``specs`` over all ranks of ``group`` and return the whole
    batch's result on every rank.  ``runner`` simulates a list of sets on this
    rank (``simulate_batch`` with fixed keyword arguments, for instance)."""
    import torch.distributed as dist
    if world is None:
        world = dist.get_world_size(group) if dist.is_initialized() else 1
    if rank is None:
        rank = dist.get_rank(group) if dist.is_initialized() else 0
    mine = shard_for_rank(specs, rank, world)
    local = [specs[i] for i in mine]
    if local:
        lum, alive, fates = _split(runner(local), len(local))
    else:
        lum, alive, fates = [], None, None
    part = (mine, lum, alive, fates)
    if world == 1:
        return assemble(specs, [part])
    parts = [None] * world
    dist.all_gather_object(parts, part, group=group)
    return assemble(specs, parts)


def simulate_batch_sharded(specs: Sequence[SetSpec], group=None, **kw) -> BatchResult:
    """``simulate_batch`` over all ranks of an initialised process group (one
    GPU per rank); every rank gets the full result."""
    from .batch import simulate_batch
    return run_sharded(specs, lambda local: simulate_batch(local, **kw), group=group)
