"""Whole-system sharding of a batched ensemble across processes (one GPU each).

The networks of an ensemble are independent, so several GPUs share an ensemble by splitting it
into whole systems: each rank steps its own sub-ensemble with the persistent batched kernel and
no data crosses between ranks during the steps. The split balances particle counts, since a
step's cost grows with the particles it moves.

Every rank computes the same assignment from the system sizes alone (no communication), so the
ranks agree on it by construction.
"""

from __future__ import annotations

import heapq

import numpy as np

from .workloads import System


def partition_systems(sizes, world: int) -> list[np.ndarray]:
    """Assigns every system to one of `world` ranks: systems in decreasing size (ties by index)
    each go to the rank holding the fewest particles so far (ties by rank). Returns, per rank,
    its system indices in increasing order.

    Longest-processing-time-first scheduling: the largest rank load exceeds the mean by at most
    the size of one system."""
    if world < 1:
        raise ValueError("world must be >= 1")
    sizes = np.asarray(sizes, np.int64)
    if sizes.ndim != 1 or (sizes < 0).any():
        raise ValueError("sizes must be a 1-D array of non-negative particle counts")
    order = sorted(range(sizes.shape[0]), key=lambda b: (-int(sizes[b]), b))
    heap = [(0, r) for r in range(world)]
    owned: list[list[int]] = [[] for _ in range(world)]
    for b in order:
        load, r = heapq.heappop(heap)
        owned[r].append(b)
        heapq.heappush(heap, (load + int(sizes[b]), r))
    return [np.array(sorted(o), np.int64) for o in owned]


def shard(ensemble: System, systems) -> System:
    """The sub-ensemble of the given systems of `ensemble` (their particles, springs and the
    per-particle arrays, in the order given), with meta["offsets"] of the new ensemble and
    meta["systems_of"] the original system indices."""
    off = np.asarray(ensemble.meta["offsets"], np.int64)
    systems = np.asarray(systems, np.int64)
    sel = [np.arange(off[b], off[b + 1]) for b in systems]
    idx = np.concatenate(sel) if sel else np.zeros(0, np.int64)
    new_off = np.zeros(len(systems) + 1, np.int64)
    for k, b in enumerate(systems):
        new_off[k + 1] = new_off[k] + (off[b + 1] - off[b])
    remap = np.full(ensemble.n, -1, np.int64)
    remap[idx] = np.arange(idx.shape[0])
    keep = remap[ensemble.ij[:, 0]] >= 0
    ij = remap[ensemble.ij[keep]].astype(np.int32)
    arrays = {k: (None if v is None else np.asarray(v)[idx]) for k, v in ensemble.arrays().items() if k != "xyz"}
    meta = dict(ensemble.meta, offsets=new_off, systems=int(len(systems)), systems_of=systems,
                springs=int(ij.shape[0]))
    return System(f"{ensemble.name}_shard", ensemble.xyz[idx].copy(), ij, ensemble.r0[keep].copy(),
                  ensemble.k[keep].copy(), dict(ensemble.config), meta=meta, **arrays)
