"""Whole-system sharding of a batched ensemble over two gloo ranks on the CPU.

Each rank computes the assignment of systems to ranks from the sizes alone; the ranks gather
what they computed and check that they agree, that every system lands on exactly one rank, that
the loads are balanced to within one system, and that each rank's sub-ensemble holds exactly its
systems' particles and springs. The aggregate throughput the bench reports (all particle-steps
over the slowest rank's time) is checked against the per-rank parts."""

from __future__ import annotations

import os
import socket

import numpy as np
import pytest
import torch
import torch.distributed as dist
import torch.multiprocessing as mp

from biospring_gb300 import shard
from biospring_gb300 import workloads as W

SIZES_SEED = 2024


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank: int, world: int, port: int, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        sizes = W.ensemble_sizes(count=512, seed=SIZES_SEED)
        parts = shard.partition_systems(sizes, world)
        # every rank's view of the whole assignment, as one owner per system
        owner = np.full(sizes.shape[0], -1, np.int64)
        for r, p in enumerate(parts):
            owner[p] = r
        views = [torch.zeros(sizes.shape[0], dtype=torch.int64) for _ in range(world)]
        dist.all_gather(views, torch.from_numpy(owner))
        # a small ensemble actually split: this rank's shard against the systems it owns
        small = W.ensemble([200, 350, 500, 260, 610, 420, 300], seed=9)
        mine = shard.partition_systems(np.diff(small.meta["offsets"]), world)[rank]
        sub = shard.shard(small, mine)
        off = small.meta["offsets"]
        expect = np.concatenate([small.xyz[off[b]:off[b + 1]] for b in mine])
        springs = sum(int(((small.ij[:, 0] >= off[b]) & (small.ij[:, 0] < off[b + 1])).sum()) for b in mine)
        # aggregate throughput: each rank "steps" its particles for a rank-dependent time
        steps = 100
        my_ms = 10.0 + 3.0 * rank
        t = torch.tensor([my_ms], dtype=torch.float64)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        my_particles = int(sizes[parts[rank]].sum())
        tot = torch.tensor([my_particles], dtype=torch.int64)
        dist.all_reduce(tot)
        q.put(dict(rank=rank, views=[v.numpy() for v in views], sub_xyz_ok=bool(np.array_equal(sub.xyz, expect)),
                   sub_springs=int(sub.ij.shape[0]), springs=springs,
                   ij_inside=bool((sub.ij >= 0).all() and (sub.ij < sub.n).all()),
                   sub_offsets=sub.meta["offsets"].tolist(), sizes_mine=np.diff(off)[mine].tolist(),
                   max_ms=float(t.item()), total=int(tot.item()), steps=steps,
                   per_rank_rate=my_particles * steps / (my_ms * 1e-3)))
    finally:
        dist.destroy_process_group()


def test_two_ranks_partition_and_aggregate():
    build_synth()
    world = 2
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, world, port, q)) for r in range(world)]
    for p in procs:
        p.start()
    out = [q.get(timeout=240) for _ in range(world)]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    out.sort(key=lambda d: d["rank"])
    sizes = W.ensemble_sizes(count=512, seed=SIZES_SEED)
    # all ranks computed the same assignment, and it covers every system exactly once
    v0 = out[0]["views"][0]
    for d in out:
        for v in d["views"]:
            np.testing.assert_array_equal(v, v0)
    assert (v0 >= 0).all() and (v0 < world).all()
    loads = np.array([sizes[v0 == r].sum() for r in range(world)])
    assert loads.sum() == sizes.sum()
    assert loads.max() - loads.min() <= sizes.max()
    print(f"loads per rank {loads.tolist()} (largest system {int(sizes.max())})")
    for d in out:
        assert d["sub_xyz_ok"] and d["ij_inside"]
        assert d["sub_springs"] == d["springs"]
        assert np.array_equal(np.diff(d["sub_offsets"]), d["sizes_mine"])
    # whole-job rate = all particle-steps over the slowest rank's time
    max_ms = max(10.0 + 3.0 * r for r in range(world))
    assert all(d["max_ms"] == max_ms for d in out)
    total = out[0]["total"]
    assert total == int(sizes.sum())
    agg = total * out[0]["steps"] / (max_ms * 1e-3)
    assert agg <= sum(d["per_rank_rate"] for d in out) + 1e-6
    import bench
    assert bench.replica_throughput(total // world, out[0]["steps"], max_ms, world) == pytest.approx(
        total // world * world * out[0]["steps"] / (max_ms * 1e-3))


def test_partition_is_deterministic_and_balanced():
    rng = np.random.default_rng(1)
    for world in (1, 2, 3, 4, 8):
        sizes = rng.integers(200, 20000, size=97)
        a = shard.partition_systems(sizes, world)
        b = shard.partition_systems(sizes.copy(), world)
        assert all(np.array_equal(x, y) for x, y in zip(a, b))
        assert sorted(np.concatenate(a).tolist()) == list(range(sizes.shape[0]))
        loads = [int(sizes[p].sum()) for p in a]
        assert max(loads) - min(loads) <= sizes.max()
    with pytest.raises(ValueError):
        shard.partition_systems([1, 2], 0)


def build_synth():
    from biospring_gb300 import build
    build.build_synth()
