"""Benchmark of BioSpring's per-step force-and-integrate loop on GB300.

Workload (one "step" = one simulation step of the whole system): 100,000 particles filled
uniformly (minimum separation 3 A) in a 160 A cube, springs below 5 A (mean degree ~11.3,
stiffness log-uniform in [0.1, 10] kJ/mol/A^2), 20% charged +-1, Coulomb with the
distance-dependent dielectric eps = 4 r and Amber 12-6 LJ (eps 0.2 kcal/mol, r 3.5 A), both
cut at 12 A, pair list rebuilt every 10 steps. Synthetic, seeded (no dataset).

Native arm: inputs resident in HBM; before every timed step L2 is flushed (a 256 MB write,
untimed); each step (the rebuild every 10th step, then the step kernel) is bracketed by CUDA
events on the library's stream. ``e2e`` drives the same steps through the C ABI with host
buffers: per step, external forces H2D from pinned memory, one bs_step call, energies D2H.

Two more figures ride on the same line (rank 0, one GPU):
  batched  512 independent Calpha networks (sizes log-uniform in 200..20,000, ~2.1M particles),
           springs < 10 A, linear steric 8 A, viscosity, rebuild every 10 steps, stepped by the
           persistent clustered kernel with the autotuned shape, against the same systems stepped
           one after another through the single-system path (inputs larger than L2);
  adjoint  loss and dL/dk, dL/dr0 of all springs of a 10,000-particle network after 200 steps with
           checkpoints every 20 (precise positions), timed against the plain 200-step forward of
           the same system (L2 flushed before every timed call).

Reference arm (--impl reference): the CPU restatement of the reference's step (the reference
itself cannot be built where the sources are absent) timed on all host cores with OpenMP.

Prints one JSON line.
"""

from __future__ import annotations

import argparse
import dataclasses
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "particle-steps/s (100k-particle plain step; batched and adjoint/forward beside it)"
UNIT = "particle-steps/s"
N_PARTICLES = 100_000
BOX = 160.0
REBUILD = 10
# Verlet buffer of the device pair list. The largest drift of a particle over a 10-step period
# here grows from 4e-5 A at the start to 3e-3 A after 1,000 steps and 1.1e-2 A after 5,000, so a
# 0.1 A skin (a rebuild is forced past half of it) keeps a margin of 4.6 or more over 5,000 steps
LIST_SKIN = 0.1
STEP_BYTES_PER_PARTICLE_BASE = 84.0   # positions r+w 32, velocities r+w 32, parameters 16, row pointer 4
SPRING_BYTES_PER_ENTRY = 12.0         # partner index + stiffness + rest length
REBUILD_BYTES_PER_PARTICLE = 104.0    # key 4 + permutation 4 + gather/scatter of x, v, parameters 3 x 32
CTL_BYTES = 288                       # device control block (status, step count, energies) read per bs_step
# DRAM bytes (read + write) of one k_step launch on this workload after an L2 flush, from one ncu
# capture of dram__bytes_read.sum + dram__bytes_write.sum, and the digest of the step kernel's
# sources that capture ran on: when the sources have changed since, the line marks the figure stale.
STEP_KERNEL_TRAFFIC = {"bytes": 69.48992e6 + 1.682176e6, "sources_sha": "d0671f577e273adc", "captured": "2026-12-04"}
STEP_KERNEL_SOURCES = ("biospring_gb300/csrc/bs_device.cuh", "biospring_gb300/csrc/bs_kernels.cu",
                       "biospring_gb300/csrc/bs_kernels.cuh", "biospring_gb300/csrc/bs_common.cuh")
DIELECTRIC_NOTE = ("Coulomb eps = 4r (distance-dependent), as the 100k configuration states; the reference's "
                   "electrostatic.hpp has the constant form only, so this term follows the restatement's "
                   "extension (E = K q q / (4 r^2)); the restatement is bit-exact with the reference in constant mode")


def step_sources_sha() -> str:
    import hashlib
    h = hashlib.sha256()
    for rel in STEP_KERNEL_SOURCES:
        with open(os.path.join(ROOT, rel), "rb") as f:
            h.update(f.read())
    return h.hexdigest()[:16]


def peaks() -> dict:
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        with open(path) as f:
            d = json.load(f)
        return {"hbm_gbs": float(d["hbm_gbs"]), "src": "measured"}
    return {"hbm_gbs": 6800.0, "src": "fallback"}


class ClockSampler:
    """Samples nvidia-smi clocks and throttle reasons while the timed region runs."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int = 0, interval_ms: int = 50):
        self.device = device
        self.interval_ms = interval_ms
        self.proc = None
        self.lines: list[str] = []
        self.thread = None

    def start(self, wait_s: float = 5.0):
        """Starts sampling and returns once the first sample has arrived (nvidia-smi takes a while
        to start), so that the timed region that follows is sampled from its beginning."""
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", str(self.interval_ms)], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except (OSError, FileNotFoundError):
            self.proc = None
            return
        self.thread = threading.Thread(target=self._read, daemon=True)
        self.thread.start()
        t_end = time.perf_counter() + wait_s
        while not self.lines and self.proc.poll() is None and time.perf_counter() < t_end:
            time.sleep(0.01)
        self.skip = len(self.lines)  # samples taken before the timed region are not counted

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self) -> dict:
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        if self.thread:
            self.thread.join(timeout=2)
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        # the samples from the timed region on; the last one before it if none came during
        lines = self.lines[getattr(self, "skip", 0):] or self.lines[-1:]
        for line in lines:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx.append(float(parts[2]))
            except ValueError:
                continue
            for name, flag in zip(names, parts[5:9]):
                if flag.lower() == "active":
                    reasons.add(name)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def max_over_ranks(x: float, dist=None, device: str = "cpu") -> float:
    """The slowest rank's time: replicas run in parallel, the job ends with the last one."""
    if dist is None:
        return x
    import torch
    t = torch.tensor([x], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def replica_throughput(n: int, steps: int, slowest_ms: float, world: int) -> float:
    """Whole-job particle-steps/s of `world` independent replicas of n particles (no exchange:
    the plain path does not shard, each GPU steps its own system)."""
    return world * n * steps / (slowest_ms * 1e-3)


def make_workload(seed: int = 42, dielectric_mode: int = 1):
    from biospring_gb300 import workloads as W
    return W.uniform_lj(n=N_PARTICLES, box=BOX, seed=seed, dielectric_mode=dielectric_mode, rebuild_every=REBUILD,
                        list_skin=LIST_SKIN)


def workload_config(system, world: int) -> dict:
    """The `config` object of both arms' lines (identical for the same workload and N)."""
    dbar = 2.0 * system.ij.shape[0] / system.n
    return {
        "workload": f"uniform_lj_100k: N={system.n}, cube {BOX:g} A, springs<5A (mean degree {dbar:.2f}), "
                    f"20% charged, Coulomb eps=4r 12 A, LJ 12-6 Amber 12 A, rebuild every {REBUILD} steps, "
                    f"list skin {LIST_SKIN:g} A",
        "global_batch": system.n * world,
        "parallelism": f"replicas{world}" if world > 1 else "single",
        "dielectric": DIELECTRIC_NOTE,
        "l2": "GPU arm: flushed (256 MB write) before every timed step; CPU arm: no flush (host caches)",
    }


def algorithmic(system, net) -> dict:
    """Algorithmic bytes and FLOPs of one step kernel launch (counts of unique interactions)."""
    n = system.n
    s = system.ij.shape[0]
    dbar = 2.0 * s / n
    pairs_lj = int(net.getPairs(0).shape[0])
    pairs_q = int(net.getPairs(1).shape[0])
    step_bytes = n * (STEP_BYTES_PER_PARTICLE_BASE + SPRING_BYTES_PER_ENTRY * dbar)
    flops = 30.0 * pairs_lj + 12.0 * pairs_q + 24.0 * s + 23.0 * n
    return {"mean_spring_degree": dbar, "unique_lj_pairs": pairs_lj, "unique_coulomb_pairs": pairs_q,
            "step_kernel_bytes": step_bytes, "step_flops": flops,
            "bytes_per_particle_step": step_bytes / n + REBUILD_BYTES_PER_PARTICLE / REBUILD}


def run_native(args) -> dict:
    import torch
    from biospring_gb300 import SpringNetwork

    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))

    system = make_workload(seed=42 + rank)
    net = SpringNetwork()
    net.addParticles(**{k: v for k, v in system.arrays().items() if v is not None})
    net.addSprings(system.ij, system.r0, system.k)
    net.setup(system.bs_config())
    stream = torch.cuda.ExternalStream(net.stream())
    flush = torch.empty(256 * 1024 * 1024, dtype=torch.uint8, device="cuda")

    # warm-up: full graph-captured periods plus the timed loop's launch pattern
    net.computeStep(max(args.warmup, 3) * REBUILD)
    alg = algorithmic(system, net)

    steps = args.steps
    ev = [[torch.cuda.Event(enable_timing=True) for _ in range(3)] for _ in range(steps)]
    launches0 = net.launchCount()
    step0 = net.stepCount()
    sampler = ClockSampler(local)
    sampler.start()
    if dist is not None:
        dist.barrier()
    torch.cuda.synchronize()
    with torch.cuda.stream(stream):
        for i in range(steps):
            flush.zero_()  # evict L2 (untimed: before the start event)
            ev[i][0].record(stream)
            if i % REBUILD == 0:
                net.launchPhase(0)
            ev[i][1].record(stream)
            net.launchPhase(1)
            ev[i][2].record(stream)
    torch.cuda.synchronize()
    if dist is not None:
        dist.barrier()
    clocks = sampler.stop()
    # steps the timed launches completed, read before synchronize() would complete any that a
    # drift past half the list skin stopped (those would make the timed figure too fast)
    done = net.stepCount() - step0
    net.synchronize()
    launches = net.launchCount() - launches0
    if done != steps:
        raise RuntimeError(f"timed region completed {done} of {steps} steps (a stale list stopped the rest)")
    step_ms = [ev[i][0].elapsed_time(ev[i][2]) for i in range(steps)]
    kern_ms = [ev[i][1].elapsed_time(ev[i][2]) for i in range(steps)]
    total_ms = max_over_ranks(float(sum(step_ms)), dist, "cuda")
    value = replica_throughput(system.n, steps, total_ms, world)

    # warm, continuous throughput (graph-captured periods, no flush), for context
    torch.cuda.synchronize()
    w0 = torch.cuda.Event(enable_timing=True)
    w1 = torch.cuda.Event(enable_timing=True)
    net.synchronize()
    w0.record(stream)
    net.computeStepAsync(10 * REBUILD)
    w1.record(stream)
    net.synchronize()
    warm_ms = w0.elapsed_time(w1)

    # end to end through the C ABI with host buffers
    ext = torch.zeros((system.n, 3), dtype=torch.float32).pin_memory().numpy()
    e2e_steps = max(steps, 20)
    for _ in range(3):
        net.setExternalForces(ext, wait=False)
        net.computeStep(1)
        net.energies()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        net.setExternalForces(ext, wait=False)
        net.computeStep(1)
        net.energies()
    t1 = time.perf_counter()
    e2e_value = world * system.n * e2e_steps / (t1 - t0)

    pk = peaks()
    kernel_s = statistics.mean(kern_ms) * 1e-3
    achieved = alg["step_kernel_bytes"] / kernel_s / 1e9
    out = {
        "metric": METRIC,
        "value": value,
        "unit": UNIT,
        "n_gpus": world,
        "steps": steps,
        "warmup": args.warmup,
        "ms_per_step": total_ms / steps,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f32",
        "data": "synthetic (seeded uniform fill, springs, charges)",
        "config": workload_config(system, world),
        "timing": "CUDA events on the library stream around each step (rebuild on every 10th), L2 flushed "
                  "before each",
        "gpu_launches": int(launches),
        "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": int(system.n * 12 + 4),
                "d2h_bytes_per_step": CTL_BYTES,
                "path": "bs_set_external_forces_async (pinned float[3n], copied straight to the device "
                        "in stream order) + bs_step(1) + bs_get_energies per step: one wait per step, "
                        "in bs_step; the energies come with the control block bs_step reads back to "
                        "check the step"},
        "roofline": {
            "bound": "hbm",
            "kernel": "k_step (forces + Euler step)",
            "achieved": achieved,
            "peak": pk["hbm_gbs"],
            "unit": "GB/s",
            "frac": achieved / pk["hbm_gbs"],
            "traffic": STEP_KERNEL_TRAFFIC["bytes"],
            "traffic_src": f"ncu dram__bytes_read.sum + dram__bytes_write.sum of one launch after an L2 flush, "
                           f"captured {STEP_KERNEL_TRAFFIC['captured']}",
            "traffic_stale": STEP_KERNEL_TRAFFIC["sources_sha"] != step_sources_sha(),
            "peak_src": pk["src"],
            "algorithmic_bytes_per_launch": alg["step_kernel_bytes"],
            "kernel_ms": kernel_s * 1e3,
            "flops_per_step": alg["step_flops"],
            "fp32_tflops": alg["step_flops"] / kernel_s / 1e12,
            # no FP32 peak is measured on this part: the nominal one (152 SMs x 128 lanes x 2 flops
            # at the maximum SM clock) gives context only
            "fp32_frac_of_nominal": alg["step_flops"] / kernel_s / (152 * 128 * 2 * 2.07e9),
            "dram_frac": STEP_KERNEL_TRAFFIC["bytes"] / kernel_s / 1e9 / pk["hbm_gbs"],
        },
        "warm_continuous": {"value": system.n * 10 * REBUILD / (warm_ms * 1e-3), "unit": UNIT,
                            "ms_per_step": warm_ms / (10 * REBUILD)},
        "clocks": clocks,
        "interactions": {k: alg[k] for k in ("unique_lj_pairs", "unique_coulomb_pairs")},
    }
    net.close()
    if not args.no_extras:
        batched = run_batched(rank=rank, world=world, dist=dist)
        if rank == 0:
            out["batched"] = batched
    if rank == 0 and world == 1 and not args.no_extras:
        out["adjoint"] = run_adjoint()
        out["frames"] = run_frames(system)
        out["interactive"] = run_interactive(system)
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        out["cpu_baseline"] = cpu_baseline(system, seconds=args.cpu_seconds)
    if dist is not None:
        dist.destroy_process_group()
    return out if rank == 0 else None


def run_batched(steps: int = 100, rank: int = 0, world: int = 1, dist=None) -> dict:
    """The batched ensemble against its systems stepped one after another. With several ranks the
    ensemble is split into whole systems balanced by particle count (biospring_gb300.shard): each
    rank steps its own sub-ensemble, no data is exchanged, and the figure is all the ensemble's
    particle-steps over the slowest rank's time."""
    import torch
    from biospring_gb300 import SpringNetwork, shard, workloads as W

    full = W.ensemble(W.ensemble_sizes(), seed=2024)
    owned = shard.partition_systems(np.diff(full.meta["offsets"]), world)[rank]
    ens = full if world == 1 else shard.shard(full, owned)
    off = ens.meta["offsets"]
    nsys = len(off) - 1
    net = SpringNetwork()
    net.addParticles(xyz=ens.xyz)
    net.addSprings(ens.ij, ens.r0, ens.k)
    net.setSystems(off)
    net.setup(ens.bs_config())
    net.computeStep(3 * REBUILD)
    shape = net.batchAutotune()
    net.computeStep(3 * REBUILD)
    stream = torch.cuda.ExternalStream(net.stream())
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    launches0 = net.launchCount()
    net.synchronize()
    torch.cuda.synchronize()
    if dist is not None:
        dist.barrier()
    e0.record(stream)
    net.computeStepAsync(steps)
    e1.record(stream)
    net.synchronize()
    torch.cuda.synchronize()
    launches = net.launchCount() - launches0
    ms = max_over_ranks(e0.elapsed_time(e1), dist, "cuda")
    batched = full.n * steps / (ms * 1e-3)
    net.close()
    # the same systems, one handle each, stepped one after another (2 periods each)
    seq_steps = 2 * REBUILD
    nets = []
    for b in range(nsys):
        i0, i1 = int(off[b]), int(off[b + 1])
        m = (ens.ij[:, 0] >= i0) & (ens.ij[:, 0] < i1)
        h = SpringNetwork()
        h.addParticles(xyz=ens.xyz[i0:i1])
        h.addSprings(ens.ij[m] - i0, ens.r0[m], ens.k[m])
        h.setup(ens.bs_config())
        h.computeStep(REBUILD)
        nets.append(h)
    torch.cuda.synchronize()
    if dist is not None:
        dist.barrier()
    t0 = time.perf_counter()
    for h in nets:
        h.computeStep(seq_steps)
    torch.cuda.synchronize()
    seq_s = max_over_ranks(time.perf_counter() - t0, dist, "cuda")
    for h in nets:
        h.close()
    sequential = full.n * seq_steps / seq_s
    dbar = 2.0 * full.ij.shape[0] / full.n
    step_bytes = STEP_BYTES_PER_PARTICLE_BASE + SPRING_BYTES_PER_ENTRY * dbar
    pk = peaks()
    return {
        "value": batched, "unit": UNIT, "systems": len(full.meta["offsets"]) - 1, "particles": int(full.n),
        "n_gpus": world, "systems_per_rank": f"{nsys} on rank {rank} (whole systems, balanced by particles)",
        "steps": steps, "ms_per_step": ms / steps, "gpu_launches": int(launches),
        "shape": {"block": shape[0], "lanes": shape[1], "cluster": shape[2], "picked_by": "bs_batch_autotune"},
        "sequential_plain": {"value": sequential, "unit": UNIT,
                             "how": f"each system alone through bs_step({seq_steps}), one after another"},
        "speedup_vs_sequential": batched / sequential,
        "roofline": {"bound": "hbm", "achieved": batched * step_bytes / 1e9 / world, "peak": pk["hbm_gbs"],
                     "unit": "GB/s", "frac": batched * step_bytes / 1e9 / world / pk["hbm_gbs"], "peak_src": pk["src"],
                     "bytes_per_particle_step": step_bytes, "per": "GPU"},
        "workload": "512 Calpha networks, sizes log-uniform 200..20000 (seed 2024), springs < 10 A "
                    f"(mean degree {dbar:.1f}), linear steric 8 A, viscosity 1, dt 0.01 fs, rebuild every 10",
        "l2": "inputs larger than L2",
    }


def run_frames(system=None, every: int = 10, steps: int = 200) -> dict:
    """Cost of the frame recorder on the 100k workload: the same warm run with and without a frame
    (positions in caller order and energies, written by the device into the host ring) every
    `every` steps."""
    import torch
    from biospring_gb300 import SpringNetwork
    s = system if system is not None else make_workload()
    net = SpringNetwork()
    net.addParticles(**{k: v for k, v in s.arrays().items() if v is not None})
    net.addSprings(s.ij, s.r0, s.k)
    net.setup(s.bs_config())
    net.computeStep(2 * REBUILD)
    stream = torch.cuda.ExternalStream(net.stream())

    def timed():
        a = torch.cuda.Event(enable_timing=True)
        b = torch.cuda.Event(enable_timing=True)
        net.synchronize()
        a.record(stream)
        net.computeStepAsync(steps)
        b.record(stream)
        net.synchronize()
        return a.elapsed_time(b)

    timed()
    off_ms = min(timed() for _ in range(3))
    net.setFrames(every, 4 * steps // every)
    timed()
    net.readFrames(4 * steps // every)
    on_ms = min(timed() for _ in range(3))
    got, _xyz, _en, dropped = net.readFrames(4 * steps // every)
    net.close()
    return {"value": s.n * steps / (on_ms * 1e-3), "unit": UNIT, "every": every,
            "without_frames": s.n * steps / (off_ms * 1e-3), "overhead": on_ms / off_ms - 1.0,
            "frames_read": int(len(got)), "dropped": int(dropped),
            "bytes_per_frame": int(s.n * 12 + 64),
            "how": "warm run of 200 steps (graph-replayed periods), CUDA events; frames go from the device "
                   "straight into page-locked host memory"}


def run_interactive(system=None, every: int = 10, frames: int = 50) -> dict:
    """Interactive coupling at the 100k workload (an IMD-style loop): each frame the host pushes a
    pulling force on 100 particles from page-locked memory, the device steps `every` steps and the
    host reads every position back (wall clock)."""
    import torch
    from biospring_gb300 import SpringNetwork
    s = system if system is not None else make_workload()
    net = SpringNetwork()
    net.addParticles(**{k: v for k, v in s.arrays().items() if v is not None})
    net.addSprings(s.ij, s.r0, s.k)
    net.setup(s.bs_config())
    ext = torch.zeros((s.n, 3), dtype=torch.float32).pin_memory().numpy()
    ext[:100, 0] = 1e-3
    for _ in range(3):
        net.setExternalForces(ext, wait=False)
        net.computeStep(every)
        net.getPositions()
    t0 = time.perf_counter()
    for _ in range(frames):
        net.setExternalForces(ext, wait=False)
        net.computeStep(every)
        xyz = net.getPositions()
    dt = (time.perf_counter() - t0) / frames
    net.close()
    assert np.isfinite(xyz).all()
    return {"frame_rate_hz": 1.0 / dt, "ms_per_frame": dt * 1e3, "steps_per_frame": every,
            "value": s.n * every / dt, "unit": UNIT,
            "h2d_bytes_per_frame": int(s.n * 12 + 4), "d2h_bytes_per_frame": int(s.n * 12 + CTL_BYTES),
            "how": "bs_set_external_forces_async + bs_step(every) + bs_get_positions per frame, wall clock"}


def run_adjoint(reps: int = 5) -> dict:
    """Adjoint (loss + gradients) against the plain forward of the same 200 steps."""
    import torch
    from biospring_gb300 import SpringNetwork, workloads as W

    s, target, nsteps = W.adjoint_fit(10_000, seed=4)
    s.config["precise_positions"] = 1
    flush = torch.empty(256 * 1024 * 1024, dtype=torch.uint8, device="cuda")

    def handle():
        h = SpringNetwork()
        h.addParticles(**{k: v for k, v in s.arrays().items() if v is not None})
        h.addSprings(s.ij, s.r0, s.k)
        h.setup(s.bs_config())
        return h

    fwd, adj = handle(), handle()
    x0 = fwd.getPositions()
    fwd.computeStep(nsteps)
    adj.adjoint(nsteps, target, 20)

    def timed(fn, before=None):
        ts = []
        for _ in range(reps):
            if before:
                before()
            flush.zero_()
            torch.cuda.synchronize()
            t = time.perf_counter()
            fn()
            torch.cuda.synchronize()
            ts.append(time.perf_counter() - t)
        return statistics.median(ts)

    t_fwd = timed(lambda: fwd.computeStep(nsteps), before=lambda: fwd.setPositions(x0))
    result = {}

    def run_adj():
        result["r"] = adj.adjoint(nsteps, target, 20)

    t_adj = timed(run_adj)
    launches0 = adj.launchCount()
    run_adj()
    launches = adj.launchCount() - launches0
    loss, gk, gr = result["r"]
    fwd.close()
    adj.close()
    return {
        "ratio": t_adj / t_fwd, "adjoint_ms": t_adj * 1e3, "forward_ms": t_fwd * 1e3, "loss": loss,
        "gradients": int(2 * gk.shape[0]), "gpu_launches": int(launches),
        "workload": f"Calpha network N={s.n} ({s.ij.shape[0]} springs), target = start + smooth 2 A field, "
                    f"{nsteps} steps, checkpoints every 20, precise positions",
        "timing": "median wall time of bs_adjoint vs bs_step(200) from the same state, L2 flushed before each",
    }


def run_case(name: str) -> dict:
    """Small fixed drivers for profiling one kernel family under ncu: each sets up one workload,
    runs a few warm-up steps and then the launches to capture."""
    import torch
    from biospring_gb300 import SpringNetwork, workloads as W

    if name == "step100k":
        system = make_workload()
        net = SpringNetwork()
        net.addParticles(**{k: v for k, v in system.arrays().items() if v is not None})
        net.addSprings(system.ij, system.r0, system.k)
        net.setup(system.bs_config())
        net.computeStep(50)
        stream = torch.cuda.ExternalStream(net.stream())
        e = [torch.cuda.Event(enable_timing=True) for _ in range(4)]
        with torch.cuda.stream(stream):
            e[0].record(stream)
            for _ in range(20):
                net.launchPhase(0)
            e[1].record(stream)
            e[2].record(stream)
            for _ in range(50):
                net.launchPhase(1)
            e[3].record(stream)
        torch.cuda.synchronize()
        net.synchronize()
        out = {"case": name, "rebuild_us": e[0].elapsed_time(e[1]) * 1000 / 20,
               "step_us": e[2].elapsed_time(e[3]) * 1000 / 50}
        net.close()
        return out
    if name == "batch64":
        ens = W.ensemble(W.ensemble_sizes(count=64, seed=7), seed=11)
        net = SpringNetwork()
        net.addParticles(xyz=ens.xyz)
        net.addSprings(ens.ij, ens.r0, ens.k)
        net.setSystems(ens.meta["offsets"])
        net.setBatchShape(512, 2, 4)
        net.setup(ens.bs_config())
        net.computeStep(2 * REBUILD)
        net.close()
        return {"case": name, "particles": int(ens.n), "systems": 64}
    if name == "adjoint10k":
        s, target, _ = W.adjoint_fit(10_000, seed=4)
        s.config["precise_positions"] = 1
        net = SpringNetwork()
        net.addParticles(**{k: v for k, v in s.arrays().items() if v is not None})
        net.addSprings(s.ij, s.r0, s.k)
        net.setup(s.bs_config())
        loss, _, _ = net.adjoint(40, target, 20)
        net.close()
        return {"case": name, "loss": loss}
    if name == "batch512":
        # the bench's ensemble (512 systems, 2.1M particles): rebuild chain and whole periods
        ens = W.ensemble(W.ensemble_sizes(), seed=2024)
        net = SpringNetwork()
        net.addParticles(xyz=ens.xyz)
        net.addSprings(ens.ij, ens.r0, ens.k)
        net.setSystems(ens.meta["offsets"])
        net.setup(ens.bs_config())
        net.computeStep(3 * REBUILD)
        shape = net.batchAutotune()
        net.computeStep(3 * REBUILD)
        net.synchronize()
        stream = torch.cuda.ExternalStream(net.stream())
        e = [torch.cuda.Event(enable_timing=True) for _ in range(4)]
        with torch.cuda.stream(stream):
            e[0].record(stream)
            for _ in range(3):
                net.launchPhase(0)
            e[1].record(stream)
        net.synchronize()
        net.computeStep(REBUILD)  # back to a whole period after the extra rebuilds
        net.synchronize()
        e[2].record(stream)
        net.computeStepAsync(5 * REBUILD)
        e[3].record(stream)
        net.synchronize()
        torch.cuda.synchronize()
        out = {"case": name, "particles": int(ens.n), "shape": list(shape),
               "rebuild_ms": e[0].elapsed_time(e[1]) / 3, "period_ms": e[2].elapsed_time(e[3]) / 5}
        net.close()
        return out
    if name == "clusterpairs":
        return cluster_pair_counts()
    raise SystemExit(f"unknown case {name}")


def cluster_pair_counts(cluster_sizes=(4, 8)) -> dict:
    """Pair evaluations a cluster-pair tile kernel would make on the 100k workload, against the
    ordered pairs within the cutoff and the Verlet list entries the gather kernel reads (CPU,
    scipy). Clusters are built as in cluster-pair MD codes: columns on an x-y grid whose cells
    hold `c` particles per unit of the mean spacing, sorted by z, cut into groups of `c`; a cluster
    pair is kept when the bounding boxes are closer than the list radius, and every slot of the
    c x c tile is evaluated."""
    from scipy.spatial import cKDTree
    system = make_workload()
    x = system.xyz.astype(np.float64)
    n = x.shape[0]
    rc = float(system.config["steric_cutoff"])
    rl = rc + LIST_SKIN
    tree = cKDTree(x)
    useful = int(tree.count_neighbors(tree, rc)) - n
    listed = int(tree.count_neighbors(tree, rl)) - n
    lo, hi = x.min(0), x.max(0)
    dens = n / float(np.prod(hi - lo))
    out = {"case": "clusterpairs", "ordered_pairs_within_cutoff": useful, "verlet_entries_upper": listed}
    for c in cluster_sizes:
        a = (c / dens) ** (1.0 / 3.0)
        ncol = np.maximum(1, np.floor((hi[:2] - lo[:2]) / a).astype(int))
        cx = np.minimum(((x[:, 0] - lo[0]) / (hi[0] - lo[0]) * ncol[0]).astype(int), ncol[0] - 1)
        cy = np.minimum(((x[:, 1] - lo[1]) / (hi[1] - lo[1]) * ncol[1]).astype(int), ncol[1] - 1)
        col = cx * ncol[1] + cy
        order = np.lexsort((x[:, 2], col))
        starts = np.r_[0, np.flatnonzero(np.diff(col[order])) + 1]
        ends = np.r_[starts[1:], n]
        cid = np.empty(n, np.int64)
        nc = 0
        for b, e in zip(starts, ends):
            k = np.arange(e - b) // c
            cid[order[b:e]] = nc + k
            nc += int(k[-1]) + 1
        bmin = np.full((nc, 3), np.inf)
        bmax = np.full((nc, 3), -np.inf)
        np.minimum.at(bmin, cid, x)
        np.maximum.at(bmax, cid, x)
        cen, half = (bmin + bmax) / 2, (bmax - bmin) / 2
        reach = rl + 2.0 * float(np.linalg.norm(half, axis=1).max())
        pr = cKDTree(cen).query_pairs(reach, output_type="ndarray")
        pr = np.vstack([pr, pr[:, ::-1], np.c_[np.arange(nc), np.arange(nc)]])
        gap = np.maximum(0.0, np.maximum(bmin[pr[:, 0]] - bmax[pr[:, 1]], bmin[pr[:, 1]] - bmax[pr[:, 0]]))
        kept = int(((gap * gap).sum(1) < rl * rl).sum())
        out[f"clusters_{c}"] = {"clusters": nc, "cluster_pairs": kept, "evaluations": kept * c * c,
                                "evaluations_per_useful_pair": kept * c * c / useful}
    return out


def _oracle_steps_per_s(system, steps: int, warmup: int) -> tuple[float, float]:
    """(particle-steps/s, seconds) of the CPU restatement on all host cores: `warmup` untimed
    steps, then `steps` timed ones."""
    from oracle import pyoracle
    orc = pyoracle.Oracle(system)
    for _ in range(warmup):
        orc.time_steps(1)
    t = orc.time_steps(steps)
    orc.close()
    return system.n * steps / t, t


def cpu_baseline(system, seconds: float = 15.0) -> dict:
    """The CPU restatement of the reference step on all host cores (OpenMP), bounded sample of
    the same workload; beside it the same sample with the constant dielectric (eps = 4), the
    reference's own Coulomb form."""
    from oracle import pyoracle
    pyoracle.build_oracle()
    cores = os.cpu_count() or 1
    os.environ["OMP_NUM_THREADS"] = str(cores)
    probe, t1 = _oracle_steps_per_s(system, 1, 1)
    nsteps = max(1, min(30, int(seconds / max(t1, 1e-3))))
    value, _ = _oracle_steps_per_s(system, nsteps, 2)
    const = dict(system.config)
    const["dielectric_mode"] = 0
    cs = dataclasses.replace(system, config=const)
    cvalue, _ = _oracle_steps_per_s(cs, max(1, nsteps // 3), 1)
    return {"value": value, "unit": UNIT, "cores": cores, "kind": "port",
            "sample": f"{nsteps} full steps of the 100k workload after 2 untimed ones",
            "dielectric": "eps = 4r, as the native arm",
            "constant_dielectric_value": cvalue}


REFERENCE_MAX_STEPS = 300  # about a minute of the 100k step on 16 host cores


def run_reference(args) -> dict | None:
    """The reference arm: the CPU restatement (bit-exact with the reference's own step in constant
    dielectric mode, and its eps = 4r extension here) on all host cores, on the native arm's
    workload, config, metric and warm-up. Neither the system nor the configuration comes from a
    product library: the oracle's library holds its own copy of the generators and its own
    restatement of the reference's default parameters."""
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    if rank != 0:
        return None
    from oracle import pyoracle
    pyoracle.build_oracle()
    pyoracle.use_oracle_generator()
    cores = os.cpu_count() or 1
    os.environ["OMP_NUM_THREADS"] = str(cores)
    system = make_workload(seed=42)
    steps = max(1, min(args.steps, REFERENCE_MAX_STEPS))
    value, t = _oracle_steps_per_s(system, steps, args.warmup)
    sample = (f"{steps} full steps after {args.warmup} untimed ones, OpenMP on all {cores} host cores"
              + ("" if steps == args.steps else f" (bounded sample of the {args.steps} requested)"))
    return {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world,
        "steps": steps, "warmup": args.warmup, "ms_per_step": t * 1e3 / steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded uniform fill, springs, charges)",
        "config": workload_config(system, world),
        "impl": "reference",
        "timing": "wall clock around the oracle's step loop (host code, no GPU)",
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": "port", "sample": sample},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=1000)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="native", choices=["native", "reference"])
    ap.add_argument("--cpu-seconds", type=float, default=15.0)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-extras", action="store_true", help="skip the batched and adjoint figures")
    ap.add_argument("--case", choices=["step100k", "batch64", "batch512", "adjoint10k", "clusterpairs"],
                    help="run one small profiling driver instead of the benchmark")
    args = ap.parse_args()
    if args.case:
        from biospring_gb300 import build
        if not os.path.exists(build.LIB):
            build.build_all()
        print(json.dumps(run_case(args.case)))
        return
    args.warmup = max(args.warmup, 3)
    if args.impl == "reference":
        out = run_reference(args)
    else:
        from biospring_gb300 import build
        if not os.path.exists(build.LIB):
            build.build_all()
        out = run_native(args)
    if out is not None:
        print(json.dumps(out))


if __name__ == "__main__":
    main()
