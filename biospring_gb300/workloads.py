"""Seeded synthetic systems for the parity tests and the benchmark.

No dataset is involved: every system is generated from a seed.

* ``ca_network``   -- compact Calpha-like chain (confined self-avoiding walk, 3.8 A bonds,
  radius of gyration ~ 2.2 N^0.38 A), springs between all pairs closer than a cutoff with
  rest length = initial distance, linear steric, viscosity on, and a Gaussian position kick
  of 1 A (per coordinate) on a seeded 5% of the particles.
* ``uniform_lj``   -- N particles filled uniformly (random sequential addition with a minimum
  separation) in a cube, springs below 5 A with log-uniform stiffness, a seeded 20% charged
  +-1 (balanced), Amber 12-6 LJ and Coulomb with 12 A cutoffs.
* ``membrane_globule`` -- compact bead globule with per-bead IMPALA transfer energy and
  accessible surface, flat membrane.
* ``ensemble_sizes`` -- the log-uniform sizes of a batched ensemble.
"""

from __future__ import annotations

import ctypes as C
import dataclasses
import os

import numpy as np

from . import capi

PKG = os.path.dirname(os.path.abspath(__file__))
SYNTH_PATH = os.path.join(PKG, "libbs_synth.so")
KCAL_TO_KJ = 4.1840  # src/forcefield/constants.hpp:46

_synth = None
_synth_path = SYNTH_PATH


def set_generator_library(path: str) -> None:
    """Takes the generators (the bs_synth_* functions of csrc/synth.cpp) from another shared
    library built from the same source; the same seed gives the same system."""
    global _synth, _synth_path
    if path != _synth_path:
        _synth, _synth_path = None, path


def _lib():
    global _synth
    if _synth is None:
        if not os.path.exists(_synth_path):
            raise RuntimeError(f"{_synth_path} is missing: run the package build first")
        lib = C.CDLL(_synth_path)
        lib.bs_synth_ca_chain.restype = C.c_double
        lib.bs_synth_ca_chain.argtypes = [C.c_int64, C.c_uint64, C.c_double, C.c_double, C.c_double,
                                          C.POINTER(C.c_float)]
        lib.bs_synth_rsa.restype = C.c_int64
        lib.bs_synth_rsa.argtypes = [C.c_int64, C.c_double, C.c_double, C.c_uint64, C.c_int64,
                                     C.POINTER(C.c_float)]
        lib.bs_synth_pairs_within.restype = C.c_int64
        lib.bs_synth_pairs_within.argtypes = [C.c_int64, C.POINTER(C.c_float), C.c_double,
                                              C.POINTER(C.c_int32), C.c_int64]
        _synth = lib
    return _synth


@dataclasses.dataclass
class System:
    """A particle system in the reference's units, plus its run parameters."""

    name: str
    xyz: np.ndarray                      # float32 (n, 3)
    ij: np.ndarray                       # int32 (s, 2)
    r0: np.ndarray                       # float32 (s,)
    k: np.ndarray                        # float32 (s,)
    config: dict
    vel: np.ndarray | None = None
    mass: np.ndarray | None = None
    charge: np.ndarray | None = None
    radius: np.ndarray | None = None
    epsilon: np.ndarray | None = None
    hydrophobicity: np.ndarray | None = None
    sasa: np.ndarray | None = None
    transfer: np.ndarray | None = None
    is_static: np.ndarray | None = None
    bodies: list | None = None
    meta: dict = dataclasses.field(default_factory=dict)

    @property
    def n(self) -> int:
        return int(self.xyz.shape[0])

    def arrays(self) -> dict:
        return {k: getattr(self, k) for k in ("xyz", "vel", "mass", "charge", "radius", "epsilon",
                                              "hydrophobicity", "sasa", "transfer", "is_static")}

    def bs_config(self) -> capi.BsConfig:
        cfg = capi.default_config()
        for key, v in self.config.items():
            setattr(cfg, key, v)
        return cfg


def ca_chain(n: int, seed: int, step: float = 3.8, rg: float | None = None, min_sep: float = 4.0) -> np.ndarray:
    """Confined self-avoiding walk, float32 (n, 3), centred on the origin."""
    rg = 2.2 * n ** 0.38 if rg is None else rg
    out = np.zeros((n, 3), dtype=np.float32)
    _lib().bs_synth_ca_chain(n, seed, step, rg, min_sep, out.ctypes.data_as(C.POINTER(C.c_float)))
    return out


def rsa_fill(n: int, box: float, min_sep: float, seed: int, max_trials: int = 200000) -> np.ndarray:
    out = np.zeros((n, 3), dtype=np.float32)
    placed = _lib().bs_synth_rsa(n, box, min_sep, seed, max_trials, out.ctypes.data_as(C.POINTER(C.c_float)))
    if placed < n:
        raise ValueError(f"random sequential addition jammed at {placed} of {n} particles (box {box} A)")
    return out


def pairs_within(xyz: np.ndarray, cutoff: float) -> np.ndarray:
    xyz = np.ascontiguousarray(xyz, dtype=np.float32)
    lib = _lib()
    cnt = lib.bs_synth_pairs_within(xyz.shape[0], xyz.ctypes.data_as(C.POINTER(C.c_float)), cutoff, None, 0)
    ij = np.zeros((max(cnt, 1), 2), dtype=np.int32)
    lib.bs_synth_pairs_within(xyz.shape[0], xyz.ctypes.data_as(C.POINTER(C.c_float)), cutoff,
                              ij.ctypes.data_as(C.POINTER(C.c_int32)), cnt)
    return ij[:cnt]


def _distances(xyz: np.ndarray, ij: np.ndarray) -> np.ndarray:
    d = xyz[ij[:, 1]].astype(np.float64) - xyz[ij[:, 0]].astype(np.float64)
    return np.sqrt((d * d).sum(axis=1)).astype(np.float32)


def ca_network(n: int = 2000, seed: int = 1, spring_cutoff: float = 10.0, k: float = 1.0 * KCAL_TO_KJ,
               steric_cutoff: float = 8.0, kick_fraction: float = 0.05, kick_sigma: float = 1.0,
               name: str | None = None) -> System:
    """Plain Calpha elastic network (the 2,000-particle CPU/GPU configuration at n=2000)."""
    xyz = ca_chain(n, seed)
    ij = pairs_within(xyz, spring_cutoff)
    r0 = _distances(xyz, ij)
    kk = np.full(ij.shape[0], k, dtype=np.float32)
    rng = np.random.default_rng(seed + 7919)
    nk = int(round(kick_fraction * n))
    kicked = np.sort(rng.choice(n, size=nk, replace=False)) if nk else np.zeros(0, np.int64)
    xyz = xyz.copy()
    xyz[kicked] += rng.normal(0.0, kick_sigma, size=(nk, 3)).astype(np.float32)
    cfg = dict(timestep=0.01, spring_enable=1, steric_enable=1, steric_cutoff=steric_cutoff,
               steric_mode=capi.BS_STERIC_LINEAR, viscosity_enable=1, viscosity_value=1.0,
               rebuild_every=10, list_skin=1.0)
    return System(name or f"ca_network_n{n}_s{seed}", xyz, ij, r0, kk, cfg,
                  meta=dict(seed=seed, kicked=int(nk), springs=int(ij.shape[0])))


def uniform_lj(n: int = 100_000, box: float = 160.0, seed: int = 42, min_sep: float = 3.0,
               spring_cutoff: float = 5.0, charged_fraction: float = 0.2, dielectric_mode: int = 0,
               dielectric: float = 4.0, cutoff: float = 12.0, eps_kcal: float = 0.2, radius: float = 3.5,
               list_skin: float = 0.5, rebuild_every: int = 10) -> System:
    """Uniform large system: LJ 12-6 Amber + Coulomb + springs (the 100k-particle configuration)."""
    xyz = rsa_fill(n, box, min_sep, seed)
    ij = pairs_within(xyz, spring_cutoff)
    r0 = _distances(xyz, ij)
    rng = np.random.default_rng(seed + 104729)
    kk = np.exp(rng.uniform(np.log(0.1), np.log(10.0), size=ij.shape[0])).astype(np.float32)
    nq = int(round(charged_fraction * n)) // 2 * 2
    q_idx = rng.choice(n, size=nq, replace=False)
    charge = np.zeros(n, dtype=np.float32)
    charge[q_idx[: nq // 2]] = 1.0
    charge[q_idx[nq // 2:]] = -1.0
    cfg = dict(timestep=0.01, spring_enable=1, steric_enable=1, steric_cutoff=cutoff,
               steric_mode=capi.BS_STERIC_LJ_12_6_AMBER, coulomb_enable=1, coulomb_cutoff=cutoff,
               coulomb_dielectric=dielectric, dielectric_mode=dielectric_mode,
               rebuild_every=rebuild_every, list_skin=list_skin)
    return System(f"uniform_lj_n{n}_L{box:g}_s{seed}", xyz, ij, r0, kk, cfg, charge=charge,
                  radius=np.full(n, radius, np.float32), epsilon=np.full(n, eps_kcal * KCAL_TO_KJ, np.float32),
                  meta=dict(seed=seed, springs=int(ij.shape[0]), charged=nq, box=box))


def membrane_globule(n: int = 20_000, seed: int = 3, spring_cutoff: float = 8.0, k: float = 1.0 * KCAL_TO_KJ,
                     z0: float = 15.75, nbodies: int = 0, body_size: int = 500) -> System:
    """IMPALA + (optionally) rigid bodies on a compact bead globule (4 beads per residue)."""
    rg = 2.2 * (n / 4) ** 0.38
    xyz = ca_chain(n, seed, step=3.0, rg=rg, min_sep=2.5)
    ij = pairs_within(xyz, spring_cutoff)
    r0 = _distances(xyz, ij)
    kk = np.full(ij.shape[0], k, dtype=np.float32)
    rng = np.random.default_rng(seed + 15485863)
    transfer = rng.uniform(-0.05, 0.05, size=n).astype(np.float32)
    sasa = rng.uniform(0.0, 60.0, size=n).astype(np.float32)
    bodies = None
    if nbodies:
        starts = np.linspace(0, n - body_size, nbodies).astype(np.int64)
        bodies = [np.arange(s, s + body_size, dtype=np.int32) for s in starts]
    cfg = dict(timestep=0.01, spring_enable=1, impala_enable=1, impala_z0=z0, viscosity_enable=1,
               viscosity_value=1.0, rigidbody_enable=1 if nbodies else 0, rebuild_every=10, list_skin=1.0)
    return System(f"membrane_globule_n{n}_s{seed}", xyz, ij, r0, kk, cfg, sasa=sasa, transfer=transfer,
                  bodies=bodies, meta=dict(seed=seed, springs=int(ij.shape[0])))


def ensemble_sizes(count: int = 512, lo: int = 200, hi: int = 20_000, seed: int = 2024) -> np.ndarray:
    rng = np.random.default_rng(seed)
    return np.exp(rng.uniform(np.log(lo), np.log(hi), size=count)).astype(np.int64)


def ensemble(sizes, seed: int = 2024, **kw) -> System:
    """Batched ensemble: independent Calpha networks (built as ``ca_network``, one seed each)
    concatenated into one System; ``meta["offsets"]`` (int64, len(sizes) + 1) gives each
    system's particle range."""
    parts = [ca_network(int(nb), seed=seed + 1000 * b + 1, **kw) for b, nb in enumerate(sizes)]
    offsets = np.zeros(len(parts) + 1, dtype=np.int64)
    for b, s in enumerate(parts):
        offsets[b + 1] = offsets[b] + s.n
    xyz = np.concatenate([s.xyz for s in parts]).astype(np.float32)
    ij = np.concatenate([s.ij + np.int32(offsets[b]) for b, s in enumerate(parts)]).astype(np.int32)
    r0 = np.concatenate([s.r0 for s in parts]).astype(np.float32)
    kk = np.concatenate([s.k for s in parts]).astype(np.float32)
    return System(f"ensemble_{len(parts)}_s{seed}", xyz, ij, r0, kk, dict(parts[0].config),
                  meta=dict(seed=seed, offsets=offsets, systems=len(parts), springs=int(ij.shape[0])))


def smooth_displacement(xyz: np.ndarray, seed: int, amplitude: float = 2.0, modes: int = 3) -> np.ndarray:
    """A seeded smooth displacement field: a sum of `modes` low-wavenumber sinusoids per axis with
    seeded directions and phases, scaled so that max |u| = amplitude (A)."""
    rng = np.random.default_rng(seed)
    x = xyz.astype(np.float64)
    span = max(float(np.ptp(x, axis=0).max()), 1.0)
    u = np.zeros_like(x)
    for _ in range(modes):
        kvec = rng.normal(size=3)
        kvec *= (2.0 * np.pi / span) / np.linalg.norm(kvec)
        phase = rng.uniform(0.0, 2.0 * np.pi, size=3)
        amp = rng.normal(size=3)
        u += amp[None, :] * np.sin(x @ kvec[:, None] + phase[None, :])
    u *= amplitude / np.sqrt((u * u).sum(axis=1)).max()
    return u


def adjoint_fit(n: int = 10_000, seed: int = 4, amplitude: float = 2.0, nsteps: int = 200) -> tuple:
    """The adjoint workload: a Calpha network built as ``ca_network`` and a target equal to the
    start positions plus a seeded smooth displacement field of the given amplitude. Returns
    (System, target float32 (n, 3), nsteps)."""
    s = ca_network(n, seed=seed)
    target = (s.xyz.astype(np.float64) + smooth_displacement(s.xyz, seed + 17, amplitude)).astype(np.float32)
    s.meta["nsteps"] = nsteps
    return s, target, nsteps


def field_map(shape, origin, spacing, seed: int, amplitude: float = 100.0, centres: int = 6) -> np.ndarray:
    """A smooth synthetic scalar map (a sum of Gaussian wells and hills, like an electrostatic
    potential in kT/e around charged groups) on a regular grid, float32 of the given shape."""
    rng = np.random.default_rng(seed)
    axes = [origin[a] + spacing[a] * np.arange(shape[a]) for a in range(3)]
    gx, gy, gz = np.meshgrid(*axes, indexing="ij")
    lo = np.array(origin, np.float64)
    hi = lo + np.array(spacing, np.float64) * np.array(shape)
    out = np.zeros(tuple(shape), np.float64)
    for _ in range(centres):
        c = rng.uniform(lo, hi)
        w = rng.uniform(0.15, 0.35) * float(np.min(hi - lo))
        out += rng.choice([-1.0, 1.0]) * amplitude * np.exp(-((gx - c[0]) ** 2 + (gy - c[1]) ** 2 + (gz - c[2]) ** 2)
                                                             / (2.0 * w * w))
    return out.astype(np.float32)


def write_dx(path: str, scalar: np.ndarray, origin, spacing) -> None:
    """Writes a scalar map as an OpenDX regular grid (the layout OpenDXReader reads: counts,
    origin, three delta lines, two object lines, then the values three per line, z fastest).
    Values are printed with 9 significant digits, so float32 values read back exactly."""
    sc = np.ascontiguousarray(scalar, np.float32)
    n0, n1, n2 = sc.shape
    with open(path, "w") as f:
        f.write("# synthetic map\n")
        f.write(f"object 1 class gridpositions counts {n0} {n1} {n2}\n")
        f.write("origin {:.9g} {:.9g} {:.9g}\n".format(*origin))
        f.write(f"delta {spacing[0]:.9g} 0 0\ndelta 0 {spacing[1]:.9g} 0\ndelta 0 0 {spacing[2]:.9g}\n")
        f.write(f"object 2 class gridconnections counts {n0} {n1} {n2}\n")
        f.write(f'object 3 class array type double rank 0 items {sc.size} data follows\n')
        flat = sc.reshape(-1)
        for i in range(0, flat.size, 3):
            f.write(" ".join(f"{v:.9g}" for v in flat[i:i + 3]) + "\n")
        f.write('attribute "dep" string "positions"\n')
        f.write('object "regular positions regular connections" class field\n')
        f.write('component "positions" value 1\ncomponent "connections" value 2\ncomponent "data" value 3\n')
