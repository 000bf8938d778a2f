"""Generates the golden fixtures of tests/golden/ by running the compiled reference.

Run where the reference sources are present (they are compiled by oracle/ref.mk into
oracle/_ref/libbsref.so):

    python tests/golden/make_golden.py

Each fixture holds the inputs of a small seeded system and the reference's outputs for it.
The reference is run single-threaded (OMP_NUM_THREADS=1) so that its kinetic-energy
reduction has the serial order.

Fixtures:
  scans.npz       two-particle distance scans of the reference's regression tests
                  (src/tests/regression/test-{spring,steric,electrostatic,hydrophobic}-energy.cpp):
                  x from 0.01 while x < 5, x += 0.01 in float, energy and force per point
  ca300.npz       300-particle Calpha network: positions/velocities/energies after 1, 10, 30 steps
  mixed_m{0..3}.npz  800 particles, all nonbonded terms, static particles, IMPALA, one per steric
                  mode: forces and energies at the start, state after 3 steps; pair sets and cell
                  ids of each term (mixed_m1 only; pairs do not depend on the steric mode)
  rigid1.npz      one rigid body made of every dynamic particle (SpringNetwork::run,
                  SpringNetwork.cpp:281-292): positions after 20 steps
  nsearch.npz     1000 random particles in [-100, 100]^3, steric cutoff 10: the neighbour pairs
                  (src/tests/test-nsearch.cpp:103-129)
  fields.npz      a charged 300-particle network with Coulomb under an electrostatic potential
                  map and a density map read from OpenDX files (potentialgrid.*, densitygrid.*),
                  per-particle burying: the reference's grid cells (scalar, force vector), forces
                  and energies at the start, positions and energies after 1, 10 and 30 steps of a
                  fresh handle
  membrane.npz    a 600-bead globule (displaced 0.2 A off its springs' rest lengths) with springs,
                  IMPALA and viscosity under three double-membrane
                  settings (offsets and tube curvatures of ForceField::setImpDoubleMembrane*):
                  forces and energies at the start, positions and energies after 5 steps
  probe.npz       a charged 300-particle network with LJ 12-6 Amber and Coulomb, and the probe
                  particle (probe.*, SpringNetwork.cpp:156-182) steric and electrostatic on:
                  positions, probe state and energies after 1, 10 and 30 steps

Usage: python tests/golden/make_golden.py [fixture ...]   (default: all; names without .npz)
"""

from __future__ import annotations

import os
import sys

os.environ["OMP_NUM_THREADS"] = "1"
HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

import numpy as np  # noqa: E402

from biospring_gb300 import build, capi, workloads as W  # noqa: E402
from oracle import pyoracle as po  # noqa: E402


def scan_x() -> np.ndarray:
    xs = []
    x = np.float32(0.01)
    while x < 5:
        xs.append(x)
        x = np.float32(float(x) + 0.01)
    return np.array(xs, dtype=np.float32)


def two_particle(config: dict, **props) -> W.System:
    xyz = np.zeros((2, 3), np.float32)
    ij = props.pop("ij", np.zeros((0, 2), np.int32))
    r0 = props.pop("r0", np.zeros(0, np.float32))
    k = props.pop("k", np.zeros(0, np.float32))
    return W.System("two", xyz, ij, r0, k, config, **props)


def make_scans(out: dict) -> None:
    xs = scan_x()
    out["x"] = xs
    cc = dict(charge=np.full(2, 0.5973, np.float32), radius=np.full(2, 1.908, np.float32),
              epsilon=np.full(2, 0.086, np.float32), mass=np.full(2, 12.01, np.float32))
    base = dict(nbsteps=1, timestep=0.01)
    cases = {
        "spring": dict(config=dict(base, spring_enable=1), ij=np.array([[0, 1]], np.int32),
                       r0=np.zeros(1, np.float32), k=np.ones(1, np.float32), **cc),
        "steric_linear": dict(config=dict(base, steric_enable=1, steric_cutoff=16.0, steric_mode=0), **cc),
        "steric_amber": dict(config=dict(base, steric_enable=1, steric_cutoff=16.0, steric_mode=1), **cc),
        "coulomb": dict(config=dict(base, coulomb_enable=1, coulomb_cutoff=16.0, coulomb_dielectric=1.0), **cc),
        "hydrophobic": dict(config=dict(base, hydrophobicity_enable=1, hydrophobicity_cutoff=16.0),
                            hydrophobicity=np.array([0.5, 0.3], np.float32)),
    }
    for name, spec in cases.items():
        cfg = dict(spec.pop("config"))
        sysm = two_particle(cfg, **spec)
        ref = po.Reference(sysm)
        energies = np.zeros((xs.size, 6), np.float64)
        forces = np.zeros((xs.size, 2, 3), np.float32)
        for t, x in enumerate(xs):
            xyz = np.array([[0, 0, 0], [x, 0, 0]], np.float32)
            ref.set_positions(xyz)
            ref.compute_forces()
            energies[t] = ref.energies()
            forces[t] = ref.forces()
        out[f"{name}_energy"] = energies
        out[f"{name}_force"] = forces
        ref.close()


def system_arrays(prefix: str, s: W.System, out: dict) -> None:
    for key, v in s.arrays().items():
        if v is not None:
            out[f"{prefix}{key}"] = v
    out[f"{prefix}ij"] = s.ij
    out[f"{prefix}r0"] = s.r0
    out[f"{prefix}k"] = s.k
    cfg = s.bs_config()
    out[f"{prefix}config"] = np.array([repr(cfg.to_dict())])


def make_ca300() -> dict:
    s = W.ca_network(n=300, seed=5)
    out: dict = {}
    system_arrays("in_", s, out)
    ref = po.Reference(s)
    done = 0
    for mark in (1, 10, 30):
        ref.step(mark - done)
        done = mark
        out[f"pos_{mark}"] = ref.positions()
        out[f"vel_{mark}"] = ref.velocities()
        out[f"energy_{mark}"] = ref.energies()
    ref.close()
    return out


def mixed_system(mode: int) -> W.System:
    s = W.uniform_lj(n=800, box=32.0, seed=17)
    s.config["steric_mode"] = mode
    rng = np.random.default_rng(23)
    h = np.zeros(s.n, np.float32)
    idx = rng.choice(s.n, 160, replace=False)
    h[idx] = rng.uniform(-1, 1, 160).astype(np.float32)
    s.hydrophobicity = h
    s.sasa = rng.uniform(0, 60, s.n).astype(np.float32)
    s.transfer = rng.uniform(-0.05, 0.05, s.n).astype(np.float32)
    st = np.zeros(s.n, np.uint8)
    st[rng.choice(s.n, 40, replace=False)] = 1
    s.is_static = st
    s.xyz = (s.xyz - np.float32(16.0)).astype(np.float32)
    s.config.update(hydrophobicity_enable=1, hydrophobicity_cutoff=9.0, impala_enable=1, viscosity_enable=1,
                    viscosity_value=0.5)
    return s


def make_mixed(mode: int) -> dict:
    s = mixed_system(mode)
    out: dict = {}
    system_arrays("in_", s, out)
    ref = po.Reference(s)
    ref.compute_forces()
    out["force0"] = ref.forces()
    out["energy0"] = ref.energies()
    ref.close()
    ref = po.Reference(s)
    if mode == 1:
        for term in (0, 1, 2):
            out[f"pairs{term}"] = ref.pairs(term).astype(np.int32)
            out[f"cells{term}"] = ref.cells(term).astype(np.int32)
    ref.step(3)
    out["pos3"] = ref.positions()
    out["vel3"] = ref.velocities()
    out["energy3"] = ref.energies()
    ref.close()
    return out


def make_rigid() -> dict:
    s = W.membrane_globule(n=200, seed=4)
    s.config["rigidbody_enable"] = 1
    s.bodies = [np.arange(s.n, dtype=np.int32)]
    out: dict = {}
    system_arrays("in_", s, out)
    ref = po.Reference(s)
    ref.step(20)
    out["pos20"] = ref.positions()
    out["energy20"] = ref.energies()
    ref.close()
    return out


# upper offset, lower offset, upper curvature, lower curvature
MEMBRANES = np.array([[20.0, 20.0, 0.0, 0.0], [12.0, 14.0, 0.02, -0.015], [0.0, 25.0, 0.0, 0.03]], np.float32)


def membrane_system() -> W.System:
    s = W.membrane_globule(n=600, seed=6)
    s.config.update(viscosity_value=0.5)
    # off the springs' rest lengths, so that spring forces are real forces and not rounding residue
    s.xyz = (s.xyz + np.random.default_rng(8).normal(0.0, 0.2, s.xyz.shape)).astype(np.float32)
    return s


def make_membrane() -> dict:
    s = membrane_system()
    out: dict = {"membranes": MEMBRANES}
    system_arrays("in_", s, out)
    for k, m in enumerate(MEMBRANES):
        ref = po.Reference(s)
        ref.set_membrane(*m)
        ref.compute_forces()
        out[f"force0_{k}"] = ref.forces()
        out[f"energy0_{k}"] = ref.energies()
        ref.close()
        ref = po.Reference(s)
        ref.set_membrane(*m)
        ref.step(5)
        out[f"pos5_{k}"] = ref.positions()
        out[f"energy5_{k}"] = ref.energies()
        ref.close()
    return out


def probe_system() -> W.System:
    s = W.ca_network(n=300, seed=5)
    rng = np.random.default_rng(3)
    s.charge = np.where(rng.random(s.n) < 0.3, rng.choice([-1.0, 1.0], s.n), 0.0).astype(np.float32)
    s.radius = rng.uniform(1.5, 2.0, s.n).astype(np.float32)
    s.epsilon = rng.uniform(0.2, 0.5, s.n).astype(np.float32)
    s.config.update(steric_mode=1, coulomb_enable=1, coulomb_cutoff=12.0, coulomb_dielectric=4.0,
                    probe_enable=1, probe_steric=1, probe_electrostatic=1, probe_x=2.0, probe_y=-1.0,
                    probe_z=3.0, probe_charge=1.0, probe_radius=2.5, probe_epsilon=0.8, probe_mass=5.0,
                    timestep=0.05)
    return s


def make_probe() -> dict:
    s = probe_system()
    out: dict = {}
    system_arrays("in_", s, out)
    ref = po.Reference(s)
    done = 0
    for mark in (1, 10, 30):
        ref.step(mark - done)
        done = mark
        out[f"pos_{mark}"] = ref.positions()
        out[f"probe_{mark}"] = ref.probe()
        out[f"energy_{mark}"] = ref.energies()
    ref.close()
    return out


FIELD_GRIDS = {  # which: (shape, origin, spacing, seed); part of the network lies outside each box
    0: ((23, 19, 17), (-14.25, -12.5, -9.75), (1.5, 1.75, 1.25), 11),
    1: ((15, 16, 14), (-18.0, -20.5, -12.0), (2.0, 2.0, 2.25), 12),
}


def fields_system() -> W.System:
    s = W.ca_network(n=300, seed=5)
    rng = np.random.default_rng(7)
    s.charge = np.where(rng.random(s.n) < 0.3, rng.choice([-1.0, 1.0], s.n), 0.0).astype(np.float32)
    s.config.update(coulomb_enable=1, coulomb_cutoff=12.0, coulomb_dielectric=4.0, potentialgrid_enable=1,
                    potentialgrid_scale=1.5, densitygrid_enable=1, densitygrid_scale=0.7, timestep=0.05)
    return s


def make_fields() -> dict:
    """A charged 300-particle network under an electrostatic potential map and a density map
    (potentialgrid.*, densitygrid.*; Particle.cpp:136-189), both read by the reference's OpenDX
    reader from files written here; per-particle burying in [0, 2)."""
    import tempfile
    s = fields_system()
    rng = np.random.default_rng(8)
    burying = rng.uniform(0.0, 2.0, s.n).astype(np.float32)
    out: dict = {}
    with tempfile.TemporaryDirectory() as tmp:
        for which, (shape, origin, spacing, seed) in FIELD_GRIDS.items():
            sc = W.field_map(shape, origin, spacing, seed, amplitude=20000.0 if which == 0 else 5000.0)
            path = os.path.join(tmp, f"grid{which}.dx")
            W.write_dx(path, sc, origin, spacing)
            out[f"grid{which}"] = sc
            out[f"grid{which}_origin"] = np.array(origin, np.float64)
            out[f"grid{which}_spacing"] = np.array(spacing, np.float64)
            s.config["potentialgrid_path" if which == 0 else "densitygrid_path"] = path.encode()
        ref = po.Reference(s)
        for key in ("potentialgrid_path", "densitygrid_path"):
            s.config[key] = b""
        system_arrays("in_", s, out)
        out["burying"] = burying
        ref.set_burying(burying)
        out["cells0"] = ref.field_grid(0)
        out["cells1"] = ref.field_grid(1)
        ref.compute_forces()
        out["forces_0"] = ref.forces()
        out["energy_0"] = ref.energies()
        ref.close()
        # the trajectory from a fresh handle: the reference's force evaluation leaves its forces
        # in the particles, where the next step would add to them
        for key, which in (("potentialgrid_path", 0), ("densitygrid_path", 1)):
            s.config[key] = os.path.join(tmp, f"grid{which}.dx").encode()
        ref = po.Reference(s)
        for key in ("potentialgrid_path", "densitygrid_path"):
            s.config[key] = b""
        ref.set_burying(burying)
        done = 0
        for mark in (1, 10, 30):
            ref.step(mark - done)
            done = mark
            out[f"pos_{mark}"] = ref.positions()
            out[f"energy_{mark}"] = ref.energies()
        ref.close()
    return out


def make_nsearch() -> dict:
    rng = np.random.default_rng(1000)
    xyz = rng.uniform(-100, 100, size=(1000, 3)).astype(np.float32)
    s = W.System("nsearch", xyz, np.zeros((0, 2), np.int32), np.zeros(0, np.float32), np.zeros(0, np.float32),
                 dict(steric_enable=1, steric_cutoff=10.0))
    out: dict = {}
    system_arrays("in_", s, out)
    ref = po.Reference(s)
    out["pairs0"] = ref.pairs(0).astype(np.int32)
    out["cells0"] = ref.cells(0).astype(np.int32)
    ref.close()
    return out


def main() -> None:
    build.build_synth()
    if not po.build_reference():
        raise SystemExit("the reference sources are not present: cannot generate golden fixtures")
    makers = {"scans": None, "ca300": make_ca300, "rigid1": make_rigid, "nsearch": make_nsearch,
              "probe": make_probe, "fields": make_fields, "membrane": make_membrane}
    for mode in range(4):
        makers[f"mixed_m{mode}"] = (lambda m: (lambda: make_mixed(m)))(mode)
    wanted = sys.argv[1:] or list(makers)
    for name in wanted:
        if name == "scans":
            scans: dict = {}
            make_scans(scans)
            np.savez_compressed(os.path.join(HERE, "scans.npz"), **scans)
        else:
            np.savez_compressed(os.path.join(HERE, f"{name}.npz"), **makers[name]())
    for f in sorted(os.listdir(HERE)):
        if f.endswith(".npz"):
            print(f, os.path.getsize(os.path.join(HERE, f)))


if __name__ == "__main__":
    main()
