"""Parity at the full sizes of the five benchmark configurations, through the C ABI.

* 100,000 particles (the bench system: uniform fill of a 160 A cube, springs < 5 A, 20% charged,
  LJ 12-6 Amber and Coulomb at 12 A), in both dielectric modes: after the first list build and
  again after 12 steps (one rebuild on the way), with the oracle put in the GPU's state, forces
  within 1e-5 relative L2, energies within 1e-5, steric and Coulomb pair sets and cell ids bit-exact;
  the 12-step trajectories side by side. Two more 100k systems reach the list build's other paths:
  a flat slab whose neighbour offsets leave the 16-bit range (32-bit steric rows) and a cube with a
  core at twice the density, whose rows overflow the first capacity (lists regrown).
* 2,000-particle Calpha network for the full 1,000 steps.
* 20,000-bead membrane globule with four rigid bodies of 500 beads, IMPALA at the reference's
  Z0 = 15.75 A and at 15 A (the restatement), the reference time step, 200 steps.
* The 512-system ensemble of the bench, each system against the same system stepped alone.

Bars: forces 1e-5 relative L2 (the error of the GPU and of the FP32 restatement against FP64 are
printed beside it); pair sets and cells bit-exact; energies 1e-5 relative, or the FP32
restatement's own distance to FP64 when that is larger (its serial FP32 sums over millions of
pairs can be further from the exact value than the GPU's compensated sums), plus 1e-6 kJ/mol
absolute (a spring energy at rest is a sum of rounding residues of order 1e-8 kJ/mol).
"""

from __future__ import annotations

import os

import numpy as np
import pytest

from biospring_gb300 import capi
from biospring_gb300 import workloads as W
from helpers import dynamic_mask, gpu_network, rel_l2, rel_scalar
from oracle import pyoracle as po

pytestmark = pytest.mark.gpu
os.environ.setdefault("OMP_NUM_THREADS", str(os.cpu_count() or 1))

FORCE_TOL = 1e-5
ENERGY_TOL = 1e-5
E_FLOOR = 1e-6  # kJ/mol
E_STERIC, E_COULOMB, E_SPRING = 2, 3, 1  # oracle energy order: kinetic, spring, steric, electrostatic, imp, hydro


def _energies(net):
    return np.array(list(net.energies().values()))


def _check_state(net, orc, label, terms=(0, 1), near_equilibrium=False):
    """Forces, energies, pair sets and cells of the GPU against the oracle at the same state.

    near_equilibrium: the forces are sums of spring forces that nearly cancel, so the FP32
    reference arithmetic itself sits further than the force bar from FP64; the GPU is then held
    to no more than twice the reference arithmetic's own distance to FP64."""
    net.computeForces()
    orc.compute_forces()
    f_gpu, f_orc = net.getForces(), orc.forces()
    f64, e64 = orc.eval_fp64()
    err = rel_l2(f_gpu, f_orc)
    gerr, own = rel_l2(f_gpu, f64), rel_l2(f_orc, f64)
    print(f"{label}: forces vs oracle {err:.3e}, GPU vs FP64 {gerr:.3e}, oracle vs FP64 {own:.3e}")
    if near_equilibrium:
        assert own > FORCE_TOL and gerr <= 2.0 * own
    else:
        assert err <= FORCE_TOL
    e_gpu, e_orc = _energies(net), orc.energies()
    for k in (E_SPRING, E_STERIC, E_COULOMB):
        if e_orc[k] == 0.0:
            continue
        print(f"  energy {k}: GPU {e_gpu[k]:.9g} oracle {e_orc[k]:.9g} FP64 {e64[k]:.9g}")
        assert _energy_ok(e_gpu, e_orc, e64, k), (label, k)
    for term in terms:
        pg, po_ = net.getPairs(term), orc.pairs(term).astype(np.int64)
        print(f"  term {term}: {pg.shape[0]} pairs")
        np.testing.assert_array_equal(pg, po_)
        np.testing.assert_array_equal(net.getCells(term), orc.cells(term))


def _energy_ok(e_gpu, e_orc, e64, k):
    """|GPU - oracle| within 1e-5 relative, or the FP32 oracle's own distance to FP64 when that is
    larger, plus the absolute floor."""
    tol = max(ENERGY_TOL * abs(e_orc[k]), abs(e_orc[k] - e64[k]) + 1e-6 * abs(e_orc[k])) + E_FLOOR
    return abs(e_gpu[k] - e_orc[k]) <= tol


def _fresh(s):
    """An oracle that has not evaluated forces yet: the reference's computeForces leaves its forces
    in the particles' accumulators, where the next step would add them again."""
    return po.Oracle(s)


def _sync_oracle(net, orc):
    orc.set_positions(net.getPositions())
    orc.set_velocities(net.getVelocities())


@pytest.mark.parametrize("dielectric_mode", [0, 1], ids=["eps4", "eps4r"])
def test_bench_system_100k(dielectric_mode):
    import bench
    s = W.uniform_lj(n=100_000, box=160.0, seed=42, dielectric_mode=dielectric_mode, rebuild_every=10,
                     list_skin=bench.LIST_SKIN)
    net = gpu_network(s)
    orc = po.Oracle(s)
    _check_state(net, orc, f"100k eps mode {dielectric_mode}, first build")
    orc.close()
    orc = _fresh(s)
    net.computeStep(12)
    orc.step(12)
    dx = float(np.abs(net.getPositions().astype(np.float64) - orc.positions()).max())
    dv = rel_l2(net.getVelocities(), orc.velocities())
    print(f"after 12 steps: max |dx| {dx:.3e} A, velocity rel L2 {dv:.3e}")
    assert dx < 1e-5 and dv < 1e-4
    _sync_oracle(net, orc)
    _check_state(net, orc, f"100k eps mode {dielectric_mode}, after 12 steps")
    net.close()
    orc.close()


def _lattice(shape, spacing, jitter, seed):
    rng = np.random.default_rng(seed)
    axes = [np.arange(m, dtype=np.float64) * spacing for m in shape]
    xyz = np.stack(np.meshgrid(*axes, indexing="ij"), -1).reshape(-1, 3)
    return (xyz + rng.uniform(-jitter, jitter, xyz.shape)).astype(np.float32)


def _lj_system(name, xyz, seed):
    n = xyz.shape[0]
    ij = W.pairs_within(xyz, 5.0)
    d = xyz[ij[:, 1]].astype(np.float64) - xyz[ij[:, 0]].astype(np.float64)
    r0 = np.sqrt((d * d).sum(1)).astype(np.float32)
    rng = np.random.default_rng(seed)
    k = np.exp(rng.uniform(np.log(0.1), np.log(10.0), ij.shape[0])).astype(np.float32)
    charge = np.zeros(n, np.float32)
    q = rng.choice(n, n // 5 // 2 * 2, replace=False)
    charge[q[: q.size // 2]] = 1.0
    charge[q[q.size // 2:]] = -1.0
    cfg = dict(timestep=0.01, spring_enable=1, steric_enable=1, steric_cutoff=12.0,
               steric_mode=capi.BS_STERIC_LJ_12_6_AMBER, coulomb_enable=1, coulomb_cutoff=12.0,
               coulomb_dielectric=4.0, dielectric_mode=0, rebuild_every=10, list_skin=0.5)
    return W.System(name, xyz, ij, r0, k, cfg, charge=charge, radius=np.full(n, 3.5, np.float32),
                    epsilon=np.full(n, 0.2 * W.KCAL_TO_KJ, np.float32))


def test_flat_slab_100k_wide_offsets():
    """A 400 x 400 x 24 A slab at the bench density (jittered 3.45 A lattice, 116 x 116 x 8 =
    107,648 particles): a z-layer of search cells holds about 25k particles, so partners two layers
    apart sit more than 32,767 slots away and the steric rows fall back to 32-bit entries."""
    s = _lj_system("slab", _lattice((116, 116, 8), 3.45, 0.3, 5), 6)
    net = gpu_network(s)
    orc = po.Oracle(s)
    _check_state(net, orc, "slab 108k, first build")
    orc.close()
    orc = _fresh(s)
    net.computeStep(12)
    orc.step(12)
    assert float(np.abs(net.getPositions().astype(np.float64) - orc.positions()).max()) < 1e-5
    _sync_oracle(net, orc)
    _check_state(net, orc, "slab 108k, after 12 steps")
    net.close()
    orc.close()


def test_dense_core_100k_regrows_lists():
    """The 160 A cube at the bench density with a 60 A core filled at twice it (minimum separation
    2 A there): core rows hold about twice the partners the first capacity expects from the mean
    density, so the first build overflows and the lists are regrown before any force is used."""
    core = W.rsa_fill(10_600, 60.0, 2.0, 31) + np.float32(50.0)
    outer = W.rsa_fill(90_000, 160.0, 3.0, 32)
    lo, hi = 50.0 - 3.0, 110.0 + 3.0
    keep = ~np.all((outer > lo) & (outer < hi), axis=1)
    xyz = np.concatenate([outer[keep], core]).astype(np.float32)
    s = _lj_system("dense core", xyz, 33)
    net = gpu_network(s)
    orc = po.Oracle(s)
    _check_state(net, orc, f"dense core {s.n}, first build")
    orc.close()
    orc = _fresh(s)
    net.computeStep(12)
    orc.step(12)
    _sync_oracle(net, orc)
    _check_state(net, orc, f"dense core {s.n}, after 12 steps")
    net.close()
    orc.close()


def test_ca_network_2000_full_1000_steps():
    """Forces at the kicked start state under the plain bar; after 1,000 damped steps the network
    is near equilibrium (spring forces cancel), and its forces are held against FP64 instead."""
    s = W.ca_network(n=2000, seed=1)
    net = gpu_network(s)
    orc = po.Oracle(s)
    _check_state(net, orc, "ca2000 at the start", terms=(0,))
    orc.close()
    orc = _fresh(s)
    for mark in (200, 1000):
        net.computeStep(mark - (200 if mark == 1000 else 0))
        orc.step(mark - (200 if mark == 1000 else 0))
        dx = float(np.abs(net.getPositions().astype(np.float64) - orc.positions()).max())
        e_gpu, e_orc = _energies(net), orc.energies()
        print(f"ca2000 step {mark}: max |dx| {dx:.3e} A, spring energy {e_gpu[1]:.9g} vs {e_orc[1]:.9g}, "
              f"kinetic {e_gpu[0]:.6g} vs {e_orc[0]:.6g}")
        assert dx < 1e-3
        assert rel_scalar(e_gpu[1], e_orc[1]) < 1e-4
    _sync_oracle(net, orc)
    _check_state(net, orc, "ca2000 after 1000 steps", terms=(0,), near_equilibrium=True)
    net.close()
    orc.close()


@pytest.mark.parametrize("z0", [15.75, 15.0])
def test_membrane_20k_four_bodies(z0):
    s = W.membrane_globule(n=20_000, seed=3, nbodies=4, body_size=500, z0=z0)
    assert s.config["timestep"] == 0.01
    free = np.ones(s.n, bool)
    for ids in s.bodies:
        free[ids] = False
    s.xyz = s.xyz.copy()
    s.xyz[free] += np.random.default_rng(2).normal(0.0, 0.3, (int(free.sum()), 3)).astype(np.float32)
    net = gpu_network(s)
    orc = po.Oracle(s)
    net.computeForces()
    orc.compute_forces()
    f_gpu, f_orc = net.getForces(), orc.forces()
    err = rel_l2(f_gpu, f_orc, dynamic_mask(s))
    imp_g, imp_o = _energies(net)[4], orc.energies()[4]
    print(f"Z0 {z0}: forces vs oracle {err:.3e}, IMPALA energy {imp_g:.9g} vs {imp_o:.9g}")
    assert err <= FORCE_TOL
    assert rel_scalar(imp_g, imp_o) < ENERGY_TOL
    orc.close()
    orc = _fresh(s)
    for mark in (50, 200):
        net.computeStep(mark - (50 if mark == 200 else 0))
        orc.step(mark - (50 if mark == 200 else 0))
        x, xo = net.getPositions().astype(np.float64), orc.positions().astype(np.float64)
        dx = float(np.abs(x - xo).max())
        e, eo = _energies(net), orc.energies()
        assert dx < 2e-5
        assert rel_scalar(e[0], eo[0]) < 1e-4  # kinetic: FP32 sums of per-particle terms on both sides
        # A step's energies are taken at the positions before its update; the potential energies
        # are checked at the current state instead, against FP64 (the FP32 oracle's serial sum of
        # some 2e5 spring energies is itself 1e-4 from the exact value here).
        net.computeForces()
        eg = _energies(net)
        _, e64 = orc.eval_fp64()
        print(f"Z0 {z0}, step {mark}: max |dx| {dx:.2e} A, energies {eg} vs FP64 {e64} (oracle's last step {eo})")
        for k in range(1, 6):
            assert abs(eg[k] - e64[k]) <= ENERGY_TOL * abs(e64[k]) + E_FLOOR, (mark, k, eg[k], e64[k])
    net.close()
    orc.close()


def test_membrane_z0_moves_the_force():
    """The half-thickness reaches the force: a bead at |z| = 15.4 A sits outside a 15 A membrane
    and inside a 15.75 A one, so the IMPALA force on it differs between the two."""
    xyz = np.array([[0.0, 0.0, 15.4], [40.0, 0.0, 0.0]], np.float32)
    out = []
    for z0 in (15.75, 15.0):
        s = W.System("bead", xyz, np.zeros((0, 2), np.int32), np.zeros(0, np.float32), np.zeros(0, np.float32),
                     dict(timestep=0.01, impala_enable=1, impala_z0=z0), sasa=np.full(2, 50.0, np.float32),
                     transfer=np.full(2, 0.03, np.float32))
        net = gpu_network(s)
        net.computeForces()
        orc = po.Oracle(s)
        orc.compute_forces()
        assert rel_l2(net.getForces(), orc.forces()) <= FORCE_TOL
        out.append(net.getForces()[0, 2])
        net.close()
        orc.close()
    assert out[0] != out[1] and np.sign(out[0]) != 0


def test_bench_ensemble_every_system_matches_single_path():
    """All 512 networks of the bench ensemble (sizes log-uniform in 200..20,000, seed 2024),
    stepped 20 times by the persistent kernel with the autotuned shape, against each network
    stepped alone through the single-system path."""
    ens = W.ensemble(W.ensemble_sizes(), seed=2024)
    off = ens.meta["offsets"]
    nsys = len(off) - 1
    from biospring_gb300 import SpringNetwork
    net = SpringNetwork()
    net.addParticles(xyz=ens.xyz)
    net.addSprings(ens.ij, ens.r0, ens.k)
    net.setSystems(off)
    net.setup(ens.bs_config())
    shape = net.batchAutotune()  # trials step copies of the state; the state is put back after each
    net.computeStep(20)
    pos = net.getPositions()
    energies = net.getSystemEnergies()
    net.close()
    worst_dx, worst_e = 0.0, 0.0
    for b in range(nsys):
        i0, i1 = int(off[b]), int(off[b + 1])
        m = (ens.ij[:, 0] >= i0) & (ens.ij[:, 0] < i1)
        part = W.System(f"part{b}", ens.xyz[i0:i1].copy(), (ens.ij[m] - i0).astype(np.int32), ens.r0[m].copy(),
                        ens.k[m].copy(), dict(ens.config))
        h = gpu_network(part)
        h.computeStep(20)
        dx = float(np.abs(h.getPositions().astype(np.float64) - pos[i0:i1]).max())
        e = _energies(h)
        worst_dx = max(worst_dx, dx)
        assert dx < 1e-5, (b, dx)
        for k in range(6):
            if e[k] != 0.0:
                r = rel_scalar(energies[b, k], e[k])
                worst_e = max(worst_e, r)
                assert r < 1e-5, (b, k, energies[b, k], e[k])
            else:
                assert abs(energies[b, k]) < 1e-9
        h.close()
    print(f"{nsys} systems, shape {shape}: worst |dx| {worst_dx:.2e} A, worst energy rel {worst_e:.2e}")
