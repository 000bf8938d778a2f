"""Batched ensembles: every system of a batch against the same system stepped alone.

A batch handle (bs_set_systems + the persistent clustered step kernel) must give each system the
trajectory and energies the single-system path gives it, for every launch shape the autotuner
may pick, across list rebuilds and early stops on stale lists.
"""

from __future__ import annotations

import numpy as np
import pytest

from biospring_gb300 import BsError, SpringNetwork
from biospring_gb300 import workloads as W
from helpers import gpu_network, rel_scalar

pytestmark = pytest.mark.gpu

SIZES = [200, 357, 820, 1500, 2900, 5200]
POS_TOL = 1e-5      # A, after the steps below (both paths FP32, same force routine)
ENERGY_TOL = 1e-5   # relative, per system and term


def _batch(system, offsets, config=None, shape=None):
    net = SpringNetwork()
    net.addParticles(**{k: v for k, v in system.arrays().items() if v is not None})
    net.addSprings(system.ij, system.r0, system.k)
    net.setSystems(offsets)
    if shape is not None:
        net.setBatchShape(*shape)
    net.setup(system.bs_config() if config is None else config)
    return net


def _part(system, offsets, b):
    """System b of an ensemble as a stand-alone System."""
    i0, i1 = int(offsets[b]), int(offsets[b + 1])
    m = (system.ij[:, 0] >= i0) & (system.ij[:, 0] < i1)
    return W.System(f"part{b}", system.xyz[i0:i1].copy(), (system.ij[m] - i0).astype(np.int32),
                    system.r0[m].copy(), system.k[m].copy(), dict(system.config))


def _alone(system, offsets, nsteps, config_update=None):
    pos, energies = [], []
    for b in range(len(offsets) - 1):
        part = _part(system, offsets, b)
        if config_update:
            part.config.update(config_update)
        net = gpu_network(part)
        net.computeStep(nsteps)
        pos.append(net.getPositions())
        energies.append(np.array(list(net.energies().values())))
        net.close()
    return np.concatenate(pos), np.stack(energies)


@pytest.fixture(scope="module")
def ensemble():
    return W.ensemble(SIZES, seed=77)


@pytest.mark.parametrize("shape", [(256, 4, 1), (128, 2, 2), (512, 8, 4), (256, 4, 8), (128, 1, 1)],
                         ids=lambda s: f"b{s[0]}-t{s[1]}-c{s[2]}")
def test_batch_matches_single_systems(ensemble, shape):
    off = ensemble.meta["offsets"]
    nsteps = 40  # four rebuild periods
    ref_pos, ref_e = _alone(ensemble, off, nsteps)
    net = _batch(ensemble, off, shape=shape)
    assert net.batchShape() == shape
    net.computeStep(nsteps)
    pos = net.getPositions()
    e = net.getSystemEnergies()
    dx = float(np.abs(pos.astype(np.float64) - ref_pos).max())
    print(f"shape {shape}: max |dx| vs single systems {dx:.3e} A")
    assert dx < POS_TOL
    for b in range(len(SIZES)):
        for k in range(6):
            if ref_e[b, k] != 0.0:
                assert rel_scalar(e[b, k], ref_e[b, k]) < ENERGY_TOL, (b, k, e[b, k], ref_e[b, k])
            else:
                assert abs(e[b, k]) < 1e-12
    tot = net.energies()
    assert rel_scalar(tot["spring"], float(ref_e[:, 1].sum())) < ENERGY_TOL
    net.close()


def test_batch_steps_in_pieces_and_forces(ensemble):
    """Steps split across calls follow the same rebuild schedule; forces on the concatenation."""
    off = ensemble.meta["offsets"]
    a = _batch(ensemble, off)
    a.computeStep(25)
    b = _batch(ensemble, off)
    for n in (7, 3, 10, 5):
        b.computeStep(n)
    assert a.getPositions().tobytes() == b.getPositions().tobytes()
    a.computeForces()
    f = a.getForces()
    assert np.all(np.isfinite(f))
    a.close()
    b.close()


def test_batch_stale_lists_catch_up(ensemble):
    """A long timestep and a thin skin make systems stop early on stale lists; every system still
    completes the requested steps and stays close to its stand-alone trajectory."""
    off = ensemble.meta["offsets"]
    upd = dict(timestep=0.5, list_skin=0.05, viscosity_value=0.5)
    cfg = dict(ensemble.config)
    cfg.update(upd)
    sysm = W.System(ensemble.name, ensemble.xyz, ensemble.ij, ensemble.r0, ensemble.k * 50.0, cfg,
                    meta=ensemble.meta)
    nsteps = 30
    ref_pos, _ = _alone(sysm, off, nsteps)
    net = _batch(sysm, off)
    net.computeStep(nsteps)
    assert net.stepCount() == nsteps
    pos = net.getPositions()
    moved = float(np.abs(pos.astype(np.float64) - sysm.xyz).max())
    dx = float(np.abs(pos.astype(np.float64) - ref_pos).max())
    print(f"stale run: max move {moved:.3f} A, max |dx| vs single systems {dx:.3e} A")
    assert moved > 0.05  # the skin was crossed
    assert dx < 1e-3
    net.close()


def test_batch_autotune_keeps_state(ensemble):
    off = ensemble.meta["offsets"]
    net = _batch(ensemble, off)
    net.computeStep(10)
    before = net.getPositions()
    shape = net.batchAutotune()
    assert shape[0] in (128, 256, 512) and shape[1] in (2, 4, 8) and shape[2] in (1, 2, 4, 8)
    assert net.getPositions().tobytes() == before.tobytes()
    net.computeStep(10)
    ref = _batch(ensemble, off, shape=shape)
    ref.computeStep(20)
    assert np.abs(net.getPositions().astype(np.float64) - ref.getPositions()).max() < POS_TOL
    net.close()
    ref.close()


def test_batch_rejections(ensemble):
    off = ensemble.meta["offsets"]
    net = _batch(ensemble, off)
    with pytest.raises(BsError):
        net.setForce(0, [1.0, 0.0, 0.0])
    with pytest.raises(BsError):
        net.getPairs(0)
    with pytest.raises(BsError):
        net.setBatchShape(96, 4, 1)
    net.close()
    bad = SpringNetwork()
    bad.addParticles(ensemble.xyz[:400])
    bad.addSprings(np.array([[10, 300]], np.int32), np.array([5.0], np.float32), np.array([1.0], np.float32))
    bad.setSystems([0, 200, 400])
    with pytest.raises(BsError, match="two systems"):
        bad.setup(ensemble.bs_config())
    bad.close()
    grid = SpringNetwork()
    grid.addParticles(ensemble.xyz[:400])
    grid.setSystems([0, 200, 400])
    cfg = ensemble.bs_config()
    cfg.densitygrid_enable = 1
    with pytest.raises(BsError, match="field grids"):
        grid.setup(cfg)
    grid.close()
