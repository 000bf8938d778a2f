"""Field grids on the GPU (potentialgrid.* and densitygrid.*, Particle.cpp:136-189): the device
step against the reference's fixture and the oracle, maps given as arrays or read from OpenDX
files, the cell choice at cell boundaries and at the box edges, burying changes and errors."""

from __future__ import annotations

import numpy as np
import pytest

from biospring_gb300 import BsError, SpringNetwork, capi
from biospring_gb300 import workloads as W
from helpers import load_golden, rel_l2, rel_scalar, system_from_golden
from oracle import pyoracle as po

pytestmark = pytest.mark.gpu

FORCE_TOL = 1e-5    # relative L2 over the particles (FP32 force sums in another order)
ENERGY_TOL = 1e-5   # relative, per term
POS_TOL = 1e-5      # A, after 30 steps


def _net(s, g, grids=True, burying=True, config=None):
    net = SpringNetwork()
    net.addParticles(**{k: v for k, v in s.arrays().items() if v is not None})
    net.addSprings(s.ij, s.r0, s.k)
    if grids:
        for which in (0, 1):
            net.setFieldGrid(which, g[f"grid{which}"], g[f"grid{which}_origin"], g[f"grid{which}_spacing"])
    if burying:
        net.setBurying(g["burying"])
    net.setup(s.bs_config() if config is None else config)
    return net


def _compare_run(net, g):
    net.computeForces()
    f = net.getForces()
    e = np.array(list(net.energies().values()))
    err = rel_l2(f, g["forces_0"])
    print(f"forces rel L2 vs reference {err:.2e}; energies {e} vs {g['energy_0']}")
    assert err < FORCE_TOL
    for k in range(6):
        if g["energy_0"][k] != 0.0:
            assert rel_scalar(e[k], g["energy_0"][k]) < ENERGY_TOL, (k, e[k], g["energy_0"][k])
    done = 0
    for mark in (1, 10, 30):
        net.computeStep(mark - done)
        done = mark
        dx = float(np.abs(net.getPositions().astype(np.float64) - g[f"pos_{mark}"]).max())
        e = np.array(list(net.energies().values()))
        print(f"step {mark}: max |dx| {dx:.2e} A")
        assert dx < POS_TOL
        for k in range(6):
            ref = float(g[f"energy_{mark}"][k])
            if ref != 0.0:
                assert rel_scalar(e[k], ref) < ENERGY_TOL, (mark, k, e[k], ref)
    return net.getPositions()


def test_fields_match_reference():
    g = load_golden("fields.npz")
    s = system_from_golden(g)
    net = _net(s, g)
    for which in (0, 1):
        np.testing.assert_array_equal(net.fieldGrid(which), g[f"cells{which}"])  # compute_gradient, bit for bit
    _compare_run(net, g)
    net.close()


def test_fields_from_dx_files(tmp_path):
    """The same maps read at set-up from the configured paths (SpringNetwork.cpp:717-747)."""
    g = load_golden("fields.npz")
    s = system_from_golden(g)
    for which in (0, 1):
        path = str(tmp_path / f"g{which}.dx")
        W.write_dx(path, g[f"grid{which}"], g[f"grid{which}_origin"], g[f"grid{which}_spacing"])
        s.config["potentialgrid_path" if which == 0 else "densitygrid_path"] = path.encode()
    net = _net(s, g, grids=False)
    for which in (0, 1):
        np.testing.assert_array_equal(net.fieldGrid(which), g[f"cells{which}"])
    a = _compare_run(net, g)
    ref = _net(system_from_golden(g), g)
    ref.computeStep(30)
    np.testing.assert_array_equal(a, ref.getPositions())
    net.close()
    ref.close()


def _field_only_system(xyz, charge, g):
    """Particles that feel only the maps: no springs, no steric term, Coulomb on (the potential
    map needs it) with scale 0, so its pair forces are exact zeros."""
    cfg = dict(spring_enable=0, steric_enable=0, coulomb_enable=1, coulomb_cutoff=12.0, coulomb_scale=0.0,
               potentialgrid_enable=1,
               potentialgrid_scale=1.5, densitygrid_enable=1, densitygrid_scale=0.7, viscosity_enable=0)
    return W.System("fields-only", xyz.astype(np.float32), np.zeros((0, 2), np.int32), np.zeros(0, np.float32),
                    np.zeros(0, np.float32), cfg, charge=charge.astype(np.float32))


def _boundary_points(g, rng):
    """Coordinates on cell boundaries of both maps (origin + k h rounded to float, and the floats
    around them), on the box edges (origin, origin + n h - 1e-6 and their neighbours), and inside."""
    pts = []
    for which in (0, 1):
        o, h, shape = g[f"grid{which}_origin"], g[f"grid{which}_spacing"], g[f"grid{which}"].shape
        hi = o + h * np.array(shape)
        for _ in range(300):
            p = np.empty(3, np.float32)
            for a in range(3):
                kind = rng.integers(0, 4)
                if kind == 0:
                    v = np.float32(o[a] + rng.integers(0, shape[a] + 1) * h[a])
                elif kind == 1:
                    v = np.float32(hi[a] - 1e-6)
                elif kind == 2:
                    v = np.float32(o[a])
                else:
                    v = np.float32(rng.uniform(o[a], hi[a]))
                v = np.nextafter(v, np.float32(np.inf if rng.random() < 0.5 else -np.inf)) if rng.random() < 0.4 else v
                p[a] = v
            pts.append(p)
    return np.array(pts, np.float32)


def test_cell_choice_at_boundaries_is_exact():
    """At cell boundaries and box edges the device picks the cell the reference's double
    arithmetic picks: field-only forces equal the oracle's bit for bit."""
    g = load_golden("fields.npz")
    rng = np.random.default_rng(21)
    xyz = _boundary_points(g, rng)
    charge = rng.choice([-1.0, 1.0, 0.5], xyz.shape[0])
    s = _field_only_system(xyz, charge, g)
    bur = rng.uniform(0.0, 2.0, s.n).astype(np.float32)
    net = SpringNetwork()
    net.addParticles(**{k: v for k, v in s.arrays().items() if v is not None})
    for which in (0, 1):
        net.setFieldGrid(which, g[f"grid{which}"], g[f"grid{which}_origin"], g[f"grid{which}_spacing"])
    net.setBurying(bur)
    net.setup(s.bs_config())
    net.computeForces()
    orc = po.Oracle(s)
    for which in (0, 1):
        orc.set_field_grid(which, g[f"grid{which}"], g[f"grid{which}_origin"], g[f"grid{which}_spacing"])
    orc.set_burying(bur)
    orc.compute_forces()
    f, fo = net.getForces(), orc.forces()
    nz = int(np.count_nonzero(np.any(fo != 0.0, axis=1)))
    print(f"{s.n} boundary particles, {nz} inside a map")
    assert 0 < nz < s.n
    np.testing.assert_array_equal(f, fo)
    e, eo = net.energies(), orc.energies()
    assert rel_scalar(e["electrostatic"], eo[capi.ENERGY_NAMES.index("electrostatic")]) < 1e-6
    net.close()
    orc.close()


def test_burying_after_setup():
    g = load_golden("fields.npz")
    s = system_from_golden(g)
    net = _net(s, g, burying=False)
    b2 = (g["burying"] * 0.5 + 0.25).astype(np.float32)
    net.setBurying(b2)
    net.computeForces()
    orc = po.Oracle(s)
    for which in (0, 1):
        orc.set_field_grid(which, g[f"grid{which}"], g[f"grid{which}_origin"], g[f"grid{which}_spacing"])
    orc.set_burying(b2)
    orc.compute_forces()
    err = rel_l2(net.getForces(), orc.forces())
    print(f"forces rel L2 vs oracle after a burying change {err:.2e}")
    assert err < FORCE_TOL
    net.close()
    orc.close()


def test_field_errors(tmp_path):
    g = load_golden("fields.npz")
    s = system_from_golden(g)
    # enabled with neither a grid nor a path
    net = SpringNetwork()
    net.addParticles(**{k: v for k, v in s.arrays().items() if v is not None})
    with pytest.raises(BsError, match="no grid"):
        net.setup(s.bs_config())
    # a path that is not an OpenDX map
    bad = tmp_path / "bad.dx"
    bad.write_text("not a map\n")
    s.config["potentialgrid_path"] = str(bad).encode()
    s.config["densitygrid_enable"] = 0
    with pytest.raises(BsError, match="OpenDXReader"):
        net.setup(s.bs_config())
    # the potential map is inert without coulomb.enable (SpringNetwork.cpp:110-115)
    s.config.update(coulomb_enable=0)
    net.setup(s.bs_config())
    with pytest.raises(BsError):
        net.fieldGrid(0)
    net.close()
