"""Pins the CPU oracle (oracle/bs_oracle.cpp) to the reference's own outputs.

The golden fixtures were produced by the compiled reference (tests/golden/make_golden.py).
On the machine that generated them (x86-64, where the reference itself can be compiled) the
oracle must reproduce them bit for bit; elsewhere a different libm may move the last bit of
exp/pow, so the comparisons fall back to 1e-6 relative there.
"""

import os

import numpy as np
import pytest

from helpers import load_golden, system_from_golden, rel_l2
from oracle import pyoracle as po

os.environ.setdefault("OMP_NUM_THREADS", "1")
EXACT = po.have_reference()  # the fixtures were generated on this machine's toolchain


def same(a, b, rtol=1e-6):
    if EXACT:
        np.testing.assert_array_equal(a, b)
    else:
        np.testing.assert_allclose(a, b, rtol=rtol, atol=0)


def test_regression_scans():
    """Two-particle distance scans of src/tests/regression/test-*-energy.cpp."""
    from biospring_gb300 import workloads as W
    g = load_golden("scans.npz")
    xs = g["x"]
    cc = dict(charge=np.full(2, 0.5973, np.float32), radius=np.full(2, 1.908, np.float32),
              epsilon=np.full(2, 0.086, np.float32), mass=np.full(2, 12.01, np.float32))
    base = dict(nbsteps=1, timestep=0.01)
    cases = {
        "spring": (dict(base, spring_enable=1), dict(ij=np.array([[0, 1]], np.int32), r0=np.zeros(1, np.float32),
                                                     k=np.ones(1, np.float32)), cc),
        "steric_linear": (dict(base, steric_enable=1, steric_cutoff=16.0, steric_mode=0), {}, cc),
        "steric_amber": (dict(base, steric_enable=1, steric_cutoff=16.0, steric_mode=1), {}, cc),
        "coulomb": (dict(base, coulomb_enable=1, coulomb_cutoff=16.0, coulomb_dielectric=1.0), {}, cc),
        "hydrophobic": (dict(base, hydrophobicity_enable=1, hydrophobicity_cutoff=16.0), {},
                        dict(hydrophobicity=np.array([0.5, 0.3], np.float32))),
    }
    for name, (cfg, sp, props) in cases.items():
        s = W.System("two", np.zeros((2, 3), np.float32), sp.get("ij", np.zeros((0, 2), np.int32)),
                     sp.get("r0", np.zeros(0, np.float32)), sp.get("k", np.zeros(0, np.float32)), cfg, **props)
        orc = po.Oracle(s)
        for t, x in enumerate(xs):
            orc.set_positions(np.array([[0, 0, 0], [x, 0, 0]], np.float32))
            orc.compute_forces()
            same(orc.energies(), g[f"{name}_energy"][t])
            same(orc.forces(), g[f"{name}_force"][t])
        orc.close()


def test_scan_matches_independent_formulas():
    """The reference's own expected values (independent formulas of the regression tests)."""
    g = load_golden("scans.npz")
    x = g["x"].astype(np.float64)
    # spring: 0.5 * k * d^2 with k = 1, r0 = 0 (test-spring-energy.cpp:11-20)
    np.testing.assert_allclose(g["spring_energy"][:, 1], 0.5 * x * x, rtol=2e-6)
    # Coulomb, k = 8.9875517873681764e9 (test-electrostatic-energy.cpp:56-76)
    q = np.float64(np.float32(0.5973)) * 1.60217653e-19
    e = 8.9875517873681764e9 * q * q / (x * 1e-10) * 6.02214169e23 * 1e-3
    np.testing.assert_allclose(g["coulomb_energy"][:, 3], e, rtol=1e-5)
    # linear steric (test-steric-energy.cpp:12-22)
    dv = x - 2 * np.float64(np.float32(1.908))
    lin = np.where(dv < 0, 0.5 * dv * dv, 0.0)
    np.testing.assert_allclose(g["steric_linear_energy"][:, 2], lin, rtol=1e-5, atol=1e-6)
    # hydrophobic, h = 0.5, 0.3 (test-hydrophobic-energy.cpp:18-27)
    hy = -(np.float64(np.float32(0.5)) * np.float64(np.float32(0.3))) * np.exp(-x) * 6.02214169e23 * 1e-3
    np.testing.assert_allclose(g["hydrophobic_energy"][:, 5], hy, rtol=1e-5)


def test_ca_network_trajectory():
    g = load_golden("ca300.npz")
    s = system_from_golden(g)
    orc = po.Oracle(s)
    done = 0
    for mark in (1, 10, 30):
        orc.step(mark - done)
        done = mark
        same(orc.positions(), g[f"pos_{mark}"])
        same(orc.velocities(), g[f"vel_{mark}"])
        same(orc.energies(), g[f"energy_{mark}"])


@pytest.mark.parametrize("mode", [0, 1, 2, 3])
def test_mixed_terms(mode):
    g = load_golden(f"mixed_m{mode}.npz")
    s = system_from_golden(g)
    orc = po.Oracle(s)
    orc.compute_forces()
    same(orc.forces(), g["force0"])
    same(orc.energies(), g["energy0"])
    orc.close()
    orc = po.Oracle(s)
    if mode == 1:
        for term in (0, 1, 2):
            np.testing.assert_array_equal(orc.pairs(term), g[f"pairs{term}"])
            np.testing.assert_array_equal(orc.cells(term), g[f"cells{term}"])
    orc.step(3)
    same(orc.positions(), g["pos3"])
    same(orc.velocities(), g["vel3"])
    same(orc.energies(), g["energy3"])


def test_single_rigid_body():
    g = load_golden("rigid1.npz")
    s = system_from_golden(g)
    s.bodies = [np.arange(s.n, dtype=np.int32)]
    orc = po.Oracle(s)
    orc.step(20)
    same(orc.positions(), g["pos20"])
    same(orc.energies(), g["energy20"])


def test_neighbour_search_against_brute_force():
    """Reference grid pairs (test-nsearch.cpp:103-129) == oracle grid pairs == O(N^2)."""
    g = load_golden("nsearch.npz")
    s = system_from_golden(g)
    orc = po.Oracle(s)
    pairs = orc.pairs(0)
    np.testing.assert_array_equal(pairs, g["pairs0"])
    np.testing.assert_array_equal(orc.cells(0), g["cells0"])
    x = s.xyz.astype(np.float64)
    d = np.sqrt(((x[:, None, :] - x[None, :, :]) ** 2).sum(-1))
    i, j = np.nonzero(np.triu(d < 10.0, k=1))
    brute = np.stack([i, j], 1)
    np.testing.assert_array_equal(pairs, brute)


def test_fp64_evaluator_close_to_reference_arithmetic():
    """The FP64 evaluator agrees with the FP32 reference arithmetic to FP32 accuracy."""
    g = load_golden("mixed_m1.npz")
    s = system_from_golden(g)
    orc = po.Oracle(s)
    orc.compute_forces()
    f32 = orc.forces()
    f64, e64 = orc.eval_fp64()
    dyn = np.asarray(s.is_static) == 0
    assert rel_l2(f32, f64, dyn) < 1e-5
    e32 = orc.energies()
    for k in (2, 3, 4):
        assert abs(e32[k] - e64[k]) <= 1e-5 * abs(e64[k]) + 1e-6


def test_probe_particle():
    """The probe (SpringNetwork.cpp:156-182): every dynamic particle against one extra particle,
    steric and electrostatic, no cutoff; the probe integrates alone after the particle loop."""
    g = load_golden("probe.npz")
    s = system_from_golden(g)
    orc = po.Oracle(s)
    done = 0
    for mark in (1, 10, 30):
        orc.step(mark - done)
        done = mark
        same(orc.positions(), g[f"pos_{mark}"])
        same(orc.probe(), g[f"probe_{mark}"])
        same(orc.energies(), g[f"energy_{mark}"])


def test_double_membrane_matches_reference():
    """IMPALA double membrane with tube curvatures (energy/imp.hpp:29-159 with the offsets and
    curvatures of ForceField.h:23-25 set): forces and energies at the start and the state after 5
    steps, under three settings."""
    g = load_golden("membrane.npz")
    s = system_from_golden(g)
    for k, m in enumerate(g["membranes"]):
        orc = po.Oracle(s)
        orc.set_membrane(*m)
        orc.compute_forces()
        same(orc.forces(), g[f"force0_{k}"])
        same(orc.energies(), g[f"energy0_{k}"])
        orc.close()
        orc = po.Oracle(s)
        orc.set_membrane(*m)
        orc.step(5)
        same(orc.positions(), g[f"pos5_{k}"])
        same(orc.energies(), g[f"energy5_{k}"])
        orc.close()
