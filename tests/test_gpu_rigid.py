"""Rigid bodies on the GPU against the reference (one body, golden fixture) and the oracle's
multi-body restatement (RigidBody.cpp:430-635 with each particle's index inside its own body).

The body kernel sums member forces and torques in a different order than the reference's serial
loop, so agreement is to FP32 rounding, not bit for bit.
"""

from __future__ import annotations

import numpy as np
import pytest

from biospring_gb300 import BsError, SpringNetwork
from biospring_gb300 import workloads as W
from helpers import gpu_network, load_golden, rel_scalar, system_from_golden
from oracle import pyoracle as po

pytestmark = pytest.mark.gpu


def test_single_body_matches_reference():
    g = load_golden("rigid1.npz")
    s = system_from_golden(g)
    s.config["rigidbody_enable"] = 1
    s.bodies = [np.arange(s.n, dtype=np.int32)]
    net = gpu_network(s)
    net.computeStep(20)
    x = net.getPositions()
    dx = float(np.abs(x.astype(np.float64) - g["pos20"]).max())
    e = np.array(list(net.energies().values()))
    print(f"one body, 20 steps: max |dx| vs reference {dx:.2e} A; energies {e} vs {g['energy20']}")
    assert dx < 1e-5
    for k in range(6):
        ref = float(g["energy20"][k])
        if ref != 0.0:
            assert rel_scalar(e[k], ref) < 1e-5, (k, e[k], ref)
        else:
            assert abs(e[k]) < 1e-9
    net.close()


@pytest.fixture(scope="module")
def globule():
    s = W.membrane_globule(n=4000, seed=3, nbodies=4, body_size=500)
    s.config["steric_enable"] = 1
    s.config["steric_cutoff"] = 6.0
    s.config["timestep"] = 0.2
    # displace the free beads (rest lengths stay): stretched springs pull the bodies along
    free = np.ones(s.n, bool)
    for ids in s.bodies:
        free[ids] = False
    s.xyz = s.xyz.copy()
    s.xyz[free] += np.random.default_rng(1).normal(0.0, 0.3, (int(free.sum()), 3)).astype(np.float32)
    return s


def test_multi_body_matches_oracle(globule):
    s = globule
    net = gpu_network(s)
    orc = po.Oracle(s)
    done = 0
    for mark in (1, 10, 40):
        net.computeStep(mark - done)
        orc.step(mark - done)
        done = mark
        x, xo = net.getPositions().astype(np.float64), orc.positions().astype(np.float64)
        dx = float(np.abs(x - xo).max())
        e, eo = np.array(list(net.energies().values())), orc.energies()
        print(f"4 bodies, step {mark}: max |dx| vs oracle {dx:.2e} A, energies {e} vs {eo}")
        assert dx < 2e-5
        for k in range(6):
            if abs(eo[k]) > 1e-12:
                assert rel_scalar(e[k], eo[k]) < 1e-4, (mark, k, e[k], eo[k])
    # members keep their distances to each other (a rigid motion)
    start = s.xyz.astype(np.float64)
    for ids in s.bodies:
        a, b = ids[0], ids[-1]
        d0 = np.linalg.norm(start[a] - start[b])
        d1 = np.linalg.norm(x[a] - x[b])
        assert abs(d1 - d0) < 1e-3
    moved = float(np.abs(x - start).max())
    body_moved = min(float(np.abs(x[ids] - start[ids]).max()) for ids in s.bodies)
    print(f"max move {moved:.3e} A, least-moved body {body_moved:.3e} A")
    assert moved > 1e-2 and body_moved > 1e-4
    net.close()
    orc.close()


def test_rigid_runs_are_deterministic(globule):
    a, b = gpu_network(globule), gpu_network(globule)
    a.computeStep(25)
    b.computeStep(25)
    assert a.getPositions().tobytes() == b.getPositions().tobytes()
    a.close()
    b.close()


def test_rigid_body_errors(globule):
    s = globule
    net = SpringNetwork()
    net.addParticles(xyz=s.xyz, is_static=np.r_[np.ones(1, np.uint8), np.zeros(s.n - 1, np.uint8)])
    with pytest.raises(BsError, match="static"):
        net.setRigidBodies([np.arange(10, dtype=np.int32)])
    with pytest.raises(BsError, match="two bodies"):
        net.setRigidBodies([np.arange(1, 10, dtype=np.int32), np.arange(5, 12, dtype=np.int32)])
    net.close()
