"""The probe particle on the GPU (SpringNetwork.cpp:156-182, Particle.cpp:434-465) against the
reference's own trajectory (golden fixture) and the oracle, in every steric mode."""

from __future__ import annotations

import numpy as np
import pytest

from helpers import gpu_network, load_golden, rel_scalar, system_from_golden
from oracle import pyoracle as po

pytestmark = pytest.mark.gpu


def test_probe_matches_reference():
    g = load_golden("probe.npz")
    s = system_from_golden(g)
    net = gpu_network(s)
    done = 0
    for mark in (1, 10, 30):
        net.computeStep(mark - done)
        done = mark
        x = net.getPositions()
        pr = net.getProbe()
        e = np.array(list(net.energies().values()))
        dx = float(np.abs(x.astype(np.float64) - g[f"pos_{mark}"]).max())
        dp = float(np.abs(pr.astype(np.float64) - g[f"probe_{mark}"]).max())
        print(f"step {mark}: max |dx| {dx:.2e} A, probe |d| {dp:.2e}, energies {e} vs {g[f'energy_{mark}']}")
        assert dx < 1e-5 and dp < 1e-5
        for k in range(6):
            ref = float(g[f"energy_{mark}"][k])
            if ref != 0.0:
                assert rel_scalar(e[k], ref) < 1e-5, (mark, k, e[k], ref)
    net.close()


@pytest.mark.parametrize("mode", [0, 1, 2, 3])
def test_probe_all_steric_modes_against_oracle(mode):
    g = load_golden("probe.npz")
    s = system_from_golden(g)
    s.config.update(steric_mode=mode, timestep=0.2, probe_x=0.5, probe_y=0.5, probe_z=0.5)
    net = gpu_network(s)
    orc = po.Oracle(s)
    net.computeStep(25)
    orc.step(25)
    dx = float(np.abs(net.getPositions().astype(np.float64) - orc.positions()).max())
    dp = float(np.abs(net.getProbe().astype(np.float64) - orc.probe()).max())
    moved = float(np.abs(orc.probe()[:3] - np.array([0.5, 0.5, 0.5])).max())
    print(f"mode {mode}: max |dx| {dx:.2e} A, probe |d| {dp:.2e}, probe moved {moved:.3e} A")
    assert dx < 1e-4 and dp < 1e-4
    net.close()
    orc.close()
