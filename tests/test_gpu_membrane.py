"""IMPALA double membrane with tube curvatures on the GPU (bs_set_membrane) against the reference
(golden fixture, tests/golden/membrane.npz) and the oracle.

Bars: forces 1e-5 relative L2 over the dynamic particles, the IMPALA energy 1e-5 relative,
positions within 1e-5 A after 5 steps."""

from __future__ import annotations

import numpy as np
import pytest

from biospring_gb300 import BsError
from biospring_gb300 import workloads as W
from helpers import dynamic_mask, gpu_network, load_golden, rel_l2, rel_scalar, system_from_golden
from oracle import pyoracle as po

pytestmark = pytest.mark.gpu


def test_double_membrane_matches_reference():
    g = load_golden("membrane.npz")
    s = system_from_golden(g)
    dyn = dynamic_mask(s)
    for k, m in enumerate(g["membranes"]):
        net = gpu_network(s)
        net.setMembrane(*m)
        net.computeForces()
        err = rel_l2(net.getForces(), g[f"force0_{k}"], dyn)
        e = np.array(list(net.energies().values()))
        print(f"membrane {m}: forces vs reference {err:.2e}, IMPALA energy {e[4]:.9g} vs {g[f'energy0_{k}'][4]:.9g}")
        assert err <= 1e-5
        assert rel_scalar(e[4], g[f"energy0_{k}"][4]) < 1e-5
        net.close()
        net = gpu_network(s)
        net.setMembrane(*m)
        net.computeStep(5)
        assert np.abs(net.getPositions() - g[f"pos5_{k}"]).max() < 1e-5
        net.close()


def test_double_membrane_against_oracle_and_reset():
    """A 4,000-bead globule spread across both membranes; the setting changes between steps of one
    handle (captured step graphs are rebuilt) and goes back to the flat membrane."""
    s = W.membrane_globule(n=4000, seed=12)
    s.xyz = (s.xyz * np.float32(1.6)).astype(np.float32)  # reach both membranes
    net = gpu_network(s)
    for m in ([18.0, 22.0, 0.01, 0.02], [10.0, 10.0, -0.03, 0.0], [0.0, 0.0, 0.0, 0.0]):
        net.setMembrane(*m)
        net.computeForces()
        orc = po.Oracle(W.System(s.name, net.getPositions(), s.ij, s.r0, s.k, s.config, vel=net.getVelocities(),
                                 sasa=s.sasa, transfer=s.transfer))
        orc.set_membrane(*m)
        orc.compute_forces()
        err = rel_l2(net.getForces(), orc.forces())
        e, eo = np.array(list(net.energies().values())), orc.energies()
        print(f"membrane {m}: forces vs oracle {err:.2e}, IMPALA {e[4]:.9g} vs {eo[4]:.9g}")
        assert err <= 1e-5
        assert rel_scalar(e[4], eo[4]) < 1e-5
        net.computeStep(3)
        orc.close()
    with pytest.raises(BsError):
        net.setMembrane(float("nan"), 0.0, 0.0, 0.0)
    net.close()
