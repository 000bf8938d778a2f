"""A topology loaded from a NetCDF file (bs_load_nc, NetCDFReader.cpp) steps exactly like the same
arrays uploaded by hand, and like the oracle."""

from __future__ import annotations

import numpy as np
import pytest

from biospring_gb300 import SpringNetwork, capi
from biospring_gb300 import workloads as W
from oracle import pyoracle as po
from test_nc_cpu import write_topology

pytestmark = pytest.mark.gpu


def test_loaded_topology_steps_like_uploaded_arrays(tmp_path):
    path = str(tmp_path / "t.nc")
    rng = np.random.default_rng(9)
    i = rng.integers(0, 400, 900)
    springs = np.stack([i, (i + rng.integers(1, 400, 900)) % 400], axis=1).astype(np.int32)
    write_topology(path, n=400, m=900, seed=3, version=2, zero_mass=(5,), springs=springs)
    t = capi.read_nc(path)
    cfg = dict(spring_enable=1, steric_enable=1, steric_cutoff=8.0, coulomb_enable=1, coulomb_cutoff=12.0,
               impala_enable=1, hydrophobicity_enable=1, hydrophobicity_cutoff=8.0, viscosity_enable=1,
               timestep=0.05)
    s = W.System("nc", t["xyz"], t["ij"], t["r0"], t["k"], cfg, mass=t["mass"], charge=t["charge"],
                 radius=t["radius"], epsilon=t["epsilon"], sasa=t["sasa"], transfer=t["transfer"],
                 hydrophobicity=t["hydrophobicity"], is_static=t["is_static"])
    a = SpringNetwork()
    n, m = a.loadNetCDF(path)
    assert (n, m) == (400, 900)
    a.setup(s.bs_config())
    b = SpringNetwork()
    b.addParticles(**{k: v for k, v in s.arrays().items() if v is not None})
    b.addSprings(s.ij, s.r0, s.k)
    b.setup(s.bs_config())
    a.computeStep(20)
    b.computeStep(20)
    np.testing.assert_array_equal(a.getPositions(), b.getPositions())
    assert a.energies() == b.energies()
    orc = po.Oracle(s)
    orc.step(20)
    dx = float(np.abs(a.getPositions().astype(np.float64) - orc.positions()).max())
    print(f"max |dx| vs oracle after 20 steps: {dx:.2e} A")
    assert dx < 1e-5
    a.close()
    b.close()
    orc.close()
