"""CPU checks of the benchmark's reference arm: it runs without any product library, on the
same seeded system and the same configuration as the native arm.

The reference arm times the CPU restatement. It generates its system with the oracle library's
own copy of the generators and builds its configuration from the oracle's own restatement of
the reference's defaults, so the product library is never mapped into that process."""

from __future__ import annotations

import os
import subprocess
import sys

import numpy as np
import pytest

from biospring_gb300 import build, capi
from biospring_gb300 import workloads as W
from oracle import pyoracle

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_oracle_defaults_equal_the_library_defaults():
    if not os.path.exists(build.LIB):
        build.build_library()
    lib_cfg = capi.default_config()
    orc_cfg = pyoracle.oracle_config(W.System("empty", np.zeros((1, 3), np.float32), np.zeros((0, 2), np.int32),
                                              np.zeros(0, np.float32), np.zeros(0, np.float32), {}))
    assert lib_cfg.to_dict() == orc_cfg.to_dict()


def test_oracle_generators_give_the_library_generators_systems():
    build.build_synth()
    W.set_generator_library(W.SYNTH_PATH)
    a = W.uniform_lj(n=3000, box=50.0, seed=5)
    b_chain = W.ca_network(n=500, seed=9)
    pyoracle.use_oracle_generator()
    try:
        b = W.uniform_lj(n=3000, box=50.0, seed=5)
        a_chain = W.ca_network(n=500, seed=9)
    finally:
        W.set_generator_library(W.SYNTH_PATH)
    for x, y in ((a, b), (a_chain, b_chain)):
        assert np.array_equal(x.xyz, y.xyz)
        assert np.array_equal(x.ij, y.ij)
        assert np.array_equal(x.r0, y.r0)
        assert np.array_equal(x.k, y.k)


def test_reference_arm_maps_no_product_library():
    code = (
        "import sys, runpy, json\n"
        "sys.argv = ['bench.py', '--impl', 'reference', '--steps', '1', '--warmup', '3']\n"
        "runpy.run_path('bench.py', run_name='__main__')\n"
        "maps = open('/proc/self/maps').read().splitlines()\n"
        f"print(json.dumps(sorted({{l.split()[-1] for l in maps if l.endswith('.so') and {ROOT!r} in l}})))\n"
    )
    env = dict(os.environ, OMP_NUM_THREADS=str(os.cpu_count() or 1))
    proc = subprocess.run([sys.executable, "-c", code], cwd=ROOT, env=env, stdout=subprocess.PIPE,
                          stderr=subprocess.PIPE, text=True, timeout=600)
    assert proc.returncode == 0, proc.stderr[-2000:]
    import json
    lines = [ln for ln in proc.stdout.splitlines() if ln.strip()]
    line = json.loads(lines[-2])
    mapped = json.loads(lines[-1])
    assert mapped and all(os.path.relpath(p, ROOT).startswith("oracle" + os.sep) for p in mapped), mapped
    assert line["impl"] == "reference"
    assert line["warmup"] == 3 and line["steps"] == 1
    assert line["cpu_baseline"]["kind"] == "port"
    assert "eps=4r" in line["config"]["workload"]


@pytest.mark.parametrize("dielectric_mode", [0, 1])
def test_oracle_config_carries_the_system_parameters(dielectric_mode):
    s = W.uniform_lj(n=2000, box=44.0, seed=1, dielectric_mode=dielectric_mode)
    cfg = pyoracle.oracle_config(s)
    assert cfg.dielectric_mode == dielectric_mode
    assert cfg.steric_mode == capi.BS_STERIC_LJ_12_6_AMBER
    assert cfg.coulomb_cutoff == 12.0 and cfg.coulomb_dielectric == 4.0
