"""CPU checks of the C ABI and the host logic: exported symbols, the .msp reader, the defaults,
and the replica aggregation of the benchmark over two gloo ranks. No kernel is launched."""

from __future__ import annotations

import ctypes as C
import os
import re

import pytest

from biospring_gb300 import build, capi

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def lib():
    if not os.path.exists(build.LIB):
        build.build_library()
    return C.CDLL(build.LIB)


def declared_functions() -> list[str]:
    with open(os.path.join(ROOT, "include", "biospring_gb300.h")) as f:
        text = f.read()
    return sorted(set(re.findall(r"^int (bs_\w+)\(", text, flags=re.M)))


def test_every_declared_entry_point_is_exported(lib):
    names = declared_functions()
    assert len(names) > 30
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing


def test_python_binding_covers_the_header():
    names = declared_functions()
    extra = {"bs_nonbonded_forces_noalloc"}  # bound by its own test with device pointers
    assert set(names) - extra <= set(capi.SIGNATURES), sorted(set(names) - extra - set(capi.SIGNATURES))


def test_defaults_follow_the_reference():
    c = capi.default_config()
    # configuration::defaultConfiguration (Configuration.hpp:153-234)
    assert c.timestep == pytest.approx(0.01)
    assert c.viscosity_value == 1.0 and c.viscosity_enable == 0
    assert c.steric_mode == capi.BS_STERIC_LINEAR
    assert c.coulomb_dielectric == 1.0
    assert (c.probe_x, c.probe_y, c.probe_z, c.probe_mass, c.probe_radius) == (1.0, 1.0, 1.0, 1.0, 1.0)
    assert c.probe_enable == 0 and c.rigidbody_enable == 0
    assert c.rebuild_every == 10 and c.list_skin == 1.0 and c.precise_positions == 0


def test_msp_reader_values_and_errors():
    text = """
# a comment
simulation.timestep = 0.02
steric.enable = true
steric.mode = lennard-jones-8-6Zacharias
steric.cutoff = 9.5
coulomb.enable = 1
coulomb.dielectric = 80
viscosity.enable = yes
viscosity.value = 0.5
probe.enable = on
probe.enablesteric = true
probe.x = -3.5
probe.charge = 2
cuda.dielectricmode = distance
cuda.rebuildevery = 7
cuda.listskin = 0.75
cuda.precisepositions = true
"""
    c = capi.parse_msp(text)
    assert c.timestep == pytest.approx(0.02)
    assert c.steric_enable == 1 and c.steric_mode == capi.BS_STERIC_LJ_8_6_ZACHARIAS
    assert c.steric_cutoff == pytest.approx(9.5)
    assert c.coulomb_enable == 1 and c.coulomb_dielectric == 80.0
    assert c.viscosity_enable == 1 and c.viscosity_value == 0.5
    assert c.probe_enable == 1 and c.probe_steric == 1 and c.probe_electrostatic == 0
    assert c.probe_x == -3.5 and c.probe_charge == 2.0
    assert c.dielectric_mode == capi.BS_DIELECTRIC_DISTANCE
    assert c.rebuild_every == 7 and c.list_skin == 0.75 and c.precise_positions == 1
    # SafeConfigurationReader: unknown and duplicated parameters are errors
    for bad, word in (("steric.nosuch = 1", "invalid parameter"),
                      ("steric.cutoff = 1\nsteric.cutoff = 2", "duplicate"),
                      ("steric.enable = maybe", "boolean"),
                      ("steric.mode = cubic", "invalid choice"),
                      ("no equals sign here", "syntax")):
        with pytest.raises(capi.BsError, match=word):
            capi.parse_msp(bad)


def _rank(rank: int, world: int, port: int, out: list) -> None:
    import torch.distributed as dist
    import bench
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    slowest = bench.max_over_ranks(10.0 + rank, dist)
    out.append((rank, slowest, bench.replica_throughput(1000, 5, slowest, world)))
    dist.destroy_process_group()


def _worker(rank, world, port, q):
    res: list = []
    _rank(rank, world, port, res)
    q.put(res[0])


def test_replica_aggregation_two_gloo_ranks():
    import multiprocessing as mp
    import socket
    with socket.socket() as sk:
        sk.bind(("127.0.0.1", 0))
        port = sk.getsockname()[1]
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    # both ranks agree on the slowest rank's time and on the whole-job throughput
    assert [r[1] for r in res] == [11.0, 11.0]
    assert res[0][2] == res[1][2] == pytest.approx(2 * 1000 * 5 / 11e-3)
