"""Field grids on the CPU: the OpenDX reader of the library and the oracle's field forces,
pinned to the reference (potentialgrid.* and densitygrid.*, Particle.cpp:136-189).

The fixture tests/golden/fields.npz holds the reference's grid cells (scalar and force vector,
PotentialGrid::compute_gradient) and its forces, energies and trajectory for a charged network
under an electrostatic potential map and a density map. On the machine that generated it the
oracle reproduces it bit for bit; elsewhere to 1e-6 relative.
"""

from __future__ import annotations

import ctypes as C
import os

import numpy as np
import pytest

from biospring_gb300 import capi
from biospring_gb300 import workloads as W
from helpers import load_golden, system_from_golden
from oracle import pyoracle as po

EXACT = po.have_reference()


def same(a, b, rtol=1e-6):
    if EXACT:
        np.testing.assert_array_equal(a, b)
    else:
        np.testing.assert_allclose(a, b, rtol=rtol, atol=0)


def fields_oracle(g):
    s = system_from_golden(g)
    orc = po.Oracle(s)
    for which in (0, 1):
        orc.set_field_grid(which, g[f"grid{which}"], g[f"grid{which}_origin"], g[f"grid{which}_spacing"])
    orc.set_burying(g["burying"])
    return s, orc


def test_oracle_field_cells_match_reference():
    g = load_golden("fields.npz")
    _, orc = fields_oracle(g)
    for which in (0, 1):
        np.testing.assert_array_equal(orc.field_grid(which), g[f"cells{which}"])


def test_oracle_field_forces_and_trajectory():
    g = load_golden("fields.npz")
    _, orc = fields_oracle(g)
    orc.compute_forces()
    same(orc.forces(), g["forces_0"])
    same(orc.energies(), g["energy_0"])
    _, orc = fields_oracle(g)
    done = 0
    for mark in (1, 10, 30):
        orc.step(mark - done)
        done = mark
        same(orc.positions(), g[f"pos_{mark}"])
        same(orc.energies(), g[f"energy_{mark}"])


def test_field_terms_matter_and_offgrid_is_zero():
    """The maps move the result (the fixture would not test them otherwise), and a particle
    outside a map's box gets nothing from it (test-offgrid-force.cpp)."""
    g = load_golden("fields.npz")
    s, orc = fields_oracle(g)
    orc.compute_forces()
    with_fields = orc.forces()
    s.config.update(potentialgrid_enable=0, densitygrid_enable=0)
    plain = po.Oracle(s)
    plain.compute_forces()
    diff = np.abs(with_fields.astype(np.float64) - plain.forces())
    assert diff.max() > 0.1 * np.abs(plain.forces()).max()
    # particles outside both boxes feel no field
    out = np.ones(s.n, bool)
    for which in (0, 1):
        o = g[f"grid{which}_origin"]
        hi = o + g[f"grid{which}_spacing"] * np.array(g[f"grid{which}"].shape)
        inside = np.all((s.xyz >= o) & (s.xyz <= hi - 1e-6), axis=1)
        out &= ~inside
    assert out.sum() > 0
    np.testing.assert_array_equal(diff[out], 0.0)


def _read_dx(path):
    lib = capi.load()
    shape = np.zeros(3, np.int32)
    origin = np.zeros(3, np.float64)
    spacing = np.zeros(3, np.float64)
    err = C.create_string_buffer(256)
    p = lambda a, t: a.ctypes.data_as(C.POINTER(t))  # noqa: E731
    rc = lib.bs_read_dx(path.encode(), p(shape, C.c_int32), p(origin, C.c_double), p(spacing, C.c_double), None,
                        err, 256)
    if rc != capi.BS_OK:
        return rc, err.value.decode(), None, None, None
    sc = np.zeros(tuple(shape), np.float32)
    rc = lib.bs_read_dx(path.encode(), p(shape, C.c_int32), p(origin, C.c_double), p(spacing, C.c_double),
                        p(sc, C.c_float), err, 256)
    return rc, err.value.decode(), sc, origin, spacing


def test_library_dx_reader_matches_reference(tmp_path):
    """bs_read_dx reads what OpenDXReader reads: the fixture's map written as OpenDX, an odd
    value count (the last line short) and comment lines."""
    g = load_golden("fields.npz")
    for which in (0, 1):
        path = str(tmp_path / f"g{which}.dx")
        W.write_dx(path, g[f"grid{which}"], g[f"grid{which}_origin"], g[f"grid{which}_spacing"])
        rc, msg, sc, origin, spacing = _read_dx(path)
        assert rc == capi.BS_OK, msg
        np.testing.assert_array_equal(sc, g[f"cells{which}"][..., 0])
        np.testing.assert_array_equal(origin, g[f"grid{which}_origin"])
        np.testing.assert_array_equal(spacing, g[f"grid{which}_spacing"])


def test_library_dx_reader_errors(tmp_path):
    good = tmp_path / "good.dx"
    W.write_dx(str(good), np.ones((3, 3, 3), np.float32), (0, 0, 0), (1, 1, 1))
    text = good.read_text().splitlines()
    cases = {
        "missing.dx": None,
        "counts.dx": ["object 1 class gridpositions count 3 3 3"] + text[2:],
        "origin.dx": text[:2] + ["origin 0 0"] + text[3:],
        "delta.dx": text[:3] + ["delt 1 0 0"] + text[4:],
        "short.dx": text[:8],
        "tokens.dx": text[:8] + ["1 1 1 1"] + text[9:],
        # refused from the header alone, before a size is derived or allocated
        "huge.dx": ["object 1 class gridpositions counts 5000 4000 3000"] + text[2:],
        "axis.dx": ["object 1 class gridpositions counts 1 1 20000000"] + text[2:],
        "zero_delta.dx": text[:3] + ["delta 0 0 0"] + text[4:],
    }
    reason = {"huge.dx": "too short for the 5000 x 4000 x 3000", "axis.dx": "more than 16777216",
              "zero_delta.dx": "cell size > 0"}
    for name, lines in cases.items():
        path = tmp_path / name
        if lines is not None:
            path.write_text("\n".join(lines) + "\n")
        rc, msg, *_ = _read_dx(str(path))
        assert rc == capi.BS_E_ARG, name
        assert msg.startswith("OpenDXReader:"), (name, msg)
        assert reason.get(name, "") in msg, (name, msg)


@pytest.mark.skipif(not po.have_reference(), reason="the compiled reference is not present")
def test_reference_reads_the_same_dx(tmp_path):
    """The reference's own reader on a map the library wrote: same grid cells as the fixture."""
    g = load_golden("fields.npz")
    s = system_from_golden(g)
    for which in (0, 1):
        path = str(tmp_path / f"g{which}.dx")
        W.write_dx(path, g[f"grid{which}"], g[f"grid{which}_origin"], g[f"grid{which}_spacing"])
        s.config["potentialgrid_path" if which == 0 else "densitygrid_path"] = path.encode()
    ref = po.Reference(s)
    for which in (0, 1):
        np.testing.assert_array_equal(ref.field_grid(which), g[f"cells{which}"])
    ref.close()


def test_msp_grid_keys():
    c = capi.parse_msp("potentialgrid.enable = true\npotentialgrid.path = /tmp/x.dx\npotentialgrid.scale = 2.5\n"
                       "densitygrid.enable = 1\ndensitygrid.path = maps/d.dx\ndensitygrid.scale = 0.25\n")
    assert c.potentialgrid_enable == 1 and c.densitygrid_enable == 1
    assert c.potentialgrid_path == b"/tmp/x.dx" and c.densitygrid_path == b"maps/d.dx"
    assert c.potentialgrid_scale == 2.5 and c.densitygrid_scale == 0.25
    d = capi.default_config()
    assert d.potentialgrid_scale == 1.0 and d.densitygrid_scale == 1.0 and d.potentialgrid_path == b""


def test_dx_reader_survives_truncation_and_corruption(tmp_path):
    """An OpenDX map cut short anywhere, or with a character overwritten, is either read (and then
    holds as many values as its header declares) or refused with an error code."""
    src = str(tmp_path / "ok.dx")
    g = np.random.default_rng(1).standard_normal((5, 4, 3)).astype(np.float32)
    W.write_dx(src, g, np.array([1.0, 2.0, 3.0]), np.array([0.5, 0.5, 0.5]))
    text = open(src, "rb").read()
    rng = np.random.default_rng(2)
    blobs = [text[:cut] for cut in range(0, len(text), 5)]
    for _ in range(400):
        b = bytearray(text)
        b[int(rng.integers(0, len(b)))] = int(rng.choice(list(b"0123456789 -.e\nabxyz#")))
        blobs.append(bytes(b))
    path = str(tmp_path / "t.dx")
    read = 0
    for blob in blobs:
        with open(path, "wb") as fh:
            fh.write(blob)
        rc, _, sc, _, _ = _read_dx(path)
        if rc == capi.BS_OK:
            read += 1
            assert sc.size == int(np.prod(sc.shape))
    assert 0 < read < len(blobs)
