"""BioSpring topologies from NetCDF classic files (NetCDFReader, src/IO/NetCDFReader.cpp:8-264)
read by the library's own reader, checked against scipy's independent NetCDF implementation:
every variable, the optional arrays, record (unlimited) dimensions, both offset sizes, the zero-
mass rule and the reader's error messages."""

from __future__ import annotations

import os

import numpy as np
import pytest

from biospring_gb300 import BsError, capi

netcdf = pytest.importorskip("scipy.io").netcdf_file
from oracle import pyoracle as po  # noqa: E402

# the example topology shipped with BioSpring, where the reference sources are present
REF_NC = os.path.join(po.reference_dir(), "scripts", "outdated", "articulatedrigidbody", "example", "1IYT.nc")


def write_topology(path, n=57, m=80, seed=0, version=1, optional=True, record=False, zero_mass=(), **override):
    rng = np.random.default_rng(seed)
    a = dict(coordinates=rng.uniform(-30, 30, (n, 3)).astype(np.float32),
             particleids=np.arange(n, dtype=np.int32), resids=(np.arange(n) // 4).astype(np.int32),
             charges=rng.choice([-1.0, 0.0, 0.5, 1.0], n).astype(np.float32),
             radii=rng.uniform(1.0, 3.0, n).astype(np.float32), epsilon=rng.uniform(0.1, 1.0, n).astype(np.float32),
             mass=rng.uniform(10.0, 200.0, n).astype(np.float32),
             dynamicstate=(rng.random(n) < 0.8).astype(np.int8),
             springs=rng.integers(0, n, (m, 2)).astype(np.int32),
             springsstiffness=rng.uniform(0.5, 5.0, m).astype(np.float32),
             springsequilibrium=rng.uniform(3.0, 9.0, m).astype(np.float32))
    for i in zero_mass:
        a["mass"][i] = 0.0
    if optional:
        a.update(surfaceaccessibility=rng.uniform(0, 60, n).astype(np.float32),
                 hydrophobicityscale=rng.uniform(-0.05, 0.05, n).astype(np.float32),
                 hydrophobicity=rng.uniform(0, 1, n).astype(np.float32))
    a.update(override)
    with netcdf(path, "w", version=version) as f:
        f.createDimension("particle_number", None if record else n)
        f.createDimension("spatialdim", 3)
        for d in ("particlename_length", "resname_length", "chainname_length"):
            f.createDimension(d, 4)
        f.createDimension("springdim", 2)
        f.createDimension("spring_number", m)
        dims = {"coordinates": ("particle_number", "spatialdim"), "springs": ("spring_number", "springdim"),
                "springsstiffness": ("spring_number",), "springsequilibrium": ("spring_number",)}
        for name, v in a.items():
            dd = dims.get(name, ("particle_number",) + (("spatialdim",) if v.ndim == 2 and v.shape[1] == 3 else ())
                          + (("springdim",) if v.ndim == 2 and v.shape[1] == 2 else ()))
            var = f.createVariable(name, v.dtype, dd)
            var[:] = v
        for name, dim in (("particlenames", "particlename_length"), ("resnames", "resname_length"),
                          ("chainnames", "chainname_length")):
            var = f.createVariable(name, "c", ("particle_number", dim))
            var[:] = np.full((n, 4), b"A", "S1")
        f.title = "synthetic topology"
    return a


@pytest.mark.parametrize("version,record", [(1, False), (2, False), (1, True)], ids=["cdf1", "cdf2", "record"])
def test_reader_matches_scipy(tmp_path, version, record):
    path = str(tmp_path / "t.nc")
    a = write_topology(path, version=version, record=record, zero_mass=(3, 11))
    t = capi.read_nc(path)
    np.testing.assert_array_equal(t["xyz"], a["coordinates"])
    for key, name in (("charge", "charges"), ("radius", "radii"), ("epsilon", "epsilon"),
                      ("sasa", "surfaceaccessibility"), ("transfer", "hydrophobicityscale"),
                      ("hydrophobicity", "hydrophobicity")):
        np.testing.assert_array_equal(t[key], a[name])
    mass = a["mass"].copy()
    mass[[3, 11]] = 1.0  # NetCDFReader.cpp:31-37
    np.testing.assert_array_equal(t["mass"], mass)
    np.testing.assert_array_equal(t["is_static"], (a["dynamicstate"] == 0).astype(np.uint8))
    np.testing.assert_array_equal(t["ij"], a["springs"])
    np.testing.assert_array_equal(t["r0"], a["springsequilibrium"])
    np.testing.assert_array_equal(t["k"], a["springsstiffness"])


def test_optional_arrays_absent(tmp_path):
    path = str(tmp_path / "t.nc")
    write_topology(path, optional=False)
    t = capi.read_nc(path)
    assert t["sasa"] is None and t["transfer"] is None and t["hydrophobicity"] is None


def test_types_are_converted(tmp_path):
    """getVar converts: double coordinates and short ids read as the reader's float and int."""
    path = str(tmp_path / "t.nc")
    rng = np.random.default_rng(4)
    xyz = rng.uniform(-5, 5, (57, 3))
    write_topology(path, coordinates=xyz, charges=np.ones(57, np.float64))
    t = capi.read_nc(path)
    np.testing.assert_array_equal(t["xyz"], xyz.astype(np.float32))
    np.testing.assert_array_equal(t["charge"], np.ones(57, np.float32))


def test_reader_errors(tmp_path):
    cases = {
        "no_particle_dim": "Dimension \"particle_number\" not present",
        "bad_coordinates": "\"coordinates\" array has 1 dimension(s) whereas it should be 2.",
        "missing_radii": "Array \"radii\" not found in topology file.",
        "hdf5": "not a NetCDF classic file",
        "missing": "not found.",
        "bad_spring": "out of range",
    }
    for name, expect in cases.items():
        path = str(tmp_path / f"{name}.nc")
        if name == "no_particle_dim":
            with netcdf(path, "w") as f:
                f.createDimension("atoms", 3)
        elif name == "bad_coordinates":
            write_topology(path)
            with netcdf(path, "r", mmap=False) as f:
                keep = {k: (v.dimensions, v[:].copy()) for k, v in f.variables.items()}
                dims = dict(f.dimensions)
            with netcdf(path, "w") as f:
                for d, s in dims.items():
                    f.createDimension(d, s)
                for k, (dd, v) in keep.items():
                    if k == "coordinates":
                        f.createVariable(k, "f", ("particle_number",))[:] = v[:, 0]
                    else:
                        f.createVariable(k, v.dtype, dd)[:] = v
        elif name == "missing_radii":
            write_topology(path)
            with netcdf(path, "r", mmap=False) as f:
                keep = {k: (v.dimensions, v[:].copy()) for k, v in f.variables.items() if k != "radii"}
                dims = dict(f.dimensions)
            with netcdf(path, "w") as f:
                for d, s in dims.items():
                    f.createDimension(d, s)
                for k, (dd, v) in keep.items():
                    f.createVariable(k, v.dtype, dd)[:] = v
        elif name == "hdf5":
            with open(path, "wb") as fh:
                fh.write(b"\x89HDF\r\n\x1a\n" + bytes(64))
        elif name == "bad_spring":
            write_topology(path, springs=np.full((80, 2), 57, np.int32))
        with pytest.raises(BsError, match="NetCDFReader"):
            capi.read_nc(path)
        try:
            capi.read_nc(path)
        except BsError as e:
            assert expect in str(e), (name, str(e))


@pytest.mark.skipif(not os.path.exists(REF_NC), reason="the reference's example topology is not present")
def test_reference_example_topology():
    """The example topology shipped with BioSpring, against scipy's reading of it."""
    t = capi.read_nc(REF_NC)
    with netcdf(REF_NC, "r", mmap=False) as f:
        v = {k: f.variables[k][:].copy() for k in f.variables}
    assert t["xyz"].shape[0] == v["coordinates"].shape[0] == 867
    np.testing.assert_array_equal(t["xyz"], v["coordinates"])
    np.testing.assert_array_equal(t["charge"], v["charges"])
    np.testing.assert_array_equal(t["ij"], v["springs"])
    np.testing.assert_array_equal(t["k"], v["springsstiffness"])
    np.testing.assert_array_equal(t["r0"], v["springsequilibrium"])
    np.testing.assert_array_equal(t["is_static"], (v["dynamicstate"] == 0).astype(np.uint8))
    np.testing.assert_array_equal(t["sasa"], v["surfaceaccessibility"])
    assert t["hydrophobicity"] is None


def test_truncated_and_corrupted_files_fail_cleanly(tmp_path):
    """A topology cut short anywhere, or with a header byte overwritten, is either read or refused
    with an error: the reader checks every size and offset against the file before it reads."""
    src = str(tmp_path / "ok.nc")
    write_topology(src)
    data = open(src, "rb").read()
    rng = np.random.default_rng(5)
    blobs = [data[:cut] for cut in range(0, len(data), 7)]
    for _ in range(400):
        b = bytearray(data)
        b[int(rng.integers(0, min(len(b), 400)))] = int(rng.integers(0, 256))
        blobs.append(bytes(b))
    path = str(tmp_path / "t.nc")
    refused = 0
    for blob in blobs:
        with open(path, "wb") as fh:
            fh.write(blob)
        try:
            capi.read_nc(path)
        except BsError:
            refused += 1
    assert refused >= len(data) // 7  # every cut file is refused


def test_zero_length_arrays(tmp_path):
    """A topology without springs: the spring arrays have a zero-length dimension and read as empty."""
    from biospring_gb300 import capi
    path = str(tmp_path / "nosprings.nc")
    write_topology(path, n=20, m=0)
    out = capi.read_nc(path)
    assert out["ij"].shape == (0, 2) and out["r0"].shape == (0,) and out["xyz"].shape == (20, 3)
