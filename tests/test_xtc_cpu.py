"""XTC frames (bs_xtc_encode_frame / bs_xtc_decode_frame) on the CPU.

* Round trips: every coordinate comes back within half a quantisation step, over compact
  chains, uniform fills, water-like triples (the swapped first pair of a group), coordinates whose
  range needs the wide three-field form, and frames of at most 9 atoms (stored uncompressed).
* Against the reference's own writer (write_xtc of its vendored xdrfile library, compiled into
  oracle/_ref where the reference sources are present): the bytes of a file written here equal
  the bytes the reference writes for the same frames, and the reference's read_xtc reads our
  file back to the coordinates our decoder gives.
* The frame writer's XTC output (biospring_gb300.trajectory): the reference's unit and header
  conventions (Angstrom -> nm, identity box, frame counter as step and time, precision 1000).
"""

from __future__ import annotations

import ctypes as C
import os

import numpy as np
import pytest

from biospring_gb300 import build, capi
from biospring_gb300 import workloads as W
from oracle import pyoracle


@pytest.fixture(scope="module", autouse=True)
def _lib():
    if not os.path.exists(build.LIB):
        build.build_library()
    capi.load()


def _cases():
    rng = np.random.default_rng(3)
    chain = W.ca_chain(500, seed=4) / 10.0
    uniform = rng.uniform(0.0, 16.0, (3000, 3))
    waters = []
    for c in rng.uniform(0.0, 3.0, (400, 3)):
        waters += [c, c + [0.0957, 0.0, 0.0], c + [-0.024, 0.0927, 0.0]]
    waters = np.array(waters)
    # ranges beyond 2^24 quantised units (three fixed-width fields per full atom), steps small
    wide = np.concatenate([W.ca_chain(100, seed=5) / 10.0, W.ca_chain(100, seed=6) / 10.0 + 30000.0])
    sparse = rng.uniform(-30000.0, 30000.0, (50, 3))  # every step beyond the largest scale entry
    tiny = rng.uniform(-1.0, 1.0, (9, 3))
    two = rng.uniform(-1.0, 1.0, (2, 3))
    single = np.array([[0.1234, -5.0, 7.25]])
    clustered = np.concatenate([rng.normal(0.0, 0.01, (200, 3)), rng.normal(5.0, 2.0, (300, 3))])
    return {"chain": chain, "uniform": uniform, "waters": waters, "wide": wide, "sparse": sparse, "tiny9": tiny,
            "two": two, "single": single, "clustered": clustered}


CASES = _cases()


@pytest.mark.parametrize("name", list(CASES))
def test_round_trip(name):
    x = np.ascontiguousarray(CASES[name], np.float32)
    box = np.diag([3.0, 4.0, 5.0]).astype(np.float32)
    data = capi.xtc_encode(x, step=17, time=2.5, box=box, precision=1000.0)
    assert len(data) % 4 == 0
    got = capi.xtc_decode(data, x.shape[0])
    assert got["step"] == 17 and got["time"] == 2.5 and got["consumed"] == len(data)
    np.testing.assert_array_equal(got["box"], box)
    if x.shape[0] <= 9:
        np.testing.assert_array_equal(got["xyz"], x)
    else:
        assert got["precision"] == 1000.0
        err = np.abs(got["xyz"].astype(np.float64) - x).max()
        bound = 0.5 / 1000.0 + 4e-7 * np.abs(x).max()
        print(f"{name}: {x.shape[0]} atoms, {len(data)} bytes, max error {err:.2e} nm")
        assert err <= bound


def test_corrupt_frames_are_refused():
    x = np.ascontiguousarray(CASES["uniform"], np.float32)
    data = capi.xtc_encode(x, 0, 0.0)
    with pytest.raises(capi.BsError):
        capi.xtc_decode(data[:-40], x.shape[0])
    with pytest.raises(capi.BsError):
        capi.xtc_decode(data, x.shape[0] + 1)
    bad = bytearray(data)
    bad[3] ^= 0xFF  # magic
    with pytest.raises(capi.BsError):
        capi.xtc_decode(bytes(bad), x.shape[0])


def _reference_xdr():
    if not pyoracle.have_reference():
        pytest.skip("compiled reference (oracle/_ref) absent: its xdrfile library is not available here")
    lib = C.CDLL(pyoracle.REF_SO)
    lib.xdrfile_open.restype = C.c_void_p
    lib.xdrfile_open.argtypes = [C.c_char_p, C.c_char_p]
    lib.xdrfile_close.restype = C.c_int
    lib.xdrfile_close.argtypes = [C.c_void_p]
    lib.write_xtc.restype = C.c_int
    lib.write_xtc.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_float, C.POINTER(C.c_float), C.POINTER(C.c_float),
                              C.c_float]
    lib.read_xtc.restype = C.c_int
    lib.read_xtc.argtypes = [C.c_void_p, C.c_int, C.POINTER(C.c_int), C.POINTER(C.c_float), C.POINTER(C.c_float),
                             C.POINTER(C.c_float), C.POINTER(C.c_float)]
    return lib


def _f(a):
    return a.ctypes.data_as(C.POINTER(C.c_float))


@pytest.mark.parametrize("name", [k for k in CASES if k not in ("wide", "sparse")])
def test_bytes_equal_the_reference_writer(name, tmp_path):
    lib = _reference_xdr()
    x = np.ascontiguousarray(CASES[name], np.float32)
    frames = [x, (x + np.float32(0.0123)).astype(np.float32), (x * np.float32(1.01)).astype(np.float32)]
    box = np.eye(3, dtype=np.float32)
    path = str(tmp_path / "ref.xtc")
    xd = lib.xdrfile_open(path.encode(), b"w")
    assert xd
    for k, fr in enumerate(frames):
        assert lib.write_xtc(xd, fr.shape[0], k, float(k), _f(box), _f(np.ascontiguousarray(fr)), 1000.0) == 0
    lib.xdrfile_close(xd)
    ours = b"".join(capi.xtc_encode(fr, k, float(k), box, 1000.0) for k, fr in enumerate(frames))
    with open(path, "rb") as f:
        theirs = f.read()
    print(f"{name}: {len(ours)} bytes ours, {len(theirs)} bytes the reference's")
    assert ours == theirs
    # the reference reads our bytes back to what our decoder gives
    mine = str(tmp_path / "ours.xtc")
    with open(mine, "wb") as f:
        f.write(ours)
    xd = lib.xdrfile_open(mine.encode(), b"r")
    off = 0
    for k, fr in enumerate(frames):
        step, t, prec = C.c_int(), C.c_float(), C.c_float()
        b = np.zeros((3, 3), np.float32)
        got = np.zeros_like(fr)
        assert lib.read_xtc(xd, fr.shape[0], C.byref(step), C.byref(t), _f(b), _f(got), C.byref(prec)) == 0
        dec = capi.xtc_decode(ours, fr.shape[0], off)
        off += dec["consumed"]
        assert step.value == k == dec["step"]
        np.testing.assert_array_equal(got, dec["xyz"])
    lib.xdrfile_close(xd)


def test_wide_range_read_by_the_reference(tmp_path):
    """Coordinate ranges beyond 2^24 quantised units take the three-field form; the reference's
    reader decodes our frame to the coordinates our decoder gives."""
    lib = _reference_xdr()
    x = np.ascontiguousarray(CASES["wide"], np.float32)
    data = capi.xtc_encode(x, 3, 3.0, None, 1000.0)
    path = str(tmp_path / "wide.xtc")
    with open(path, "wb") as f:
        f.write(data)
    xd = lib.xdrfile_open(path.encode(), b"r")
    step, t, prec = C.c_int(), C.c_float(), C.c_float()
    b = np.zeros((3, 3), np.float32)
    got = np.zeros_like(x)
    assert lib.read_xtc(xd, x.shape[0], C.byref(step), C.byref(t), _f(b), _f(got), C.byref(prec)) == 0
    lib.xdrfile_close(xd)
    np.testing.assert_array_equal(got, capi.xtc_decode(data, x.shape[0])["xyz"])


class _FakeRing:
    """Stands in for a network's frame ring: two frames, then nothing."""

    def __init__(self, frames):
        self.frames = list(frames)

    def readFrames(self, max_frames):
        if not self.frames:
            return np.zeros(0, np.int64), np.zeros((0, 1, 3), np.float32), np.zeros((0, 6)), 0
        steps = np.array([s for s, _ in self.frames], np.int64)
        xyz = np.stack([x for _, x in self.frames])
        self.frames = []
        return steps, xyz, np.zeros((len(steps), 6)), 0

    def synchronize(self):
        pass


def test_frame_writer_xtc_follows_the_reference_conventions(tmp_path):
    from biospring_gb300 import trajectory as T
    rng = np.random.default_rng(8)
    frames = [(10, rng.uniform(-40.0, 40.0, (300, 3)).astype(np.float32)),
              (20, rng.uniform(-40.0, 40.0, (300, 3)).astype(np.float32))]
    path = str(tmp_path / "traj.xtc")
    w = T.FrameWriter(_FakeRing(frames), xtc_path=path, poll=0.001)
    assert w.close() == (2, 0)
    with open(path, "rb") as f:
        data = f.read()
    off = 0
    for k, (_, x) in enumerate(frames):
        got = capi.xtc_decode(data, x.shape[0], off)
        off += got["consumed"]
        assert got["step"] == k and got["time"] == float(k) and got["precision"] == 1000.0
        np.testing.assert_array_equal(got["box"], np.eye(3, dtype=np.float32))
        nm = (x.astype(np.float64) / 10.0).astype(np.float32)
        assert np.abs(got["xyz"] - nm).max() <= 0.5e-3 + 1e-6
    assert off == len(data)
