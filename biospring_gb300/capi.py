"""ctypes view of the C ABI declared in ``include/biospring_gb300.h``.

The shared library is loaded from the package directory; there is no fallback: a
missing or unloadable library raises, so nothing silently runs on the CPU.
"""

from __future__ import annotations

import ctypes as C
import os

import numpy as np

PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(PKG, "libbiospring_gb300.so")

BS_OK = 0
BS_E_ARG = 1
BS_E_CUDA = 2
BS_E_NONFINITE = 3
BS_E_CAPACITY = 4
BS_E_TIMEOUT = 5
BS_E_STATE = 6

BS_STERIC_LINEAR = 0
BS_STERIC_LJ_12_6_AMBER = 1
BS_STERIC_LJ_8_6_LEWITT = 2
BS_STERIC_LJ_8_6_ZACHARIAS = 3
STERIC_MODES = {
    "linear": BS_STERIC_LINEAR,
    "lennard-jones-12-6Amber": BS_STERIC_LJ_12_6_AMBER,
    "lennard-jones-8-6Lewitt": BS_STERIC_LJ_8_6_LEWITT,
    "lennard-jones-8-6Zacharias": BS_STERIC_LJ_8_6_ZACHARIAS,
}

BS_DIELECTRIC_CONSTANT = 0
BS_DIELECTRIC_DISTANCE = 1

BS_GRID_POTENTIAL = 0
BS_GRID_DENSITY = 1

BS_TERM_STERIC = 0
BS_TERM_COULOMB = 1
BS_TERM_HYDROPHOBIC = 2

ENERGY_NAMES = ("kinetic", "spring", "steric", "electrostatic", "imp", "hydrophobic")


class BsConfig(C.Structure):
    """Mirror of ``bs_config`` (field order and types must match the header)."""

    _fields_ = [
        ("nbsteps", C.c_int32),
        ("timestep", C.c_double),
        ("neighborskin", C.c_double),
        ("spring_enable", C.c_int32),
        ("spring_scale", C.c_double),
        ("steric_enable", C.c_int32),
        ("steric_gridscale", C.c_double),
        ("steric_cutoff", C.c_double),
        ("steric_mode", C.c_int32),
        ("coulomb_enable", C.c_int32),
        ("coulomb_scale", C.c_double),
        ("coulomb_cutoff", C.c_double),
        ("coulomb_dielectric", C.c_double),
        ("hydrophobicity_enable", C.c_int32),
        ("hydrophobicity_scale", C.c_double),
        ("hydrophobicity_cutoff", C.c_double),
        ("impala_enable", C.c_int32),
        ("impala_scale", C.c_double),
        ("viscosity_enable", C.c_int32),
        ("viscosity_value", C.c_double),
        ("rigidbody_enable", C.c_int32),
        ("dielectric_mode", C.c_int32),
        ("impala_z0", C.c_double),
        ("impala_alpha", C.c_double),
        ("rebuild_every", C.c_int32),
        ("list_skin", C.c_double),
        ("precise_positions", C.c_int32),
        ("probe_enable", C.c_int32),
        ("probe_electrostatic", C.c_int32),
        ("probe_steric", C.c_int32),
        ("probe_x", C.c_double),
        ("probe_y", C.c_double),
        ("probe_z", C.c_double),
        ("probe_mass", C.c_double),
        ("probe_epsilon", C.c_double),
        ("probe_radius", C.c_double),
        ("probe_charge", C.c_double),
        ("potentialgrid_enable", C.c_int32),
        ("densitygrid_enable", C.c_int32),
        ("potentialgrid_scale", C.c_double),
        ("densitygrid_scale", C.c_double),
        ("potentialgrid_path", C.c_char * 512),
        ("densitygrid_path", C.c_char * 512),
    ]

    def to_dict(self) -> dict:
        return {name: getattr(self, name) for name, _ in self._fields_}


_f32p = C.POINTER(C.c_float)
_i32p = C.POINTER(C.c_int32)
_i64p = C.POINTER(C.c_int64)
_u8p = C.POINTER(C.c_uint8)
_f64p = C.POINTER(C.c_double)

# name -> (restype, argtypes); every function of the header
SIGNATURES = {
    "bs_default_config": (C.c_int, [C.POINTER(BsConfig)]),
    "bs_config_parse_msp": (C.c_int, [C.c_char_p, C.POINTER(BsConfig), C.c_char_p, C.c_size_t]),
    "bs_create": (C.c_int, [C.POINTER(C.c_void_p)]),
    "bs_destroy": (C.c_int, [C.c_void_p]),
    "bs_upload_particles": (C.c_int, [C.c_void_p, C.c_int64, _f32p, _f32p, _f32p, _f32p, _f32p, _f32p, _f32p,
                                      _f32p, _f32p, _u8p]),
    "bs_upload_springs": (C.c_int, [C.c_void_p, C.c_int64, _i32p, _f32p, _f32p]),
    "bs_set_rigid_bodies": (C.c_int, [C.c_void_p, C.c_int32, _i32p, _i32p]),
    "bs_set_frames": (C.c_int, [C.c_void_p, C.c_int32, C.c_int32]),
    "bs_read_frames": (C.c_int, [C.c_void_p, C.c_int32, _i64p, _f32p, _f64p, _i32p, _i64p]),
    "bs_load_nc": (C.c_int, [C.c_void_p, C.c_char_p, _i64p, _i64p]),
    "bs_read_nc": (C.c_int, [C.c_char_p, _i64p, _i64p, _f32p, _f32p, _f32p, _f32p, _f32p, _f32p, _f32p, _f32p,
                             _u8p, _i32p, _f32p, _f32p, _i32p, C.c_char_p, C.c_size_t]),
    "bs_set_field_grid": (C.c_int, [C.c_void_p, C.c_int32, _i32p, _f64p, _f64p, _f32p]),
    "bs_read_dx": (C.c_int, [C.c_char_p, _i32p, _f64p, _f64p, _f32p, C.c_char_p, C.c_size_t]),
    "bs_get_field_grid": (C.c_int, [C.c_void_p, C.c_int32, _i32p, _f32p]),
    "bs_set_burying": (C.c_int, [C.c_void_p, _f32p]),
    "bs_set_charges": (C.c_int, [C.c_void_p, _f32p]),
    "bs_set_membrane": (C.c_int, [C.c_void_p, C.c_float, C.c_float, C.c_float, C.c_float]),
    "bs_setup": (C.c_int, [C.c_void_p, C.POINTER(BsConfig)]),
    "bs_step": (C.c_int, [C.c_void_p, C.c_int32]),
    "bs_step_async": (C.c_int, [C.c_void_p, C.c_int32]),
    "bs_synchronize": (C.c_int, [C.c_void_p]),
    "bs_get_step_count": (C.c_int, [C.c_void_p, _i64p]),
    "bs_get_stream": (C.c_int, [C.c_void_p, C.POINTER(C.c_void_p)]),
    "bs_launch_phase": (C.c_int, [C.c_void_p, C.c_int32]),
    "bs_compute_forces": (C.c_int, [C.c_void_p]),
    "bs_get_positions": (C.c_int, [C.c_void_p, _f32p]),
    "bs_get_velocities": (C.c_int, [C.c_void_p, _f32p]),
    "bs_get_forces": (C.c_int, [C.c_void_p, _f32p]),
    "bs_set_positions": (C.c_int, [C.c_void_p, _f32p]),
    "bs_set_velocities": (C.c_int, [C.c_void_p, _f32p]),
    "bs_set_force": (C.c_int, [C.c_void_p, C.c_int64, _f32p]),
    "bs_set_external_forces": (C.c_int, [C.c_void_p, _f32p]),
    "bs_set_external_forces_async": (C.c_int, [C.c_void_p, _f32p]),
    "bs_get_energies": (C.c_int, [C.c_void_p, _f64p]),
    "bs_get_pairs": (C.c_int, [C.c_void_p, C.c_int32, _i64p, C.c_int64, _i64p]),
    "bs_get_cells": (C.c_int, [C.c_void_p, C.c_int32, _i64p]),
    "bs_get_launch_count": (C.c_int, [C.c_void_p, _i64p]),
    "bs_last_error": (C.c_int, [C.c_void_p, C.c_char_p, C.c_size_t]),
    "bs_set_systems": (C.c_int, [C.c_void_p, C.c_int32, _i64p]),
    "bs_get_probe": (C.c_int, [C.c_void_p, _f32p]),
    "bs_get_spring_count": (C.c_int, [C.c_void_p, _i64p]),
    "bs_set_spring_parameters": (C.c_int, [C.c_void_p, _f32p, _f32p]),
    "bs_adjoint": (C.c_int, [C.c_void_p, C.c_int32, C.c_int32, _f32p, _f64p, _f32p, _f32p, _f32p]),
    "bs_get_system_energies": (C.c_int, [C.c_void_p, _f64p]),
    "bs_set_batch_shape": (C.c_int, [C.c_void_p, C.c_int32, C.c_int32, C.c_int32]),
    "bs_get_batch_shape": (C.c_int, [C.c_void_p, _i32p]),
    "bs_batch_autotune": (C.c_int, [C.c_void_p, _i32p]),
    "bs_xtc_frame_bound": (C.c_int, [C.c_int64, C.POINTER(C.c_size_t)]),
    "bs_xtc_encode_frame": (C.c_int, [C.c_int64, C.c_int32, C.c_float, _f32p, _f32p, C.c_float,
                                      C.POINTER(C.c_uint8), C.c_size_t, C.POINTER(C.c_size_t)]),
    "bs_xtc_decode_frame": (C.c_int, [C.POINTER(C.c_uint8), C.c_size_t, C.c_int64, C.POINTER(C.c_int32),
                                      C.POINTER(C.c_float), _f32p, _f32p, C.POINTER(C.c_float),
                                      C.POINTER(C.c_size_t)]),
}

_lib = None


def load(path: str = LIB_PATH) -> C.CDLL:
    """Loads the CUDA library (raises if it is missing: there is no CPU fallback)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise RuntimeError(
            f"{path} is missing: build it first (python -c 'import __graft_entry__ as g; g.build()')")
    lib = C.CDLL(path)
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


class BsError(RuntimeError):
    def __init__(self, code: int, message: str):
        super().__init__(f"[{code}] {message}")
        self.code = code


def ptr(a: np.ndarray | None, ctype):
    if a is None:
        return None
    return a.ctypes.data_as(C.POINTER(ctype))


def default_config() -> BsConfig:
    cfg = BsConfig()
    load().bs_default_config(C.byref(cfg))
    return cfg


def read_nc(path: str) -> dict:
    """A BioSpring topology from a NetCDF classic file (bs_read_nc): per-particle arrays and the
    springs; the optional arrays are None when the file does not hold them."""
    import numpy as np
    lib = load()
    n = C.c_int64()
    m = C.c_int64()
    err = C.create_string_buffer(512)
    nul = [None] * 13
    rc = lib.bs_read_nc(str(path).encode(), C.byref(n), C.byref(m), *nul, err, 512)
    if rc != BS_OK:
        raise BsError(rc, err.value.decode())
    f = lambda *shape: np.zeros(shape, np.float32)  # noqa: E731
    out = dict(xyz=f(n.value, 3), mass=f(n.value), charge=f(n.value), radius=f(n.value), epsilon=f(n.value),
               sasa=f(n.value), transfer=f(n.value), hydrophobicity=f(n.value),
               is_static=np.zeros(n.value, np.uint8), ij=np.zeros((m.value, 2), np.int32), r0=f(m.value),
               k=f(m.value))
    present = np.zeros(3, np.int32)
    p = lambda a, t: a.ctypes.data_as(C.POINTER(t))  # noqa: E731
    rc = lib.bs_read_nc(str(path).encode(), C.byref(n), C.byref(m), p(out["xyz"], C.c_float),
                        p(out["mass"], C.c_float), p(out["charge"], C.c_float), p(out["radius"], C.c_float),
                        p(out["epsilon"], C.c_float), p(out["sasa"], C.c_float), p(out["transfer"], C.c_float),
                        p(out["hydrophobicity"], C.c_float), p(out["is_static"], C.c_uint8),
                        p(out["ij"], C.c_int32), p(out["r0"], C.c_float), p(out["k"], C.c_float),
                        p(present, C.c_int32), err, 512)
    if rc != BS_OK:
        raise BsError(rc, err.value.decode())
    for flag, key in zip(present, ("sasa", "transfer", "hydrophobicity")):
        if not flag:
            out[key] = None
    return out


def xtc_encode(xyz_nm, step: int, time: float, box=None, precision: float = 1000.0) -> bytes:
    """One XTC frame (bs_xtc_encode_frame) of float (n, 3) coordinates in nm."""
    lib = load()
    x = np.ascontiguousarray(xyz_nm, np.float32).reshape(-1, 3)
    n = x.shape[0]
    cap = C.c_size_t()
    lib.bs_xtc_frame_bound(n, C.byref(cap))
    out = np.zeros(cap.value, np.uint8)
    size = C.c_size_t()
    b = None if box is None else np.ascontiguousarray(box, np.float32).reshape(9)
    rc = lib.bs_xtc_encode_frame(n, int(step), float(time), ptr(b, C.c_float), ptr(x, C.c_float), float(precision),
                                 out.ctypes.data_as(C.POINTER(C.c_uint8)), cap.value, C.byref(size))
    if rc != BS_OK:
        raise BsError(rc, "bs_xtc_encode_frame failed (coordinates too large for the precision?)")
    return out[:size.value].tobytes()


def xtc_decode(data: bytes, natoms: int, offset: int = 0) -> dict:
    """One XTC frame of natoms atoms read from data[offset:] (bs_xtc_decode_frame)."""
    lib = load()
    buf = np.frombuffer(data, np.uint8)[offset:]
    buf = np.ascontiguousarray(buf)
    xyz = np.zeros((natoms, 3), np.float32)
    box = np.zeros(9, np.float32)
    step, t, prec, used = C.c_int32(), C.c_float(), C.c_float(), C.c_size_t()
    rc = lib.bs_xtc_decode_frame(buf.ctypes.data_as(C.POINTER(C.c_uint8)), buf.shape[0], natoms, C.byref(step),
                                 C.byref(t), ptr(box, C.c_float), ptr(xyz, C.c_float), C.byref(prec), C.byref(used))
    if rc != BS_OK:
        raise BsError(rc, "bs_xtc_decode_frame: not a valid XTC frame of that many atoms")
    return dict(step=step.value, time=t.value, box=box.reshape(3, 3), xyz=xyz, precision=prec.value,
                consumed=used.value)


def parse_msp(text: str, base: BsConfig | None = None) -> BsConfig:
    cfg = base if base is not None else default_config()
    err = C.create_string_buffer(512)
    rc = load().bs_config_parse_msp(text.encode(), C.byref(cfg), err, 512)
    if rc != BS_OK:
        raise BsError(rc, err.value.decode())
    return cfg
