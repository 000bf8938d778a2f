"""TEST INFRASTRUCTURE: ctypes access to the CPU oracle and to the compiled reference.

* ``Oracle``    -- the CPU restatement in oracle/bs_oracle.cpp (libbs_oracle.so), built on
  any machine by :func:`build_oracle`.
* ``Reference`` -- the unmodified reference engine compiled from its sources by oracle/ref.mk
  into oracle/_ref/libbsref.so; only present where the reference sources are.

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg use this module, and
only as the checker or the timed CPU baseline, never as the product path.
"""

from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ORACLE_SO = os.path.join(HERE, "libbs_oracle.so")
REF_SO = os.path.join(HERE, "_ref", "libbsref.so")


# The seeded generators of the synthetic systems (host C++, no CUDA) are compiled into the
# oracle's library as well, so that a CPU run builds its system without mapping any product
# library; the same source and seed give the same coordinates.
SYNTH_SRC = os.path.join(os.path.dirname(HERE), "biospring_gb300", "csrc", "synth.cpp")


def build_oracle() -> str:
    srcs = [os.path.join(HERE, "bs_oracle.cpp"), os.path.join(HERE, "adjoint_fp64.cpp"), SYNTH_SRC]
    hdr = os.path.join(os.path.dirname(HERE), "include", "biospring_gb300.h")
    if (not os.path.exists(ORACLE_SO) or os.path.getmtime(ORACLE_SO) < max([os.path.getmtime(f) for f in srcs] +
                                                                           [os.path.getmtime(hdr)])):
        subprocess.run(["g++", "-std=c++17", "-O2", "-fopenmp", "-ffp-contract=off", "-fPIC", "-shared", *srcs,
                        "-o", ORACLE_SO], check=True)
    return ORACLE_SO


# Where this container mounts the reference's sources; $REF overrides it. The GPU machines have
# no copy, and there nothing is built from it.
DEFAULT_REF = "/root/reference"


def build_reference() -> str | None:
    """Builds oracle/_ref/libbsref.so when the reference sources are present (make -f oracle/ref.mk)."""
    ref = reference_dir()
    if not ref:
        return REF_SO if os.path.exists(REF_SO) else None
    proc = subprocess.run(["make", "-s", "-f", os.path.join(HERE, "ref.mk"), f"REF={ref}",
                           f"-j{os.cpu_count() or 4}"],
                          cwd=os.path.dirname(HERE), stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if proc.returncode != 0:
        raise RuntimeError("reference build failed:\n" + proc.stdout[-4000:])
    return REF_SO if os.path.exists(REF_SO) else None


def reference_dir() -> str:
    """The reference source tree: $REF, else the default mount when it holds the sources; empty
    where there is none."""
    ref = os.environ.get("REF") or DEFAULT_REF
    return ref if os.path.exists(os.path.join(ref, "src", "spn", "SpringNetwork.cpp")) else ""


def have_reference() -> bool:
    return os.path.exists(REF_SO)


def use_oracle_generator() -> None:
    """Makes biospring_gb300.workloads generate systems with the oracle library's copy of the
    generators (no product library is loaded)."""
    from biospring_gb300 import workloads
    workloads.set_generator_library(build_oracle())


def oracle_config(system):
    """The system's run parameters over the reference's defaults as the oracle restates them
    (bso_default_config), without the product library."""
    from biospring_gb300.capi import BsConfig
    lib = C.CDLL(build_oracle())
    lib.bso_default_config.restype = None
    lib.bso_default_config.argtypes = [C.POINTER(BsConfig)]
    cfg = BsConfig()
    lib.bso_default_config(C.byref(cfg))
    for key, v in system.config.items():
        setattr(cfg, key, v)
    return cfg


_f32p = C.POINTER(C.c_float)
_i32p = C.POINTER(C.c_int32)
_i64p = C.POINTER(C.c_int64)
_u8p = C.POINTER(C.c_uint8)
_f64p = C.POINTER(C.c_double)


def _bind(lib, prefix: str, cfg_type):
    sig = {
        "create": (C.c_void_p, [C.POINTER(cfg_type), C.c_int64, _f32p, _f32p, _f32p, _f32p, _f32p, _f32p, _f32p,
                                _f32p, _f32p, _u8p, C.c_int64, _i32p, _f32p, _f32p]),
        "destroy": (None, [C.c_void_p]),
        "step": (C.c_int, [C.c_void_p, C.c_int32]),
        "time_steps": (C.c_double, [C.c_void_p, C.c_int32]),
        "compute_forces": (C.c_int, [C.c_void_p]),
        "get_positions": (None, [C.c_void_p, _f32p]),
        "get_velocities": (None, [C.c_void_p, _f32p]),
        "get_forces": (None, [C.c_void_p, _f32p]),
        "set_positions": (None, [C.c_void_p, _f32p]),
        "get_energies": (None, [C.c_void_p, _f64p]),
        "get_pairs": (C.c_int64, [C.c_void_p, C.c_int32, _i64p, C.c_int64]),
        "get_cells": (C.c_int, [C.c_void_p, C.c_int32, _i64p]),
    }
    sig["get_probe"] = (None, [C.c_void_p, _f32p])
    sig["set_membrane"] = (None, [C.c_void_p, C.c_float, C.c_float, C.c_float, C.c_float])
    sig["set_burying"] = (None, [C.c_void_p, _f32p])
    if prefix == "bsref_":
        sig["get_field_grid"] = (None, [C.c_void_p, C.c_int32, _i32p, _f32p])
    if prefix == "bso_":
        sig["set_rigid_bodies"] = (C.c_int, [C.c_void_p, C.c_int32, _i32p, _i32p])
        sig["set_velocities"] = (None, [C.c_void_p, _f32p])
        sig["eval_fp64"] = (C.c_int, [C.c_void_p, _f64p, _f64p])
        sig["set_field_grid"] = (None, [C.c_void_p, C.c_int32, _i32p, _f64p, _f64p, _f32p])
        sig["get_field_grid"] = (None, [C.c_void_p, C.c_int32, _f32p])
    fns = {}
    for name, (res, args) in sig.items():
        fn = getattr(lib, prefix + name)
        fn.restype = res
        fn.argtypes = args
        fns[name] = fn
    return fns


def _p(a, t):
    return None if a is None else a.ctypes.data_as(C.POINTER(t))


class _CpuSim:
    _lib = None
    _fns = None
    PREFIX = ""
    PATH = ""

    @classmethod
    def _load(cls):
        from biospring_gb300.capi import BsConfig
        if cls._fns is None:
            if not os.path.exists(cls.PATH):
                raise RuntimeError(f"{cls.PATH} is missing")
            cls._lib = C.CDLL(cls.PATH)
            cls._fns = _bind(cls._lib, cls.PREFIX, BsConfig)
        return cls._fns

    def __init__(self, system, cfg=None):
        f = self._load()
        cfg = oracle_config(system) if cfg is None else cfg
        self.cfg = cfg
        a = {k: (None if v is None else np.ascontiguousarray(v)) for k, v in system.arrays().items()}
        self._keep = a
        xyz = np.ascontiguousarray(a["xyz"], np.float32)
        f32 = lambda k: None if a[k] is None else np.ascontiguousarray(a[k], np.float32)  # noqa: E731
        self._arr = [xyz] + [f32(k) for k in ("vel", "mass", "charge", "radius", "epsilon", "hydrophobicity",
                                              "sasa", "transfer")]
        st = None if a["is_static"] is None else np.ascontiguousarray(a["is_static"], np.uint8)
        self._st = st
        ij = np.ascontiguousarray(system.ij, np.int32)
        r0 = np.ascontiguousarray(system.r0, np.float32)
        k = np.ascontiguousarray(system.k, np.float32)
        self._sp = (ij, r0, k)
        self.n = system.n
        self.h = f["create"](C.byref(cfg), self.n, *[_p(x, C.c_float) for x in self._arr], _p(st, C.c_uint8),
                             ij.shape[0], _p(ij, C.c_int32), _p(r0, C.c_float), _p(k, C.c_float))

    def close(self):
        if getattr(self, "h", None):
            self._fns["destroy"](self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def step(self, n=1):
        rc = self._fns["step"](self.h, int(n))
        if rc != 0:
            raise RuntimeError(f"oracle step failed with code {rc}")

    def time_steps(self, n):
        return self._fns["time_steps"](self.h, int(n))

    def compute_forces(self):
        self._fns["compute_forces"](self.h)

    def _get3(self, name):
        out = np.zeros((self.n, 3), np.float32)
        self._fns[name](self.h, _p(out, C.c_float))
        return out

    def probe(self):
        out = np.zeros(6, np.float32)
        self._fns["get_probe"](self.h, _p(out, C.c_float))
        return out

    def positions(self):
        return self._get3("get_positions")

    def velocities(self):
        return self._get3("get_velocities")

    def forces(self):
        return self._get3("get_forces")

    def set_positions(self, xyz):
        xyz = np.ascontiguousarray(xyz, np.float32)
        self._fns["set_positions"](self.h, _p(xyz, C.c_float))

    def energies(self):
        out = np.zeros(6, np.float64)
        self._fns["get_energies"](self.h, _p(out, C.c_double))
        return out

    def pairs(self, term):
        n = self._fns["get_pairs"](self.h, term, None, 0)
        out = np.zeros((max(n, 1), 2), np.int64)
        self._fns["get_pairs"](self.h, term, _p(out, C.c_int64), n)
        out = out[:n]
        return out[np.lexsort((out[:, 1], out[:, 0]))]

    def cells(self, term):
        out = np.zeros(self.n, np.int64)
        self._fns["get_cells"](self.h, term, _p(out, C.c_int64))
        return out

    def set_membrane(self, upper_offset=0.0, lower_offset=0.0, upper_curvature=0.0, lower_curvature=0.0):
        self._fns["set_membrane"](self.h, float(upper_offset), float(lower_offset), float(upper_curvature),
                                  float(lower_curvature))

    def set_burying(self, b):
        self._bur = np.ascontiguousarray(b, np.float32)
        self._fns["set_burying"](self.h, _p(self._bur, C.c_float))


class Oracle(_CpuSim):
    PREFIX = "bso_"
    PATH = ORACLE_SO

    def __init__(self, system, cfg=None):
        super().__init__(system, cfg)
        if system.bodies and self.cfg.rigidbody_enable:
            self.set_rigid_bodies(system.bodies)

    def set_rigid_bodies(self, bodies):
        offsets = np.zeros(len(bodies) + 1, np.int32)
        for b, ids in enumerate(bodies):
            offsets[b + 1] = offsets[b] + len(ids)
        ids = np.ascontiguousarray(np.concatenate([np.asarray(b, np.int32) for b in bodies]), np.int32)
        self._fns["set_rigid_bodies"](self.h, len(bodies), _p(offsets, C.c_int32), _p(ids, C.c_int32))

    def set_velocities(self, v):
        v = np.ascontiguousarray(v, np.float32)
        self._fns["set_velocities"](self.h, _p(v, C.c_float))

    def set_field_grid(self, which, scalar, origin, spacing):
        """Grid `which` (0 potential, 1 density) from a (n0, n1, n2) array of scalar values."""
        sc = np.ascontiguousarray(scalar, np.float32)
        shape = np.asarray(sc.shape, np.int32)
        o = np.asarray(origin, np.float64)
        h = np.asarray(spacing, np.float64)
        self._fns["set_field_grid"](self.h, int(which), _p(shape, C.c_int32), _p(o, C.c_double), _p(h, C.c_double),
                                    _p(sc, C.c_float))
        self._grid_shape = getattr(self, "_grid_shape", {})
        self._grid_shape[which] = tuple(sc.shape)

    def field_grid(self, which):
        out = np.zeros(self._grid_shape[which] + (4,), np.float32)
        self._fns["get_field_grid"](self.h, int(which), _p(out, C.c_float))
        return out

    def eval_fp64(self):
        f = np.zeros((self.n, 3), np.float64)
        e = np.zeros(6, np.float64)
        self._fns["eval_fp64"](self.h, _p(f, C.c_double), _p(e, C.c_double))
        return f, e


class Reference(_CpuSim):
    PREFIX = "bsref_"
    PATH = REF_SO

    def field_grid(self, which):
        shape = np.zeros(3, np.int32)
        self._fns["get_field_grid"](self.h, int(which), _p(shape, C.c_int32), None)
        out = np.zeros(tuple(int(v) for v in shape) + (4,), np.float32)
        self._fns["get_field_grid"](self.h, int(which), _p(shape, C.c_int32), _p(out, C.c_float))
        return out


# ---- FP64 gradient reference (adjoint_fp64.cpp) ------------------------------------------

_ADJ = None


def _adj_lib():
    global _ADJ
    if _ADJ is None:
        lib = C.CDLL(ORACLE_SO)
        common = [C.c_int64, _f32p, _f32p, _f32p, _f32p, _u8p, C.c_int64, _i32p, _f32p, _f32p, C.c_double, C.c_int,
                  C.c_double, C.c_int, C.c_double, C.c_double, C.c_int, C.c_double,
                  _f32p, C.c_int, C.c_double, C.c_double, C.c_int, C.c_int32, _f32p]
        lib.bso_loss_fp64.restype = C.c_double
        lib.bso_loss_fp64.argtypes = common
        lib.bso_adjoint_fp64.restype = C.c_int
        lib.bso_adjoint_fp64.argtypes = common + [_f64p, _f64p, _f64p, _f64p]
        lib.bso_fd_fp64.restype = C.c_int
        lib.bso_fd_fp64.argtypes = common + [C.c_int64, _i64p, C.c_double, _f64p, _f64p]
        lib.bso_fd_q_fp64.restype = C.c_int
        lib.bso_fd_q_fp64.argtypes = common + [C.c_int64, _i64p, C.c_double, _f64p]
        _ADJ = lib
    return _ADJ


def _adj_args(system, nsteps, target):
    cfg = oracle_config(system)
    a = system.arrays()
    f32 = lambda v: None if v is None else np.ascontiguousarray(v, np.float32)  # noqa: E731
    keep = dict(xyz=f32(a["xyz"]).reshape(-1), vel=f32(a["vel"]), mass=f32(a["mass"]), radius=f32(a["radius"]),
                st=None if a["is_static"] is None else np.ascontiguousarray(a["is_static"], np.uint8),
                ij=np.ascontiguousarray(system.ij, np.int32), k=f32(system.k), r0=f32(system.r0),
                target=f32(target).reshape(-1), q=f32(a["charge"]))
    # Coulomb constant C = conversion / (4 pi) * scale / dielectric (the device's k_elec_f, in double)
    newton = 1.0e10 * (1.0 / 1.66054e-27) * 1.0e-15 * 1.0e-15
    elec = newton * (1.60217653e-19 ** 2) / (8.854187817e-12 * 1.0e-10 * 1.0e-10) / (4.0 * 3.1415927)
    coul_c = elec * float(cfg.coulomb_scale) / float(cfg.coulomb_dielectric)
    args = [system.n, _p(keep["xyz"], C.c_float), _p(keep["vel"], C.c_float), _p(keep["mass"], C.c_float),
            _p(keep["radius"], C.c_float), _p(keep["st"], C.c_uint8), int(system.ij.shape[0]),
            _p(keep["ij"], C.c_int32), _p(keep["k"], C.c_float), _p(keep["r0"], C.c_float), float(cfg.timestep),
            int(cfg.spring_enable), float(cfg.spring_scale), int(cfg.steric_enable), float(cfg.steric_cutoff),
            float(cfg.steric_gridscale), int(cfg.viscosity_enable), float(cfg.viscosity_value),
            _p(keep["q"], C.c_float), int(cfg.coulomb_enable), float(cfg.coulomb_cutoff), coul_c,
            int(cfg.dielectric_mode == 1), int(nsteps), _p(keep["target"], C.c_float)]
    return args, keep


def loss_fp64(system, nsteps: int, target) -> float:
    """L = (1/n) sum |x(nsteps) - target|^2 of the FP64 restated dynamics."""
    args, _keep = _adj_args(system, nsteps, target)
    return float(_adj_lib().bso_loss_fp64(*args))


def adjoint_fp64(system, nsteps: int, target, with_charges: bool = False):
    """(L, dL/dk, dL/dr0) by the FP64 discrete adjoint; one entry per distinct spring. With
    with_charges, dL/dq of every particle is returned fourth."""
    args, _keep = _adj_args(system, nsteps, target)
    ns = system.ij.shape[0]
    gk = np.zeros(max(ns, 1), np.float64)
    gr = np.zeros(max(ns, 1), np.float64)
    gq = np.zeros(system.n, np.float64)
    loss = C.c_double()
    _adj_lib().bso_adjoint_fp64(*args, C.byref(loss), _p(gk, C.c_double), _p(gr, C.c_double), _p(gq, C.c_double))
    if with_charges:
        return loss.value, gk[:ns], gr[:ns], gq
    return loss.value, gk[:ns], gr[:ns]


def fd_q_fp64(system, nsteps: int, target, particles, h: float = 1e-4):
    """Central finite differences of the FP64 loss with respect to the given particles' charges."""
    args, _keep = _adj_args(system, nsteps, target)
    sel = np.ascontiguousarray(particles, np.int64)
    fq = np.zeros(sel.shape[0], np.float64)
    _adj_lib().bso_fd_q_fp64(*args, sel.shape[0], _p(sel, C.c_int64), float(h), _p(fq, C.c_double))
    return fq


def fd_fp64(system, nsteps: int, target, springs, h: float = 1e-4):
    """Central finite differences of the FP64 loss with respect to k and r0 of the given springs."""
    args, _keep = _adj_args(system, nsteps, target)
    sel = np.ascontiguousarray(springs, np.int64)
    fk = np.zeros(sel.shape[0], np.float64)
    fr = np.zeros(sel.shape[0], np.float64)
    _adj_lib().bso_fd_fp64(*args, sel.shape[0], _p(sel, C.c_int64), float(h), _p(fk, C.c_double), _p(fr, C.c_double))
    return fk, fr
