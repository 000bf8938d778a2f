"""Python host mirror of the reference engine's interface, over the C ABI.

Method names follow ``biospring::spn::SpringNetwork`` (src/spn/SpringNetwork.h): particles
and springs are added first, ``setup`` takes the .msp parameters, then ``computeStep`` /
``computeForces`` run on the GPU and the getters read the state back. Errors raise
:class:`BsError` with the library's code and message, where the reference would throw or die.
"""

from __future__ import annotations

import ctypes as C

import numpy as np

from . import capi
from .capi import BsConfig, BsError, ptr


def _f32(a, shape=None):
    if a is None:
        return None
    out = np.ascontiguousarray(a, dtype=np.float32)
    if shape is not None:
        out = out.reshape(shape)
    return out


class SpringNetwork:
    """One simulation handle on the current CUDA device."""

    def __init__(self):
        self._lib = capi.load()
        h = C.c_void_p()
        self._check(self._lib.bs_create(C.byref(h)), None)
        self._h = h
        self.n = 0
        self.config: BsConfig | None = None

    # -- plumbing ---------------------------------------------------------------------
    def _check(self, rc: int, h=None):
        if rc != capi.BS_OK:
            buf = C.create_string_buffer(512)
            self._lib.bs_last_error(h if h is not None else getattr(self, "_h", None), buf, 512)
            raise BsError(rc, buf.value.decode(errors="replace"))

    def close(self):
        if getattr(self, "_h", None):
            self._lib.bs_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    # -- topology (SpringNetwork::addParticle / addSpring) -------------------------------
    def addParticles(self, xyz, vel=None, mass=None, charge=None, radius=None, epsilon=None,
                     hydrophobicity=None, sasa=None, transfer=None, is_static=None):
        xyz = _f32(xyz, (-1, 3))
        n = xyz.shape[0]
        arrs = [_f32(vel, (-1, 3)), _f32(mass), _f32(charge), _f32(radius), _f32(epsilon),
                _f32(hydrophobicity), _f32(sasa), _f32(transfer)]
        st = None if is_static is None else np.ascontiguousarray(is_static, dtype=np.uint8)
        self._keep = (xyz, arrs, st)
        self._check(self._lib.bs_upload_particles(
            self._h, n, ptr(xyz, C.c_float), *[ptr(a, C.c_float) for a in arrs], ptr(st, C.c_uint8)), self._h)
        self.n += n

    def addSprings(self, ij, equilibrium, stiffness):
        ij = np.ascontiguousarray(ij, dtype=np.int32).reshape(-1, 2)
        r0 = _f32(equilibrium)
        k = _f32(stiffness)
        self._check(self._lib.bs_upload_springs(self._h, ij.shape[0], ptr(ij, C.c_int32), ptr(r0, C.c_float),
                                                ptr(k, C.c_float)), self._h)

    # -- frame recorder -------------------------------------------------------------------------
    def setFrames(self, every: int, capacity: int = 64):
        """Records positions and energies every `every` steps into a host ring of `capacity` frames
        that the device writes while it steps (every = 0 stops)."""
        self._check(self._lib.bs_set_frames(self._h, int(every), int(capacity)), self._h)

    def readFrames(self, max_frames: int = 1024):
        """Complete frames, oldest first, without waiting: (steps (k,), positions (k, n, 3),
        energies (k, 6), dropped)."""
        steps = np.zeros(max_frames, dtype=np.int64)
        xyz = np.zeros((max_frames, self.n, 3), dtype=np.float32)
        en = np.zeros((max_frames, 6), dtype=np.float64)
        cnt = C.c_int32()
        lost = C.c_int64()
        self._check(self._lib.bs_read_frames(self._h, int(max_frames), ptr(steps, C.c_int64), ptr(xyz, C.c_float),
                                             ptr(en, C.c_double), C.byref(cnt), C.byref(lost)), self._h)
        k = cnt.value
        return steps[:k], xyz[:k], en[:k], lost.value

    def loadNetCDF(self, path: str) -> tuple:
        """Reads a BioSpring topology (.nc, NetCDF classic) into the network, as NetCDFReader
        does: particles and springs. Returns (particles, springs)."""
        n = C.c_int64()
        m = C.c_int64()
        self._check(self._lib.bs_load_nc(self._h, str(path).encode(), C.byref(n), C.byref(m)), self._h)
        self.n += n.value
        return n.value, m.value

    # -- field grids (potentialgrid.*, densitygrid.*) ------------------------------------------
    def setFieldGrid(self, which: int, scalar, origin, spacing):
        """Map `which` (capi.BS_GRID_POTENTIAL or BS_GRID_DENSITY) from a (n0, n1, n2) array of
        scalar values on a grid of cell size `spacing` from `origin`; call before :meth:`setup`."""
        sc = np.ascontiguousarray(scalar, dtype=np.float32)
        shape = np.asarray(sc.shape, dtype=np.int32)
        o = np.ascontiguousarray(origin, dtype=np.float64)
        h = np.ascontiguousarray(spacing, dtype=np.float64)
        self._check(self._lib.bs_set_field_grid(self._h, int(which), ptr(shape, C.c_int32), ptr(o, C.c_double),
                                                ptr(h, C.c_double), ptr(sc, C.c_float)), self._h)

    def fieldGrid(self, which: int) -> np.ndarray:
        """The map after set-up, (n0, n1, n2, 4): scalar and force vector of every cell."""
        shape = np.zeros(3, dtype=np.int32)
        self._check(self._lib.bs_get_field_grid(self._h, int(which), ptr(shape, C.c_int32), None), self._h)
        out = np.zeros(tuple(int(v) for v in shape) + (4,), dtype=np.float32)
        self._check(self._lib.bs_get_field_grid(self._h, int(which), ptr(shape, C.c_int32), ptr(out, C.c_float)),
                    self._h)
        return out

    def setBurying(self, burying):
        """Per-particle burying, the weight of the density-map force (default 1)."""
        b = _f32(burying)
        self._check(self._lib.bs_set_burying(self._h, ptr(b, C.c_float)), self._h)

    def setMembrane(self, upper_offset: float = 0.0, lower_offset: float = 0.0, upper_curvature: float = 0.0,
                    lower_curvature: float = 0.0):
        """IMPALA double membrane (ForceField::setImpDoubleMembrane*): offsets in A, tube
        curvatures in 1/A; all zero is the flat membrane."""
        self._check(self._lib.bs_set_membrane(self._h, float(upper_offset), float(lower_offset),
                                              float(upper_curvature), float(lower_curvature)), self._h)

    def setCharges(self, charge):
        """Replaces every particle's charge (caller order); Coulomb list membership follows at the
        next step."""
        q = _f32(charge)
        if q.shape[0] != self.n:
            raise ValueError(f"setCharges: {q.shape[0]} charges for {self.n} particles")
        self._check(self._lib.bs_set_charges(self._h, ptr(q, C.c_float)), self._h)

    def setRigidBodies(self, bodies):
        offsets = np.zeros(len(bodies) + 1, dtype=np.int32)
        for b, ids in enumerate(bodies):
            offsets[b + 1] = offsets[b] + len(ids)
        ids = np.ascontiguousarray(np.concatenate([np.asarray(b, dtype=np.int32) for b in bodies])
                                   if bodies else np.zeros(0, np.int32), dtype=np.int32)
        self._check(self._lib.bs_set_rigid_bodies(self._h, len(bodies), ptr(offsets, C.c_int32),
                                                  ptr(ids, C.c_int32)), self._h)

    # -- setup and run --------------------------------------------------------------------
    def setup(self, config):
        if isinstance(config, dict):
            cfg = capi.default_config()
            for k, v in config.items():
                setattr(cfg, k, v)
            config = cfg
        self.config = config
        self._check(self._lib.bs_setup(self._h, C.byref(config)), self._h)

    # -- gradients ---------------------------------------------------------------------------
    def springCount(self) -> int:
        c = C.c_int64()
        self._check(self._lib.bs_get_spring_count(self._h, C.byref(c)), self._h)
        return c.value

    def setSpringParameters(self, stiffness=None, equilibrium=None):
        k = _f32(stiffness)
        r0 = _f32(equilibrium)
        self._check(self._lib.bs_set_spring_parameters(self._h, ptr(k, C.c_float), ptr(r0, C.c_float)), self._h)

    def adjoint(self, nsteps: int, target, checkpoint: int = 20, charges: bool = False):
        """Loss (1/n) sum |x(nsteps) - target|^2 and its gradient with respect to every spring's
        stiffness and rest length, by the discrete adjoint (the state is left unchanged). With
        charges, dL/dq of every particle is returned fourth."""
        tg = _f32(target, (-1, 3))
        ns = self.springCount()
        gk = np.zeros(max(ns, 1), dtype=np.float32)
        gr = np.zeros(max(ns, 1), dtype=np.float32)
        gq = np.zeros(self.n, dtype=np.float32) if charges else None
        loss = C.c_double()
        self._check(self._lib.bs_adjoint(self._h, int(nsteps), int(checkpoint), ptr(tg, C.c_float), C.byref(loss),
                                         ptr(gk, C.c_float), ptr(gr, C.c_float), ptr(gq, C.c_float)), self._h)
        if charges:
            return loss.value, gk[:ns], gr[:ns], gq
        return loss.value, gk[:ns], gr[:ns]

    # -- batched ensembles -----------------------------------------------------------------
    def setSystems(self, offsets):
        """Partitions the particles into independent systems: system b owns
        [offsets[b], offsets[b + 1]). Call before :meth:`setup`."""
        off = np.ascontiguousarray(offsets, dtype=np.int64)
        self._check(self._lib.bs_set_systems(self._h, int(off.shape[0] - 1), ptr(off, C.c_int64)), self._h)
        self.nsys = int(off.shape[0] - 1)

    def getSystemEnergies(self) -> np.ndarray:
        out = np.zeros((self.nsys, 6), dtype=np.float64)
        self._check(self._lib.bs_get_system_energies(self._h, ptr(out, C.c_double)), self._h)
        return out

    def setBatchShape(self, block: int, lanes: int, cluster: int):
        self._check(self._lib.bs_set_batch_shape(self._h, int(block), int(lanes), int(cluster)), self._h)

    def batchShape(self) -> tuple:
        out = np.zeros(3, dtype=np.int32)
        self._check(self._lib.bs_get_batch_shape(self._h, ptr(out, C.c_int32)), self._h)
        return tuple(int(v) for v in out)

    def batchAutotune(self) -> tuple:
        out = np.zeros(3, dtype=np.int32)
        self._check(self._lib.bs_batch_autotune(self._h, ptr(out, C.c_int32)), self._h)
        return tuple(int(v) for v in out)

    def computeStep(self, nsteps: int = 1):
        self._check(self._lib.bs_step(self._h, int(nsteps)), self._h)

    def computeStepAsync(self, nsteps: int = 1):
        """Enqueues steps without waiting; :meth:`synchronize` completes them."""
        self._check(self._lib.bs_step_async(self._h, int(nsteps)), self._h)

    def synchronize(self):
        self._check(self._lib.bs_synchronize(self._h), self._h)

    def stepCount(self) -> int:
        c = C.c_int64()
        self._check(self._lib.bs_get_step_count(self._h, C.byref(c)), self._h)
        return c.value

    def stream(self) -> int:
        """The cudaStream_t of the handle, as an integer."""
        p = C.c_void_p()
        self._check(self._lib.bs_get_stream(self._h, C.byref(p)), self._h)
        return p.value or 0

    def launchPhase(self, phase: int):
        self._check(self._lib.bs_launch_phase(self._h, int(phase)), self._h)

    def computeForces(self):
        self._check(self._lib.bs_compute_forces(self._h), self._h)

    # -- state ------------------------------------------------------------------------------
    def _get3(self, fn):
        out = np.empty((self.n, 3), dtype=np.float32)
        self._check(fn(self._h, ptr(out, C.c_float)), self._h)
        return out

    def getPositions(self):
        return self._get3(self._lib.bs_get_positions)

    def getVelocities(self):
        return self._get3(self._lib.bs_get_velocities)

    def getForces(self):
        return self._get3(self._lib.bs_get_forces)

    def setPositions(self, xyz):
        xyz = _f32(xyz, (-1, 3))
        self._check(self._lib.bs_set_positions(self._h, ptr(xyz, C.c_float)), self._h)

    def setVelocities(self, vel):
        vel = _f32(vel, (-1, 3))
        self._check(self._lib.bs_set_velocities(self._h, ptr(vel, C.c_float)), self._h)

    def setForce(self, i: int, f):
        f = _f32(f)
        self._check(self._lib.bs_set_force(self._h, int(i), ptr(f, C.c_float)), self._h)

    def setExternalForces(self, f, wait: bool = True):
        """Every particle's external force for the next step. wait=False enqueues the upload
        without waiting: f must then be page-locked and stay unchanged until the next
        synchronising call (computeStep, a getter)."""
        f = _f32(f, (-1, 3))
        fn = self._lib.bs_set_external_forces if wait else self._lib.bs_set_external_forces_async
        self._check(fn(self._h, ptr(f, C.c_float)), self._h)

    def energies(self) -> dict:
        out = np.zeros(6, dtype=np.float64)
        self._check(self._lib.bs_get_energies(self._h, ptr(out, C.c_double)), self._h)
        return dict(zip(capi.ENERGY_NAMES, out.tolist()))

    def getKineticEnergy(self):
        return self.energies()["kinetic"]

    def getSpringEnergy(self):
        return self.energies()["spring"]

    def getStericEnergy(self):
        return self.energies()["steric"]

    def getElectrostaticEnergy(self):
        return self.energies()["electrostatic"]

    def getIMPEnergy(self):
        return self.energies()["imp"]

    def getHydrophobicEnergy(self):
        return self.energies()["hydrophobic"]

    # -- diagnostics ------------------------------------------------------------------------
    def getPairs(self, term: int) -> np.ndarray:
        n = C.c_int64()
        self._check(self._lib.bs_get_pairs(self._h, term, None, 0, C.byref(n)), self._h)
        out = np.zeros((max(n.value, 1), 2), dtype=np.int64)
        self._check(self._lib.bs_get_pairs(self._h, term, ptr(out, C.c_int64), n.value, C.byref(n)), self._h)
        return out[: n.value]

    def getCells(self, term: int) -> np.ndarray:
        out = np.zeros(self.n, dtype=np.int64)
        self._check(self._lib.bs_get_cells(self._h, term, ptr(out, C.c_int64)), self._h)
        return out

    def getProbe(self) -> np.ndarray:
        """Probe position and velocity, float32[6] (SpringNetwork::getProbeParticle)."""
        out = np.zeros(6, dtype=np.float32)
        self._check(self._lib.bs_get_probe(self._h, ptr(out, C.c_float)), self._h)
        return out

    def launchCount(self) -> int:
        c = C.c_int64()
        self._check(self._lib.bs_get_launch_count(self._h, C.byref(c)), self._h)
        return c.value
