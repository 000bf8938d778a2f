"""The allocation-free nonbonded entry point against the handle's force evaluation and the oracle.

bs_nonbonded_forces_noalloc sums steric, Coulomb and hydrophobic forces over all pairs with its
scratch in a fixed device array; a handle built with spring.enable = 0 computes the same terms
from its cell-list pair lists, and the CPU oracle restates the reference's force loop. Every call
goes through the C ABI, twice in a row. The file is named to be collected last, so the entry
point is also exercised after every other GPU test of the suite.
"""

from __future__ import annotations

import ctypes as C

import numpy as np
import pytest

from biospring_gb300 import capi
from biospring_gb300 import workloads as W
from helpers import gpu_network, rel_l2, rel_scalar

pytestmark = pytest.mark.gpu

# forces: relative L2 over dynamic particles; energies: relative per term (FP32 pair sums on
# both sides, different summation orders)
FORCE_TOL = 1e-5
ENERGY_TOL = 1e-5
NOALLOC_MAX = 16384  # BS_NOALLOC_MAX_PARTICLES of include/biospring_gb300.h
E = {name: k for k, name in enumerate(capi.ENERGY_NAMES)}  # BS_ENERGY_* order


def _lib():
    lib = capi.load()
    fn = lib.bs_nonbonded_forces_noalloc
    fn.restype = C.c_int
    fn.argtypes = [C.POINTER(capi.BsConfig), C.c_int64] + [C.c_void_p] * 9 + [C.c_char_p, C.c_size_t]
    return lib


def _system(n: int, seed: int, cfg: dict) -> W.System:
    rng = np.random.default_rng(seed)
    xyz = W.rsa_fill(n, 55.0, 3.0, seed)
    radius = rng.uniform(1.5, 2.0, n).astype(np.float32)
    epsilon = rng.uniform(0.1, 0.3, n).astype(np.float32)
    charge = np.where(rng.random(n) < 0.3, rng.choice([-1.0, 1.0], n), 0.0).astype(np.float32)
    hydro = np.where(rng.random(n) < 0.2, rng.uniform(0.2, 0.8, n), 0.0).astype(np.float32)
    is_static = (rng.random(n) < 0.1).astype(np.uint8)
    empty = np.zeros((0, 2), np.int32)
    return W.System("noalloc", xyz, empty, np.zeros(0, np.float32), np.zeros(0, np.float32), cfg,
                    radius=radius, epsilon=epsilon, charge=charge, hydrophobicity=hydro, is_static=is_static)


CASES = [
    ("amber-constant", capi.BS_STERIC_LJ_12_6_AMBER, capi.BS_DIELECTRIC_CONSTANT),
    ("linear-distance", capi.BS_STERIC_LINEAR, capi.BS_DIELECTRIC_DISTANCE),
    ("zacharias-constant", capi.BS_STERIC_LJ_8_6_ZACHARIAS, capi.BS_DIELECTRIC_CONSTANT),
    ("lewitt-distance", capi.BS_STERIC_LJ_8_6_LEWITT, capi.BS_DIELECTRIC_DISTANCE),
]


@pytest.mark.parametrize("name,mode,diel", CASES, ids=[c[0] for c in CASES])
def test_noalloc_matches_handle_twice(name, mode, diel):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    lib = _lib()
    cfg = dict(spring_enable=0, steric_enable=1, steric_mode=mode, steric_cutoff=9.0,
               coulomb_enable=1, coulomb_cutoff=14.0, coulomb_dielectric=4.0, dielectric_mode=diel,
               hydrophobicity_enable=1, hydrophobicity_cutoff=8.0, hydrophobicity_scale=1.0,
               impala_enable=0, viscosity_enable=0, list_skin=1.0)
    s = _system(3000, 7 + mode, cfg)
    dyn = s.is_static == 0

    net = gpu_network(s)
    net.computeForces()
    f_ref = net.getForces()
    e_ref = net.energies()

    dev = torch.device("cuda", 0)
    d_xyz = torch.from_numpy(s.xyz.reshape(-1).copy()).to(dev)
    d_rad = torch.from_numpy(s.radius).to(dev)
    d_eps = torch.from_numpy(s.epsilon).to(dev)
    d_q = torch.from_numpy(s.charge).to(dev)
    d_h = torch.from_numpy(s.hydrophobicity).to(dev)
    d_st = torch.from_numpy(s.is_static).to(dev)
    d_f = torch.full((3 * s.n,), float("nan"), dtype=torch.float32, device=dev)
    d_e = torch.full((len(capi.ENERGY_NAMES),), float("nan"), dtype=torch.float64, device=dev)
    bcfg = s.bs_config()
    err = C.create_string_buffer(256)
    results = []
    for _ in range(2):
        torch.cuda.synchronize()
        rc = lib.bs_nonbonded_forces_noalloc(C.byref(bcfg), s.n, d_xyz.data_ptr(), d_rad.data_ptr(),
                                             d_eps.data_ptr(), d_q.data_ptr(), d_h.data_ptr(), d_st.data_ptr(),
                                             d_f.data_ptr(), d_e.data_ptr(), None, err, len(err))
        assert rc == capi.BS_OK, err.value.decode()
        torch.cuda.synchronize()
        results.append((d_f.cpu().numpy().reshape(-1, 3).copy(), d_e.cpu().numpy().copy()))
        d_f.fill_(float("nan"))
        d_e.fill_(float("nan"))

    for f, e in results:
        assert np.all(np.isfinite(f))
        assert np.all(f[~dyn] == 0.0)
        err_f = rel_l2(f, f_ref, dyn)
        print(f"{name}: forces rel L2 {err_f:.3e}")
        assert err_f < FORCE_TOL
        for key in ("steric", "electrostatic", "hydrophobic"):
            assert e_ref[key] != 0.0
            assert rel_scalar(e[E[key]], e_ref[key]) < ENERGY_TOL, (key, e[E[key]], e_ref[key])
        for key in ("kinetic", "spring", "imp"):
            assert e[E[key]] == 0.0
    # the second call starts from the state the first one left: same bits
    assert np.array_equal(results[0][0], results[1][0])
    assert np.array_equal(results[0][1], results[1][1])


def _call_twice(lib, bcfg, n, arrays, torch):
    """Two calls in a row on device copies of `arrays` (None stays NULL); (forces, energies) of each."""
    dev = torch.device("cuda", 0)
    dptr = {}
    keep = []
    for key, a in arrays.items():
        if a is None:
            dptr[key] = None
            continue
        t = torch.from_numpy(np.ascontiguousarray(a).reshape(-1).copy()).to(dev)
        keep.append(t)
        dptr[key] = t.data_ptr()
    d_f = torch.full((3 * n,), float("nan"), dtype=torch.float32, device=dev)
    d_e = torch.full((len(capi.ENERGY_NAMES),), float("nan"), dtype=torch.float64, device=dev)
    err = C.create_string_buffer(256)
    out = []
    for _ in range(2):
        torch.cuda.synchronize()
        rc = lib.bs_nonbonded_forces_noalloc(C.byref(bcfg), n, dptr["xyz"], dptr["radius"], dptr["epsilon"],
                                             dptr["charge"], dptr["hydrophobicity"], dptr["is_static"],
                                             d_f.data_ptr(), d_e.data_ptr(), None, err, len(err))
        assert rc == capi.BS_OK, err.value.decode()
        torch.cuda.synchronize()
        out.append((d_f.cpu().numpy().reshape(-1, 3).copy(), d_e.cpu().numpy().copy()))
        d_f.fill_(float("nan"))
        d_e.fill_(float("nan"))
    return out


# n = 1 (one particle: nothing acts on it), 63 (one partial block of the force kernel) and
# BS_NOALLOC_MAX_PARTICLES (the largest grid: every per-block energy partial of the scratch used);
# "optional-null" passes NULL charges, hydrophobicity and static flags.
ORACLE_CASES = [(1, False), (63, False), (NOALLOC_MAX, False), (2000, True)]


@pytest.mark.parametrize("n,null_optional", ORACLE_CASES,
                         ids=["n1", "n63", f"n{NOALLOC_MAX}", "optional-null"])
def test_noalloc_against_oracle(n, null_optional):
    """The entry point against the CPU oracle (the restatement of the reference's force loop)
    with the same particles and spring.enable = 0, twice in a row."""
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from oracle import pyoracle as po
    lib = _lib()
    cfg = dict(spring_enable=0, steric_enable=1, steric_mode=capi.BS_STERIC_LJ_12_6_AMBER, steric_cutoff=9.0,
               coulomb_enable=1, coulomb_cutoff=14.0, coulomb_dielectric=4.0,
               dielectric_mode=capi.BS_DIELECTRIC_CONSTANT, hydrophobicity_enable=1, hydrophobicity_cutoff=8.0)
    box = max(12.0, (n / 0.0244) ** (1.0 / 3.0) + 4.0)
    rng = np.random.default_rng(n)
    xyz = W.rsa_fill(n, box, 3.0, 100 + n)
    s = W.System("noalloc-oracle", xyz, np.zeros((0, 2), np.int32), np.zeros(0, np.float32),
                 np.zeros(0, np.float32), cfg, radius=rng.uniform(1.5, 2.0, n).astype(np.float32),
                 epsilon=rng.uniform(0.1, 0.3, n).astype(np.float32))
    if not null_optional:
        s.charge = np.where(rng.random(n) < 0.3, rng.choice([-1.0, 1.0], n), 0.0).astype(np.float32)
        s.hydrophobicity = np.where(rng.random(n) < 0.2, rng.uniform(0.2, 0.8, n), 0.0).astype(np.float32)
        s.is_static = (rng.random(n) < 0.1).astype(np.uint8)
    arrays = dict(xyz=s.xyz, radius=s.radius, epsilon=s.epsilon, charge=s.charge,
                  hydrophobicity=s.hydrophobicity, is_static=s.is_static)
    results = _call_twice(lib, po.oracle_config(s), n, arrays, torch)
    orc = po.Oracle(s)
    orc.compute_forces()
    f_ref, e_ref = orc.forces(), orc.energies()
    _, e64 = orc.eval_fp64()
    orc.close()
    dyn = np.ones(n, bool) if s.is_static is None else s.is_static == 0
    for f, e in results:
        assert np.all(np.isfinite(f))
        if n == 1:
            assert np.all(f == 0.0) and np.all(e == 0.0)
            continue
        err_f = rel_l2(f, f_ref, dyn)
        print(f"n={n} null_optional={null_optional}: forces vs oracle rel L2 {err_f:.3e}")
        assert err_f < FORCE_TOL
        assert np.all(f[~dyn] == 0.0)
        for key in ("steric", "electrostatic", "hydrophobic"):
            k = E[key]
            if e_ref[k] == 0.0:
                assert e[k] == 0.0, key
            else:
                # the oracle sums pair energies serially in FP32 (as the reference does): where
                # that sum is further from FP64 than the bar, the bar widens by its own distance
                tol = max(ENERGY_TOL * abs(e_ref[k]), abs(e_ref[k] - e64[k]) + 1e-6 * abs(e_ref[k]))
                assert abs(e[k] - e_ref[k]) <= tol, (key, e[k], e_ref[k], e64[k])
        for key in ("kinetic", "spring", "imp"):
            assert e[E[key]] == 0.0
    assert np.array_equal(results[0][0], results[1][0])
    assert np.array_equal(results[0][1], results[1][1])


def test_noalloc_rejects_oversize():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    lib = _lib()
    nmax = NOALLOC_MAX
    bcfg = capi.default_config()
    err = C.create_string_buffer(256)
    dev = torch.device("cuda", 0)
    d = torch.zeros(3 * (nmax + 1), dtype=torch.float32, device=dev)
    e = torch.zeros(len(capi.ENERGY_NAMES), dtype=torch.float64, device=dev)
    rc = lib.bs_nonbonded_forces_noalloc(C.byref(bcfg), nmax + 1, d.data_ptr(), d.data_ptr(), d.data_ptr(),
                                         None, None, None, d.data_ptr(), e.data_ptr(), None, err, len(err))
    assert rc == capi.BS_E_ARG
    assert "static scratch" in err.value.decode()
