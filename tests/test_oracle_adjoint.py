"""The FP64 gradient reference (oracle/adjoint_fp64.cpp) against FP64 central finite differences.

The device adjoint is checked against this reference; here the reference itself is pinned: its
discrete adjoint must agree with differences of its own loss (h = 1e-4), on a network with a
kick, a damped integrator and a few static particles.
"""

from __future__ import annotations

import numpy as np

from biospring_gb300 import workloads as W
from oracle import pyoracle


def _case(n=300, seed=9, steps=120):
    s = W.ca_network(n, seed=seed)
    s.is_static = np.zeros(n, np.uint8)
    s.is_static[::37] = 1
    target = (s.xyz + W.smooth_displacement(s.xyz, seed, 2.0)).astype(np.float32)
    return s, target, steps


def test_fp64_adjoint_matches_finite_differences():
    s, target, steps = _case()
    loss, gk, gr = pyoracle.adjoint_fp64(s, steps, target)
    assert abs(loss - pyoracle.loss_fp64(s, steps, target)) <= 1e-14 * abs(loss)
    sel = np.random.default_rng(1).choice(s.ij.shape[0], 24, replace=False)
    fk, fr = pyoracle.fd_fp64(s, steps, target, sel, 1e-4)
    ek = np.linalg.norm(gk[sel] - fk) / np.linalg.norm(fk)
    er = np.linalg.norm(gr[sel] - fr) / np.linalg.norm(fr)
    print(f"FP64 adjoint vs FD: dL/dk {ek:.2e}, dL/dr0 {er:.2e}")
    assert ek < 1e-6 and er < 1e-6


def test_fp64_adjoint_steric_and_mass():
    """Linear steric overlaps (springs off, particles pushed into contact) and non-unit masses."""
    s, target, steps = _case(n=200, seed=4, steps=80)
    s.config.update(spring_enable=0, steric_cutoff=8.0, timestep=0.05)
    s.radius = np.full(s.n, 2.3, np.float32)  # contact distance 4.6 A > the 3.8 A bond
    s.mass = np.linspace(0.5, 3.0, s.n).astype(np.float32)
    loss, gk, gr = pyoracle.adjoint_fp64(s, steps, target)
    # springs are off: their parameters do not enter the loss
    assert np.all(gk == 0.0) and np.all(gr == 0.0)
    # springs only along the chain (pairs under 4 A): non-bonded neighbours overlap and the
    # steric Hessian carries part of the spring gradients
    ij = W.pairs_within(s.xyz, 4.0)
    r0 = np.linalg.norm(s.xyz[ij[:, 1]].astype(np.float64) - s.xyz[ij[:, 0]], axis=1).astype(np.float32)
    kk = np.full(ij.shape[0], 4.184, np.float32)
    s2 = W.System(s.name, s.xyz, ij, r0, kk, dict(s.config, spring_enable=1), radius=s.radius, mass=s.mass)
    loss2, gk2, gr2 = pyoracle.adjoint_fp64(s2, steps, target)
    sel = np.arange(0, s2.ij.shape[0], max(1, s2.ij.shape[0] // 16))[:16]
    fk, fr = pyoracle.fd_fp64(s2, steps, target, sel, 1e-4)
    er = np.linalg.norm(gr2[sel] - fr) / np.linalg.norm(fr)
    ek = np.linalg.norm(gk2[sel] - fk) / np.linalg.norm(fk)
    print(f"steric + springs, FP64 adjoint vs FD: dL/dk {ek:.2e}, dL/dr0 {er:.2e}")
    assert er < 1e-6 and ek < 1e-6


def _charged_case(dielectric_mode: int, n=300, seed=9, steps=120):
    s, target, steps = _case(n, seed, steps)
    rng = np.random.default_rng(seed + 1)
    s.charge = np.where(rng.random(n) < 0.3, rng.choice([-1.0, 1.0], n), 0.0).astype(np.float32)
    s.config.update(coulomb_enable=1, coulomb_cutoff=12.0, coulomb_dielectric=4.0, dielectric_mode=dielectric_mode)
    return s, target, steps


def test_fp64_adjoint_coulomb_and_charge_gradients():
    """Coulomb forces in the dynamics (both dielectric modes): the adjoint's spring gradients and
    its dL/dq (charged, uncharged and static particles) against central differences."""
    for mode in (0, 1):
        s, target, steps = _charged_case(mode)
        loss, gk, gr, gq = pyoracle.adjoint_fp64(s, steps, target, with_charges=True)
        assert abs(loss - pyoracle.loss_fp64(s, steps, target)) <= 1e-14 * abs(loss)
        sel = np.random.default_rng(2).choice(s.ij.shape[0], 16, replace=False)
        fk, fr = pyoracle.fd_fp64(s, steps, target, sel, 1e-4)
        ek = np.linalg.norm(gk[sel] - fk) / np.linalg.norm(fk)
        charged = np.flatnonzero(s.charge != 0)[:8]
        neutral = np.flatnonzero((s.charge == 0) & (s.is_static == 0))[:8]
        fixed = np.flatnonzero(s.is_static != 0)[:4]
        parts = np.concatenate([charged, neutral, fixed])
        fq = pyoracle.fd_q_fp64(s, steps, target, parts, 1e-4)
        eq = np.linalg.norm(gq[parts] - fq) / np.linalg.norm(fq)
        print(f"mode {mode}: FP64 adjoint vs FD: dL/dk {ek:.2e}, dL/dq {eq:.2e}; |dL/dq| charged "
              f"{np.abs(fq[:8]).mean():.2e}, neutral {np.abs(fq[8:16]).mean():.2e}, static {np.abs(fq[16:]).mean():.2e}")
        assert ek < 1e-5 and eq < 1e-5
        assert np.abs(fq[8:16]).max() > 0.0  # an uncharged particle's charge still matters
