"""The device adjoint (bs_adjoint) against the FP64 gradient reference and FP64 finite differences.

Workload: a Calpha network built as the plain CPU/GPU configuration, a target equal to the start
positions plus a seeded smooth displacement field of 2 A, the loss after 200 damped steps with
checkpoints every 20 steps; gradients with respect to every spring's stiffness and rest length,
and, with Coulomb pairs in the dynamics, every particle's charge.

At dt = 0.01 fs a step moves a particle by 1e-7 to 1e-5 A, less than half an ulp of a coordinate
near 50 A: the reference's FP32 update x += v dt drops or rounds most of these increments, so an
FP32 trajectory (and any gradient taken along it) differs from the FP64 one by about 1e-2
relative. The gradient checks therefore run with cuda.precisepositions (float-float positions),
which brings the trajectory to FP64 accuracy; the parity-mode gradient is checked against the
same equations evaluated along its own trajectory's loss, and its distance to FP64 is reported.
"""

from __future__ import annotations

import numpy as np
import pytest

from biospring_gb300 import BsError, SpringNetwork
from biospring_gb300 import workloads as W
from helpers import gpu_network
from oracle import pyoracle

pytestmark = pytest.mark.gpu

GRAD_TOL = 1e-4  # relative L2, FP32 adjoint vs FP64


def rel(a, b):
    return float(np.linalg.norm(np.asarray(a, np.float64) - b) / np.linalg.norm(b))


@pytest.fixture(scope="module")
def fit10k():
    s, target, nsteps = W.adjoint_fit(10_000, seed=4)
    s.config["precise_positions"] = 1
    return s, target, nsteps


def test_adjoint_matches_fp64_reference_and_fd(fit10k):
    s, target, nsteps = fit10k
    net = gpu_network(s)
    loss, gk, gr = net.adjoint(nsteps, target, checkpoint=20)
    ref_loss, rk, rr = pyoracle.adjoint_fp64(s, nsteps, target)
    ek, er = rel(gk, rk), rel(gr, rr)
    print(f"10k / 200 steps: loss {loss:.9f} (FP64 {ref_loss:.9f}); dL/dk vs FP64 adjoint {ek:.2e}, "
          f"dL/dr0 {er:.2e}")
    assert abs(loss - ref_loss) <= 1e-6 * abs(ref_loss)
    assert ek < GRAD_TOL and er < GRAD_TOL
    sel = np.random.default_rng(64).choice(s.ij.shape[0], 64, replace=False)
    fk, fr = pyoracle.fd_fp64(s, nsteps, target, sel, 1e-4)
    fek, fer = rel(gk[sel], fk), rel(gr[sel], fr)
    print(f"64 springs vs FP64 central differences (h=1e-4): dL/dk {fek:.2e} (FP64 adjoint "
          f"{rel(rk[sel], fk):.2e}), dL/dr0 {fer:.2e} (FP64 adjoint {rel(rr[sel], fr):.2e})")
    assert fek < GRAD_TOL and fer < GRAD_TOL
    net.close()


def test_adjoint_leaves_state_and_matches_forward(fit10k):
    s, target, nsteps = fit10k
    # reference FP32 position update, so that setPositions below loses nothing
    cfg = dict(s.config, rebuild_every=20, precise_positions=0)
    s20 = W.System(s.name, s.xyz, s.ij, s.r0, s.k, cfg)
    a = gpu_network(s20)
    a.computeStep(5)
    x0 = a.getPositions()
    e0 = a.energies()
    loss, gk, gr = a.adjoint(nsteps, target, checkpoint=20)
    assert a.getPositions().tobytes() == x0.tobytes()
    assert a.energies() == e0
    assert a.stepCount() == 5
    # the adjoint's forward is the plain path with a rebuild every checkpoint
    a.computeStep(nsteps)
    xf = a.getPositions().astype(np.float64)
    fwd = float(((xf - target) ** 2).sum() / s.n)
    assert abs(fwd - loss) <= 1e-6 * abs(loss)
    b = gpu_network(s20)
    b.computeStep(5)
    b.setPositions(b.getPositions())  # the next step rebuilds, as after the adjoint
    b.computeStep(nsteps)
    assert b.getPositions().tobytes() == a.getPositions().tobytes()
    a.close()
    b.close()


def test_adjoint_checkpoint_interval_and_repeat():
    s, target, nsteps = W.adjoint_fit(2_000, seed=8, nsteps=60)
    net = gpu_network(s)
    runs = [net.adjoint(nsteps, target, checkpoint=c) for c in (20, 7, 60, 20)]
    for loss, gk, gr in runs[1:]:
        assert abs(loss - runs[0][0]) <= 1e-6 * abs(runs[0][0])
        assert rel(gk, runs[0][1]) < 1e-5 and rel(gr, runs[0][2]) < 1e-5
    # a repeated call (replayed graph) is bitwise identical
    assert runs[3][1].tobytes() == runs[0][1].tobytes() and runs[3][2].tobytes() == runs[0][2].tobytes()
    net.close()


def test_adjoint_steric_and_static():
    """Springs along the chain only, overlapping neighbours under the linear steric term, some
    static particles and non-unit masses: device gradients against the FP64 reference."""
    base = W.ca_network(1500, seed=21)
    ij = W.pairs_within(base.xyz, 4.0)
    r0 = np.linalg.norm(base.xyz[ij[:, 1]].astype(np.float64) - base.xyz[ij[:, 0]], axis=1).astype(np.float32)
    st = np.zeros(base.n, np.uint8)
    st[::41] = 1
    cfg = dict(base.config, timestep=0.05, steric_cutoff=8.0, precise_positions=1)
    s = W.System("chain_steric", base.xyz, ij, r0, np.full(ij.shape[0], 4.184, np.float32), cfg,
                 radius=np.full(base.n, 2.3, np.float32), mass=np.linspace(0.5, 3.0, base.n).astype(np.float32),
                 is_static=st)
    target = (s.xyz + W.smooth_displacement(s.xyz, 3, 2.0)).astype(np.float32)
    net = gpu_network(s)
    loss, gk, gr = net.adjoint(80, target, checkpoint=20)
    ref_loss, rk, rr = pyoracle.adjoint_fp64(s, 80, target)
    print(f"steric chain: dL/dk {rel(gk, rk):.2e}, dL/dr0 {rel(gr, rr):.2e}")
    assert abs(loss - ref_loss) <= 1e-6 * abs(ref_loss)
    assert rel(gk, rk) < GRAD_TOL and rel(gr, rr) < GRAD_TOL
    net.close()


def test_adjoint_parity_mode_distance_to_fp64():
    """With the reference's FP32 position update the gradient follows the FP32 trajectory: it is
    reported against FP64 and must stay within the trajectory's own error (a few 1e-2)."""
    s, target, nsteps = W.adjoint_fit(2_000, seed=4)
    net = gpu_network(s)
    loss, gk, gr = net.adjoint(nsteps, target, checkpoint=20)
    ref_loss, rk, rr = pyoracle.adjoint_fp64(s, nsteps, target)
    print(f"parity mode (FP32 positions): loss rel {abs(loss - ref_loss) / ref_loss:.2e}, "
          f"dL/dk {rel(gk, rk):.2e}, dL/dr0 {rel(gr, rr):.2e} vs FP64")
    assert rel(gk, rk) < 0.1 and rel(gr, rr) < 0.1
    s.config["precise_positions"] = 1
    net2 = gpu_network(s)
    _, gk2, gr2 = net2.adjoint(nsteps, target, checkpoint=20)
    print(f"precise positions: dL/dk {rel(gk2, rk):.2e}, dL/dr0 {rel(gr2, rr):.2e} vs FP64")
    assert rel(gk2, rk) < GRAD_TOL and rel(gr2, rr) < GRAD_TOL
    net.close()
    net2.close()


@pytest.mark.parametrize("mode", [0, 1], ids=["constant", "distance"])
def test_adjoint_coulomb_and_charge_gradients(mode):
    """Coulomb pairs in the dynamics (30% of the particles charged, eps = 4 or 4r, some static
    particles): spring and charge gradients against the FP64 adjoint, and dL/dq of charged,
    uncharged and static particles against FP64 central differences."""
    s, target, nsteps = W.adjoint_fit(2_000, seed=6, nsteps=100)
    rng = np.random.default_rng(8)
    s.charge = np.where(rng.random(s.n) < 0.3, rng.choice([-1.0, 1.0], s.n), 0.0).astype(np.float32)
    s.is_static = np.zeros(s.n, np.uint8)
    s.is_static[::53] = 1
    s.config.update(coulomb_enable=1, coulomb_cutoff=12.0, coulomb_dielectric=4.0, dielectric_mode=mode,
                    precise_positions=1)
    net = gpu_network(s)
    loss, gk, gr, gq = net.adjoint(nsteps, target, checkpoint=20, charges=True)
    ref_loss, rk, rr, rq = pyoracle.adjoint_fp64(s, nsteps, target, with_charges=True)
    print(f"Coulomb mode {mode}: loss rel {abs(loss - ref_loss) / ref_loss:.2e}; vs FP64 adjoint: "
          f"dL/dk {rel(gk, rk):.2e}, dL/dr0 {rel(gr, rr):.2e}, dL/dq {rel(gq, rq):.2e}")
    assert abs(loss - ref_loss) <= 1e-6 * abs(ref_loss)
    assert rel(gk, rk) < GRAD_TOL and rel(gr, rr) < GRAD_TOL and rel(gq, rq) < GRAD_TOL
    parts = np.concatenate([np.flatnonzero(s.charge != 0)[:8],
                            np.flatnonzero((s.charge == 0) & (s.is_static == 0))[:8],
                            np.flatnonzero(s.is_static != 0)[:4]])
    fq = pyoracle.fd_q_fp64(s, nsteps, target, parts, 1e-4)
    print(f"20 charges vs FP64 central differences: {rel(gq[parts], fq):.2e} (FP64 adjoint {rel(rq[parts], fq):.2e})")
    assert rel(gq[parts], fq) < GRAD_TOL
    # new charges (a charge fit's update; some particles change between charged and neutral)
    q2 = (s.charge + 0.1 * rng.standard_normal(s.n) * (rng.random(s.n) < 0.5)).astype(np.float32)
    net.setCharges(q2)
    loss2, gk2, gr2, gq2 = net.adjoint(nsteps, target, checkpoint=20, charges=True)
    s.charge = q2
    ref2 = pyoracle.adjoint_fp64(s, nsteps, target, with_charges=True)
    print(f"after setCharges: loss rel {abs(loss2 - ref2[0]) / ref2[0]:.2e}; dL/dk {rel(gk2, ref2[1]):.2e}, "
          f"dL/dq {rel(gq2, ref2[3]):.2e}")
    assert abs(loss2 - ref2[0]) <= 1e-6 * abs(ref2[0])
    assert rel(gk2, ref2[1]) < GRAD_TOL and rel(gr2, ref2[2]) < GRAD_TOL and rel(gq2, ref2[3]) < GRAD_TOL
    # the state is untouched and the forward path still steps
    x0 = net.getPositions()
    net.adjoint(nsteps, target, checkpoint=20)
    assert net.getPositions().tobytes() == x0.tobytes()
    net.computeStep(5)
    net.close()


def test_adjoint_rejections():
    s, target, nsteps = W.adjoint_fit(500, seed=2, nsteps=20)
    lj = dict(s.config, steric_mode=1)
    net = gpu_network(W.System(s.name, s.xyz, s.ij, s.r0, s.k, lj,
                               radius=np.full(s.n, 1.8, np.float32), epsilon=np.full(s.n, 0.5, np.float32)))
    with pytest.raises(BsError, match="linear steric"):
        net.adjoint(nsteps, target)
    net.close()
    thin = dict(s.config, list_skin=0.001, timestep=1.0)
    net = gpu_network(W.System(s.name, s.xyz, s.ij, s.r0, s.k * 100.0, thin))
    x0 = net.getPositions()
    with pytest.raises(BsError, match="list skin"):
        net.adjoint(nsteps, target, checkpoint=20)
    assert net.getPositions().tobytes() == x0.tobytes()
    net.computeStep(1)  # the handle is still usable
    net.close()


def test_fit_harness_descends():
    torch = pytest.importorskip("torch")
    from biospring_gb300.fit import SpringFitLoss
    s, target, nsteps = W.adjoint_fit(1_000, seed=5, nsteps=40)
    s.config.update(timestep=0.5)  # long enough steps for the rest lengths to matter
    net = gpu_network(s)
    r0 = torch.tensor(s.r0, requires_grad=True)
    k = torch.tensor(s.k, requires_grad=True)
    losses = []
    opt = torch.optim.SGD([r0], lr=3e4)
    for _ in range(4):
        opt.zero_grad()
        loss = SpringFitLoss.apply(k, r0, net, target, nsteps, 20)
        loss.backward()
        losses.append(float(loss.detach()))
        opt.step()
    print("fit losses", losses)
    assert all(b < a for a, b in zip(losses, losses[1:]))
    assert k.grad is not None and r0.grad is not None
    net.close()


def test_fit_harness_charges_descend():
    """Charges as the fitted tensor: the target is the end state of the same network with other
    charges, and plain gradient descent on q lowers the loss at every step."""
    torch = pytest.importorskip("torch")
    from biospring_gb300.fit import SpringFitLoss
    s, _, nsteps = W.adjoint_fit(1_000, seed=5, nsteps=40)
    rng = np.random.default_rng(12)
    q_true = np.where(rng.random(s.n) < 0.4, rng.choice([-1.0, 1.0], s.n), 0.0).astype(np.float32)
    s.charge = q_true
    s.config.update(timestep=0.5, coulomb_enable=1, coulomb_cutoff=12.0, coulomb_dielectric=1.0, dielectric_mode=0)
    net = gpu_network(s)
    x0 = net.getPositions()
    net.setVelocities(np.zeros_like(x0))
    net.computeStep(nsteps)
    target = net.getPositions()
    net.setPositions(x0)
    net.setVelocities(np.zeros_like(x0))
    k = torch.tensor(s.k)
    r0 = torch.tensor(s.r0)
    q = torch.tensor(q_true * 0.5, requires_grad=True)
    losses = []
    for _ in range(4):
        loss = SpringFitLoss.apply(k, r0, net, target, nsteps, 20, q)
        loss.backward()
        losses.append(float(loss.detach()))
        with torch.no_grad():  # a fixed-length step along the negative gradient
            q -= 0.5 * q.grad / q.grad.norm()
        q.grad = None
    print("charge fit losses", losses)
    assert all(b < a for a, b in zip(losses, losses[1:]))
    net.close()
