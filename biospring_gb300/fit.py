"""Optional fitting harness: spring parameters (and, with Coulomb forces, charges) as PyTorch
tensors, gradients from the device adjoint (bs_adjoint). PyTorch is only the optimiser's container
here; the loss and its gradient come from the CUDA kernels through the C ABI.

    net = SpringNetwork(); ...; net.setup(cfg)
    k = torch.tensor(k0, requires_grad=True); r0 = torch.tensor(r00, requires_grad=True)
    loss = SpringFitLoss.apply(k, r0, net, target, 200, 20)
    loss.backward()          # k.grad, r0.grad from the adjoint sweep
    q = torch.tensor(q0, requires_grad=True)
    loss = SpringFitLoss.apply(k, r0, net, target, 200, 20, q)
    loss.backward()          # and q.grad, dL/dq of every particle
"""

from __future__ import annotations

import numpy as np
import torch


class SpringFitLoss(torch.autograd.Function):
    """L(k, r0[, q]) = (1/n) sum_i |x_i(nsteps) - target_i|^2 from the handle's current state."""

    @staticmethod
    def forward(ctx, stiffness, equilibrium, net, target, nsteps: int = 200, checkpoint: int = 20, charges=None):
        k = stiffness.detach().cpu().numpy().astype(np.float32)
        r0 = equilibrium.detach().cpu().numpy().astype(np.float32)
        net.setSpringParameters(k, r0)
        if charges is None:
            loss, gk, gr = net.adjoint(nsteps, target, checkpoint)
            gq = torch.zeros(0)
        else:
            net.setCharges(charges.detach().cpu().numpy().astype(np.float32))
            loss, gk, gr, gq = net.adjoint(nsteps, target, checkpoint, charges=True)
            gq = torch.from_numpy(gq).to(charges.device)
        ctx.has_q = charges is not None
        ctx.save_for_backward(torch.from_numpy(gk).to(stiffness.device), torch.from_numpy(gr).to(equilibrium.device),
                              gq)
        return torch.tensor(loss, dtype=torch.float64)

    @staticmethod
    def backward(ctx, grad_out):
        gk, gr, gq = ctx.saved_tensors
        g = grad_out.to(torch.float32)
        return g * gk, g * gr, None, None, None, None, (g * gq if ctx.has_q else None)
