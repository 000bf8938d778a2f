"""Optional fitting harness: spring parameters as PyTorch tensors, gradients from the device
adjoint (bs_adjoint). PyTorch is only the optimiser's container here; the loss and its gradient
come from the CUDA kernels through the C ABI.

    net = SpringNetwork(); ...; net.setup(cfg)
    k = torch.tensor(k0, requires_grad=True); r0 = torch.tensor(r00, requires_grad=True)
    loss = SpringFitLoss.apply(k, r0, net, target, 200, 20)
    loss.backward()          # k.grad, r0.grad from the adjoint sweep
"""

from __future__ import annotations

import numpy as np
import torch


class SpringFitLoss(torch.autograd.Function):
    """L(k, r0) = (1/n) sum_i |x_i(nsteps) - target_i|^2 from the handle's current state."""

    @staticmethod
    def forward(ctx, stiffness, equilibrium, net, target, nsteps: int = 200, checkpoint: int = 20):
        k = stiffness.detach().cpu().numpy().astype(np.float32)
        r0 = equilibrium.detach().cpu().numpy().astype(np.float32)
        net.setSpringParameters(k, r0)
        loss, gk, gr = net.adjoint(nsteps, target, checkpoint)
        ctx.save_for_backward(torch.from_numpy(gk).to(stiffness.device), torch.from_numpy(gr).to(equilibrium.device))
        return torch.tensor(loss, dtype=torch.float64)

    @staticmethod
    def backward(ctx, grad_out):
        gk, gr = ctx.saved_tensors
        g = grad_out.to(torch.float32)
        return g * gk, g * gr, None, None, None, None
