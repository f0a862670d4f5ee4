"""Differentiable energies: <psi(theta)|H|psi(theta)> as a torch.autograd.Function.

The forward pass runs the engine's adjoint sweep (`pqc_energy_grad`), which
produces E and dE/dtheta together (the reference computes each gradient entry
from a separately re-run derivative state, measure.py:461-471), so backward
only scales the stored gradient.
"""
import torch

from . import engine


class PQCEnergy(torch.autograd.Function):
    @staticmethod
    def forward(ctx, theta, program, H, psi0):
        th = theta.detach()
        E, g = program.energy_grad(th if th.dim() == 2 else th.reshape(1, -1), H, psi0)
        ctx.save_for_backward(g)
        ctx.squeeze = theta.dim() == 1
        return E[0] if ctx.squeeze else E

    @staticmethod
    def backward(ctx, grad_E):
        (g,) = ctx.saved_tensors
        if ctx.squeeze:
            return grad_E * g[0], None, None, None
        return grad_E[:, None] * g, None, None, None


def energy(pqc, theta, H=None):
    """Differentiable energy of `pqc` at `theta` ([P] or [B, P], a CUDA float64 tensor)."""
    dev = engine.device()
    th = theta if isinstance(theta, torch.Tensor) else torch.as_tensor(theta, dtype=torch.float64)
    if th.device != dev:
        th = th.to(dev)
    return PQCEnergy.apply(th, pqc.program, pqc.H if H is None else H, pqc._psi0())
