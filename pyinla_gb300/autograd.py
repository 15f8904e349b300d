"""``torch.autograd.Function`` around the adjoint theta-gradient.

The forward pass evaluates f(theta) and, when a gradient is required, its adjoint
gradient in the same pass over the GPU factors (selected inversion + trace
contractions, see :mod:`pyinla_gb300.model`); backward returns it scaled by the
incoming gradient.  This replaces the 2 dim(theta) + 1 central-difference
evaluations of the reference (src/pyinla/core/pyinla.py:546-580).
"""
from __future__ import annotations

import numpy as np
import torch


class LaplaceObjective(torch.autograd.Function):
    """f = LaplaceObjective.apply(theta, model) with theta a float64 CPU tensor."""

    @staticmethod
    def forward(ctx, theta: torch.Tensor, model):
        th = theta.detach().cpu().numpy().astype(np.float64)
        if theta.requires_grad:
            f, g = model.evaluate(th, gradient=True)
            ctx.save_for_backward(torch.from_numpy(np.asarray(g, dtype=np.float64)))
        else:
            f = model.evaluate(th)
        return theta.new_tensor(f)

    @staticmethod
    def backward(ctx, grad_out):
        (g,) = ctx.saved_tensors
        return grad_out * g.to(grad_out.device), None


def value_and_grad(model, theta) -> tuple[float, np.ndarray]:
    """Plain helper for optimisers (e.g. scipy L-BFGS-B with ``jac=True``, as the
    reference's PyINLA.minimize uses, src/pyinla/core/pyinla.py:455-470)."""
    f, g = model.evaluate(np.asarray(theta, dtype=np.float64), gradient=True)
    return float(f), np.asarray(g)
