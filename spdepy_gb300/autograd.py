"""The log-likelihood as a differentiable torch function.

``loglike(model, par)`` returns the reference's normalised objective
f(par) = -like / (m r) (reference ``spdes/advection_diffusion2D.py:187-223``)
as a 0-d tensor; its backward pass applies the gradient the GPU computes in the
same evaluation (exact traces from the selected inverse of Q and
Q + tau S^T S, contracted with dQ/dtheta by the adjoint kernels, so no dQ
matrix is ever formed).  Forward and backward share one evaluation: the
gradient is computed in forward whenever ``par`` requires grad and is kept for
backward.
"""
from __future__ import annotations

import numpy as np
import torch


class LogLike(torch.autograd.Function):
    @staticmethod
    def forward(ctx, par, model, grad_mode):
        p = par.detach().to("cpu", torch.float64).numpy()
        if ctx.needs_input_grad[0]:
            f, jac = model.logLike(p, grad=True, grad_mode=grad_mode)
            ctx.save_for_backward(torch.as_tensor(np.asarray(jac), dtype=par.dtype, device=par.device))
        else:
            f = model.logLike(p, grad=False)
        return torch.tensor(float(f), dtype=par.dtype, device=par.device)

    @staticmethod
    def backward(ctx, g):
        (jac,) = ctx.saved_tensors
        return g * jac, None, None


def loglike(model, par: torch.Tensor, grad_mode: str = "exact") -> torch.Tensor:
    """Differentiable objective of ``model`` (an SPDE model object after
    ``initFit``) at the parameter vector ``par`` (reference parameter order)."""
    return LogLike.apply(par, model, grad_mode)
