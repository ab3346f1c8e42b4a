"""Learned space-time preconditioner for conjugate gradients on grids too large
to factor.

``LearnedPreconditioner`` holds the parameters of the network that maps each
node's normalised row of A = Q (+ tau S^T S) to the 27 weights of the stencil G,
with M^-1 = G^T G (kernels in ``csrc/pcg.cu``).  It starts as Jacobi (zero last
layer) and is trained on systems the method generates itself: parameters drawn
from a prior, assembled on the GPU, observation sets drawn at random, with
probe blocks z standing in for the residuals PCG feeds the preconditioner; the
loss ||z - G A G^T z||^2 / (n k) and its gradient come from the library's own
forward and backward kernels and the update from its Adam kernel.
"""
from __future__ import annotations

import numpy as np

from . import _native as nat

NPARAMS = 3323
_SIZES = [(32, 42), (32,), (32, 32), (32,), (27, 32), (27,)]


def _torch():
    import torch
    return torch


def init_params(seed=0):
    """Glorot-scaled hidden layers, zero last layer (the Jacobi preconditioner)."""
    rng = np.random.default_rng(seed)
    parts = []
    for shape in _SIZES:
        if len(shape) == 2 and shape[0] != 27:
            parts.append(rng.normal(0.0, np.sqrt(1.0 / shape[1]), shape).ravel())
        else:
            parts.append(np.zeros(int(np.prod(shape))))
    p = np.concatenate(parts).astype(np.float32)
    assert p.size == NPARAMS == nat.lib().spde_precond_nparams()
    return p


class LearnedPreconditioner:
    def __init__(self, params=None, seed=0):
        torch = _torch()
        p = init_params(seed) if params is None else np.asarray(params, dtype=np.float32)
        if p.size != NPARAMS:
            raise ValueError(f"expected {NPARAMS} parameters, got {p.size}")
        self.params = torch.as_tensor(p).cuda().contiguous()
        self.history = []

    def weights(self, plan, with_obs=False, tau=0.0, compact=True):
        """Stencil weights of G for the system currently assembled on `plan`: by
        default the compact form (rows per cell and time class, and per observed
        node), else one row per node."""
        if compact:
            return plan.precond_weights_compact(self.params, with_obs, tau)
        return plan.precond_weights(self.params, with_obs, tau)[0]

    def train(self, make_system, steps, probes=4, lr=3e-3, seed=0, smooth=2, sweeps=20):
        """`make_system(rng)` assembles one system and returns (plan, with_obs, tau).
        Of the `probes` columns of each block, `smooth` are random +-1 vectors
        after `sweeps` damped-Jacobi sweeps on the system (its slowly converging,
        smooth error directions, which the plain probes under-weight)."""
        torch = _torch()
        rng = np.random.default_rng(seed)
        gen = torch.Generator(device="cuda")
        gen.manual_seed(seed)
        m = torch.zeros_like(self.params)
        v = torch.zeros_like(self.params)
        for t in range(1, steps + 1):
            plan, with_obs, tau = make_system(rng)
            w, act = plan.precond_weights(self.params, with_obs, tau, keep_activations=True)
            n = plan.grid.n
            z = torch.randint(0, 2, (n, probes), device="cuda", generator=gen, dtype=torch.int8).double() * 2 - 1
            if smooth > 0:
                zs = plan.jacobi_smooth(z[:, :smooth].contiguous(), with_obs, tau, 0.6, sweeps)
                z = torch.cat([zs, z[:, smooth:]], 1).contiguous()
            loss, g = plan.precond_grad(self.params, w, act, z, with_obs, tau)
            plan.adam_step(self.params, g, m, v, t, lr=lr)
            self.history.append(loss)
        return self.history

    def state(self):
        return self.params.cpu().numpy().copy()


def prior_sample(w, rng):
    """Parameters of the non-stationary advection-diffusion generator drawn from
    a prior around its defaults: kappa in [0.1, 1], gamma in [0.2, 2] (tied
    B-spline coefficients), anisotropy coefficients N(0, 0.3^2), lambda in
    [0, 2], log sigma N(0, 0.3^2), tau in [25, 400] (noise sd 0.2 .. 0.05)."""
    nb2 = w.grid.Nbs2
    par = w.par.copy()
    par[0:nb2] = rng.uniform(np.log(0.1), np.log(1.0))
    par[nb2:2 * nb2] = rng.uniform(np.log(0.2), np.log(2.0))
    par[2 * nb2:4 * nb2] = rng.normal(0.0, 0.3, 2 * nb2)
    par[4 * nb2] = rng.uniform(0.0, 2.0)
    par[4 * nb2 + 1] = rng.normal(0.0, 0.3)
    par[-1] = rng.uniform(np.log(25.0), np.log(400.0))
    return par


def system_maker(w, model, obs_frac=0.01):
    """Training systems for `model` (an SPDE object on the workload's grid with
    an iterative or factor plan): A = Q(theta) + tau S^T S with theta from
    ``prior_sample`` and a fresh random observation set."""
    def make(rng):
        par = prior_sample(w, rng)
        model._assemble(par)
        n = w.grid.n
        idx = np.sort(rng.choice(n, max(1, int(round(obs_frac * n))), replace=False))
        model.plan.set_obs(idx)
        return model.plan, True, float(np.exp(par[-1]))
    return make
