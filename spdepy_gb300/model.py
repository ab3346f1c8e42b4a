"""Model facade with the reference's API (reference ``model.py:7-162``).

``Model.sample`` draws x = mu + P L^-T z from the GPU factor Q = P L L^T P^T
(reference ``model.py:73-87``), ``Model.update`` forms the conditional mean with
(Q + tau S^T S) on the GPU (``:120-127``), and ``Model.qinv`` returns the
marginal variances diag(Q^-1) from the GPU selected inverse, replacing the
R-INLA call of the reference (``:89-118``).  Because the factor's ordering is
not CHOLMOD's, samples are different draws from the same distribution.
"""
from __future__ import annotations

import numpy as np

from .grids import Grid
from .optim import Optimize
from .spdes import spde_init


def _torch():
    import torch
    return torch


class Model:
    def __init__(self, spde=None, grid: Grid = None, parameters=None, ani=True, ha=True, bc=3, mod0=None,
                 precision="mixed"):
        self.grid = grid
        self.precision = precision
        self.mod = None
        if spde is not None:
            self.model(spde=spde, grid=grid, parameters=parameters, ani=ani, ha=ha, bc=bc, mod0=mod0)
        self.Q = None
        self.mvar = None
        self.mu = np.zeros(self.grid.n)
        self.useCov = False
        self.sigmas = np.log(np.array([0.01, 140]))
        self.tau = None
        self._obs_nodes = np.zeros(0, dtype=np.int64)
        self._obs_tau = None

    def model(self, spde=None, grid=None, parameters=None, ani=True, ha=True, bc=3, mod0=None):
        assert spde is not None and grid is not None
        if grid.T > 1 and mod0 is None:
            mod0 = spde_init("whittle-matern", grid.spatial(), ani=ani, ha=ha, bc=bc, precision=self.precision)
        self.mod = spde_init(spde, grid, parameters=parameters, ani=ani, ha=ha, bc=bc, mod0=mod0,
                             precision=self.precision)
        self.spde_type = self.mod.type
        self.optim = Optimize(self.mod.logLike)

    def setQ(self, par=None):
        self.mod.setQ(par=par)

    def getPars(self, onlySelf=True):
        return self.mod.getPars(onlySelf=onlySelf)

    def fit(self, data, **kwargs):
        x0 = self.mod.initFit(data, **kwargs)
        if kwargs.get("x0") is None:
            kwargs["x0"] = x0
        res = self.optim.fit(**kwargs)
        self.setQ(par=res["x"])
        return res

    def setModel(self, mu=None, sigmas=None, useCov=None, scale=True):
        if useCov:
            raise NotImplementedError("covariate / intercept blocks are not on the GPU path")
        self.mu = np.zeros(self.grid.n) if mu is None else self.grid.getS().T @ np.asarray(mu, float)
        if self.mod.Q is None:
            self.mod.setQ()
        self.Q = self.mod.Q
        self.tau = float(np.exp(self.mod.par[-1]))
        self._obs_nodes = np.zeros(0, dtype=np.int64)
        self._obs_tau = None

    def _factor_current(self):
        plan = self.mod.plan
        self.mod._assemble(self.mod.par)
        if self._obs_nodes.size:
            plan.set_obs(self._obs_nodes)
            return plan.factor(True, self._obs_tau)
        return plan.factor(False, 0.0)

    def sample(self, n=1, simple=False, seed=None):
        """Draws S (mu + P L^-T z) (+ noise unless simple), reference model.py:73-87."""
        torch = _torch()
        if self.Q is None:
            self.setModel()
        if seed is None:
            seed = np.random.randint(100)
        nn = self.grid.n
        z = np.random.default_rng(seed).normal(size=nn * n).reshape(nn, n)
        self._factor_current()
        x = self.mod.plan.sample(torch.as_tensor(z)).cpu().numpy() + self.mu[:, None]
        S = self.grid.getS()
        data = S @ x
        if not simple:
            data += S[:, : self.grid.M * self.grid.N * self.grid.T] @ z[: self.grid.M * self.grid.N * self.grid.T] / np.sqrt(self.tau)
        return data

    def qinv(self, simple=False):
        """Marginal variances diag(Q^-1) (reference model.py:89-118)."""
        if simple:
            z = self.sample(n=1000, simple=True)
            return z.var(axis=1)
        if self.Q is None:
            self.setModel()
        self._factor_current()
        zq = self.mod.plan.selinv()
        centre = 12 if self.grid.T == 1 else 21
        self.mvar = zq[:, centre].cpu().numpy()
        return self.mvar

    def update(self, y, idx, tau=None):
        """Conditional mean with the observations (reference model.py:120-127)."""
        torch = _torch()
        if self.Q is None:
            self.setModel()
        tau = self.tau if tau is None else float(tau)
        if self._obs_tau is not None and tau != self._obs_tau:
            raise NotImplementedError("observations with different precisions in one model")
        nodes = self.grid.obs_nodes(idx)
        self._obs_nodes = np.concatenate([self._obs_nodes, nodes])
        self._obs_tau = tau
        self._factor_current()
        b = np.zeros(self.grid.n)
        np.add.at(b, nodes, tau * (np.asarray(y, float) - self.mu[nodes]))
        dx, _ = self.mod.plan.solve(torch.as_tensor(b))
        self.mu = self.mu + dx.cpu().numpy()

    def simulate(self):
        pass

    def plot(self):
        pass
