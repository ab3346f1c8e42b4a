"""Model facade with the reference's API (reference ``model.py:7-162``).

``Model.sample`` draws x = mu + P L^-T z from the GPU factor Q = P L L^T P^T
(reference ``model.py:73-87``), ``Model.update`` forms the conditional mean with
(Q + tau S^T S) on the GPU (``:120-127``), and ``Model.qinv`` returns the
marginal variances diag(Q^-1) from the GPU selected inverse, replacing the
R-INLA call of the reference (``:89-118``).  Because the factor's ordering is
not CHOLMOD's, samples are different draws from the same distribution.

With ``setModel(useCov=True)`` the latent field carries the reference's fixed
effects (intercept and covariate coefficients, ``:129-150``); their border is
eliminated on the host around the sparse GPU factor (``fixed_effects.py``).
"""
from __future__ import annotations

import numpy as np

from .fixed_effects import Border, update_step
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
        self._obs = []  # (nodes, tau) of every update since setModel
        self.border = None

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
        if kwargs.get("verbose") is not None and hasattr(self.mod, "print"):
            kwargs["print"] = self.mod.print
        res = self.optim.fit(**kwargs)
        self.setQ(par=res["x"])
        return res

    def setModel(self, mu=None, sigmas=None, useCov=None, scale=True):
        """Prior mean and, with useCov, the fixed effects (reference model.py:129-150):
        two sigmas give an intercept and a covariate coefficient (the covariate is
        `mu`, its coefficient's prior mean max(mu) when scale), one sigma an
        intercept alone; exp(sigmas) are their prior precisions."""
        self.useCov = useCov if useCov is not None else self.useCov
        if self.mod.Q is None:
            self.mod.setQ()
        self.Q = self.mod.Q
        self.tau = float(np.exp(self.mod.par[-1]))
        self._obs = []
        self.border = None
        n = self.grid.n
        if not self.useCov:
            self.mu = np.zeros(n) if mu is None else self.grid.getS().T @ np.asarray(mu, float)
            return
        self.sigmas = sigmas if sigmas is not None else self.sigmas
        if mu is None:
            raise ValueError("the fixed-effect model needs the covariate field mu")
        field = np.asarray(mu, float)
        if hasattr(self.sigmas, "__len__"):
            self.grid.addCov(field, scale=scale)
            p = self.grid._fixed_effects().shape[1]
            if scale:
                self.mu = np.zeros(n + p)
                self.mu[-2:] = [0.0, field.max()]
            else:
                self.mu = self.grid.getS().T @ field
        else:
            self.grid.addInt()
            S = self.grid.getS()
            self.mu = np.zeros(S.shape[1])
            self.mu[:-1] = S[:, :-1].T @ field
        self.border = Border(n, np.exp(np.atleast_1d(np.asarray(self.sigmas, float))))

    def _factor_current(self):
        """Factor Q plus the observation terms of every update so far: the
        reference's self.Q after Q += tau_k S_k^T S_k per call (model.py:122)."""
        plan = self.mod.plan
        self.mod._assemble(self.mod.par)
        if not self._obs:
            return plan.factor(False, 0.0)
        nodes = np.concatenate([nd for nd, _ in self._obs])
        taus = {t for _, t in self._obs}
        if len(taus) == 1:
            plan.set_obs(nodes)
            return plan.factor(True, taus.pop())
        # different precisions per call: per-observation weights tau_k, tau = 1
        plan.set_obs(nodes, weights=np.concatenate([np.full(nd.size, t) for nd, t in self._obs]))
        return plan.factor(True, 1.0)

    def _solve_A(self, R):
        """A^-1 R with the current factor (R: n x k host array)."""
        torch = _torch()
        x, _ = self.mod.plan.solve(torch.as_tensor(np.ascontiguousarray(R, dtype=np.float64)))
        return x.cpu().numpy()

    def _sample_A(self, Z):
        """P L^-T Z with the current factor (Z: n x k host array)."""
        torch = _torch()
        return self.mod.plan.sample(torch.as_tensor(np.ascontiguousarray(Z, dtype=np.float64))).cpu().numpy()

    def sample(self, n=1, simple=False, seed=None):
        """Draws S (mu + P L^-T z) (+ noise unless simple), reference model.py:73-87.
        With fixed effects z has n + p rows and the draw covers the coefficients too."""
        if self.Q is None:
            self.setModel()
        if seed is None:
            seed = np.random.randint(100)
        nn = self.grid.n
        p = self.border.p if self.useCov and self.border is not None else 0
        z = np.random.default_rng(seed).normal(size=(nn + p) * n).reshape(nn + p, n)
        self._factor_current()
        if p:
            x_n, x_b = self.border.sample(self._sample_A, self._solve_A, z[:nn], z[nn:])
            x = np.vstack([x_n, x_b]) + self.mu[:, None]
        else:
            x = self._sample_A(z) + self.mu[:, None]
        S = self.grid.getS()
        data = S @ x
        if not simple:
            data += S[:, : self.grid.M * self.grid.N * self.grid.T] @ z[: self.grid.M * self.grid.N * self.grid.T] / np.sqrt(self.tau)
        return data

    def qinv(self, simple=False):
        """Marginal variances (reference model.py:89-118), float32 like the
        reference's.  Without fixed effects: diag(Q^-1) of the current precision
        (Q plus every update's tau S^T S) from the GPU selected inverse, in place of
        R-INLA's.  With fixed effects the reference inverts S Q_aug S^T (S =
        getS() with its fixed-effect columns) and returns its diagonal in an
        (n + p)-vector; here the same diagonal comes from the selected inverse of A
        (the lattice block of Q_aug) and a Woodbury correction for the rank-2p
        border terms."""
        if simple:
            z = self.sample(n=1000, simple=True)
            return z.var(axis=1)
        if self.Q is None:
            self.setModel()
        plan = self.mod.plan
        centre = plan.nslots // 2  # the (0, 0, 0) slot of every stencil layout
        self._factor_current()
        if self.useCov and self.border is not None:
            self.mvar = self._qinv_fixed_effects(centre)
            return self.mvar
        zq = plan.selinv()
        self.mvar = zq[:, centre].cpu().numpy().astype(np.float32)
        return self.mvar

    def _qinv_fixed_effects(self, centre):
        """diag((S Q_aug S^T)^-1) with S = [I | X] and Q_aug = [[A, B], [B^T, C]]:
        S Q_aug S^T = A + U W U^T, U = [X, B], W = [[C, I], [I, 0]], so with
        Y = A^-1 U and K = (W^-1 + U^T Y)^-1, W^-1 = [[0, I], [I, -C]]:
        diag = diag(A^-1) - rowsum((Y K) * Y)."""
        g = self.grid
        if g.Ne:
            raise NotImplementedError("marginal variances with fixed effects on an extended grid: S selects a "
                                      "principal submatrix of the lattice precision, whose inverse the selected "
                                      "inverse of the whole lattice does not give")
        n, p = g.n, self.border.p
        X = g._fixed_effects()
        U = np.hstack([X, self.border.B])
        Y = self._solve_A(U).reshape(n, 2 * p)   # before the selected inversion consumes the factor
        Winv = np.block([[np.zeros((p, p)), np.eye(p)], [np.eye(p), -self.border.C]])
        K = np.linalg.inv(Winv + U.T @ Y)
        zq = self.mod.plan.selinv()
        d = zq[:, centre].cpu().numpy() - np.einsum("ij,ij->i", Y @ K, Y)
        mvar = np.zeros(n + p, dtype=np.float32)
        mvar[:n] = d
        return mvar

    def update(self, y, idx, tau=None):
        """Conditional mean with the observations (reference model.py:120-127)."""
        torch = _torch()
        if self.Q is None:
            self.setModel()
        tau = self.tau if tau is None else float(tau)
        nodes = self.grid.obs_nodes(idx)
        self._obs.append((nodes, tau))
        self._factor_current()
        if self.useCov and self.border is not None:
            rows = np.arange(self.grid.M * self.grid.N * self.grid.T) if idx is None else np.asarray(idx, np.int64)
            X = self.grid._fixed_effects()[rows]
            self.mu = update_step(self.border, self._solve_A, self.mu, nodes, X, y, tau)
            return
        b = np.zeros(self.grid.n)
        np.add.at(b, nodes, tau * (np.asarray(y, float) - self.mu[nodes]))
        dx, _ = self.mod.plan.solve(torch.as_tensor(b))
        self.mu = self.mu + dx.cpu().numpy()

    def simulate(self):
        pass

    def plot(self):
        pass
