"""Optimisers driving ``logLike`` (the caller of the GPU hot path).

``stepType="adam"`` (default) behaves as the reference's ``Optimize`` with the
Adam step (``optim/__init__.py:26-62,152-160``, ``optim/adam.py:3-43``): a fixed
number of steps, an optional per-step learning-rate schedule, a ``fix`` mask of
parameters held constant, and Polyak averaging of the last ``pol`` iterates.
``stepType="lbfgs"`` runs limited-memory BFGS (scipy's L-BFGS-B) on the exact
adjoint gradients, with fixed parameters held by equal bounds; ``max_steps``
bounds its iterations.
"""
from __future__ import annotations

import numpy as np


class Adam:
    def __init__(self, beta1=0.9, beta2=0.999, epsilon=1e-8):
        self.beta1, self.beta2, self.epsilon = beta1, beta2, epsilon
        self.reset()

    def reset(self):
        self.m = None
        self.v = None
        self.t = 0

    def __call__(self, x, f, g, lr):
        self.t += 1
        if self.m is None:
            self.m, self.v = g, g ** 2
        else:
            self.m = self.beta1 * self.m + (1 - self.beta1) * g
            self.v = self.beta2 * self.v + (1 - self.beta2) * g ** 2
        mhat = self.m / (1 - self.beta1 ** self.t)
        vhat = self.v / (1 - self.beta2 ** self.t)
        return x - lr * mhat / (np.sqrt(vhat) + self.epsilon)


class Optimize:
    def __init__(self, fun=None):
        self.fun = fun
        self.lr = 0.1
        self.pol = 10
        self.max_steps = None
        self.step = Adam()

    def fit(self, **kw):
        fun = kw.get("fun", self.fun)
        assert fun is not None
        if kw.get("stepType", "adam") == "lbfgs":
            return self._lbfgs(fun, **kw)
        x = np.asarray(kw["x0"], dtype=np.float64).copy()
        lr = kw.get("lr", self.lr)
        steps = kw.get("max_steps") or (len(lr) if hasattr(lr, "__len__") else 100)
        pol = kw.get("pol", self.pol)
        fix = kw.get("fix")
        self.step = Adam(kw.get("beta1", 0.9), kw.get("beta2", 0.999), kw.get("epsilon", 1e-8))
        self.histX, self.histF, self.histJac = [], [], []
        f = jac = None
        for it in range(steps):
            f, jac = fun(x)
            self.histF.append(f)
            self.histJac.append(jac)
            step_lr = lr[it] if hasattr(lr, "__len__") else lr
            keep = x[fix].copy() if fix is not None else None
            x = self.step(x, f, jac, step_lr)
            if fix is not None:
                x[fix] = keep
            self.histX.append(x.copy())
        x = np.array(self.histX).T[:, -pol:].mean(axis=1)
        res = {"method": "adam", "x": x, "fun": f, "jac": jac}
        if kw.get("end") is not None:
            np.save(kw["end"] + ".npy", x)
        return res

    def _lbfgs(self, fun, **kw):
        from scipy.optimize import minimize
        x0 = np.asarray(kw["x0"], dtype=np.float64).copy()
        fix = kw.get("fix")
        bounds = None
        if fix is not None:
            mask = np.zeros(x0.size, dtype=bool)
            mask[fix] = True
            bounds = [(v, v) if m else (None, None) for v, m in zip(x0, mask)]
        self.histX, self.histF, self.histJac = [], [], []

        def f(x):
            val, jac = fun(x)
            self.histX.append(x.copy())
            self.histF.append(val)
            self.histJac.append(jac)
            return val, jac

        opts = {"maxiter": kw.get("max_steps") or 200, "gtol": kw.get("gtol", 1e-6), "ftol": kw.get("ftol", 1e-12)}
        r = minimize(f, x0, jac=True, method="L-BFGS-B", bounds=bounds, options=opts)
        res = {"method": "lbfgs", "x": r.x, "fun": r.fun, "jac": r.jac, "nit": int(r.nit), "nfev": int(r.nfev),
               "message": str(r.message)}
        if kw.get("end") is not None:
            np.save(kw["end"] + ".npy", r.x)
        return res
