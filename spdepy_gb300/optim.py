"""Optimisers driving ``logLike`` (the caller of the GPU hot path).

``Optimize.fit`` behaves as the reference's (``optim/__init__.py:26-62,152-160``):
a fixed number of steps, an optional per-step learning-rate schedule, a ``fix``
mask of parameters held constant, and Polyak averaging of the last ``pol``
iterates, with the reference's step rules ``stepType`` = ``"adam"`` (default,
``optim/adam.py``), ``"rmsprop"`` (``optim/rmsprop.py``), ``"sgd"``
(``optim/sgd.py``), ``"adagrad"`` (``optim/ada_grad.py``) and ``"adadelta"``
(``optim/ada_delta.py``), each with the reference's settings and the same update
arithmetic (pinned by ``tests/golden/optim.npz``).  Two departures: a scalar
``lr`` is used for every step (the reference's loop reads it from a schedule
only), and ``"sgd"`` runs (the reference's ``SGD`` lacks the ``printInit`` its
loop calls).  ``stepType="lbfgs"`` runs limited-memory BFGS (scipy's
L-BFGS-B) on the exact adjoint gradients, with fixed parameters held by equal
bounds; ``max_steps`` bounds its iterations.
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


class RMSprop:
    """Gradient scaled by a running RMS (weight `memory`) plus momentum (`decay`);
    a zero mean square is replaced by 1, as in the reference."""

    def __init__(self, decay=0.0, memory=0.9):
        self.decay, self.memory = decay, memory
        self.gf2 = None
        self.dx = 0

    def __call__(self, x, f, g, lr):
        self.gf2 = g ** 2 if self.gf2 is None else self.memory * self.gf2 + (1 - self.memory) * g ** 2
        if hasattr(self.gf2, "__len__"):
            self.gf2[self.gf2 == 0] = 1
        self.dx = self.decay * self.dx - lr * g / np.sqrt(self.gf2)
        return x + self.dx


class SGD:
    """Gradient descent with momentum `decay`."""

    def __init__(self, decay=0.9):
        self.decay = decay
        self.dx = 0

    def __call__(self, x, f, g, lr):
        self.dx = self.decay * self.dx - lr * g
        return x + self.dx


class Adagrad:
    """Gradient scaled by the root of the summed squares.  The step adds 1e-8 to
    the root whatever `epsilon` is set to, as the reference's does."""

    def __init__(self, epsilon=1e-8):
        self.epsilon = epsilon
        self.g2 = None

    def __call__(self, x, f, g, lr):
        self.g2 = g ** 2 if self.g2 is None else self.g2 + g ** 2
        return x - lr * g / (np.sqrt(self.g2) + 1e-8)


class AdaDelta:
    """Zeiler's AdaDelta (no learning rate): running means of the squared
    gradients and steps with weight `rho`, started from zero as in the reference."""

    def __init__(self, rho=0.9, epsilon=1e-8):
        self.rho, self.epsilon = rho, epsilon
        self.egf2 = self.dx = self.edx2 = None

    def __call__(self, x, f, g, lr):
        r, e = self.rho, self.epsilon
        if self.egf2 is None:
            self.egf2 = (1 - r) * g ** 2
            self.dx = -np.sqrt(e) / np.sqrt(self.egf2 + e) * g
            self.edx2 = (1 - r) * self.dx ** 2
        else:
            self.egf2 = r * self.egf2 + (1 - r) * g ** 2
            self.dx = -np.sqrt(self.edx2 + e) / np.sqrt(self.egf2 + e) * g
            self.edx2 = r * self.edx2 + (1 - r) * self.dx ** 2
        return x + self.dx


def make_step(step_type, kw):
    """The step rule `step_type` with the settings in kw (the reference's names
    and defaults)."""
    def get(name, default):
        v = kw.get(name)
        return default if v is None else v
    if step_type == "adam":
        return Adam(get("beta1", 0.9), get("beta2", 0.999), get("epsilon", 1e-8))
    if step_type == "rmsprop":
        return RMSprop(get("decay", 0.0), get("memory", 0.9))
    if step_type == "sgd":
        return SGD(get("decay", 0.9))
    if step_type == "adagrad":
        return Adagrad(get("epsilon", 1e-8))
    if step_type == "adadelta":
        return AdaDelta(get("rho", 0.9), get("epsilon", 1e-8))
    raise ValueError("Step type not recognized")


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
        step_type = kw.get("stepType") or "adam"
        if step_type == "lbfgs":
            return self._lbfgs(fun, **kw)
        x = np.asarray(kw["x0"], dtype=np.float64).copy()
        lr = kw.get("lr", self.lr)
        steps = kw.get("max_steps") or (len(lr) if hasattr(lr, "__len__") else 100)
        pol = kw.get("pol", self.pol)
        fix = kw.get("fix")
        self.step = make_step(step_type, kw)
        self.histX, self.histF, self.histJac = [], [], []
        f = jac = None
        verbose = bool(kw.get("verbose"))
        show = kw.get("print")
        for it in range(steps):
            f, jac = fun(x)
            if verbose:  # the reference's progress line (optim/__init__.py, fitviz)
                print("# %3.0d" % it, "| fun = %2.4f" % f, show(x) if show is not None else "")
            self.histF.append(f)
            self.histJac.append(jac)
            step_lr = lr[it] if hasattr(lr, "__len__") else lr
            keep = x[fix].copy() if fix is not None else None
            x = self.step(x, f, jac, step_lr)
            if fix is not None:
                x[fix] = keep
            self.histX.append(x.copy())
        x = np.array(self.histX).T[:, -pol:].mean(axis=1)
        res = {"method": step_type, "x": x, "fun": f, "jac": jac}
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
