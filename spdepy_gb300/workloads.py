"""Synthetic workloads with the shapes of the benchmark configurations.

There is no public dataset for this path: the fields, parameters and
observations below are seeded synthetic stand-ins with the sizes and value
distributions the configurations state.

* ``nonstationary_advection_diffusion`` (200 x 200 x 24, seed 1): spatially
  varying diffusion through a 5 x 5 (Nbs = 5) degree-2 B-spline basis for the
  anisotropy vector (vx, vy) with N(0, 0.3^2) coefficients, constant kappa and
  gamma (their B-spline coefficients tied), advection by a smooth random velocity
  field built from 16 Fourier modes (amplitude 0.5, wavelengths 20-80 cells)
  scaled by lambda, a stationary anisotropic Whittle-Matern initial field, 1 % of
  nodes observed with noise sd 0.1.  The model class is the reference's
  CovAdvectionVarDiffusion2D generalised to Nbs = 5 (reference
  ``spdes/cov_advection_var_diffusion2D.py``).
* ``stationary_advection_diffusion`` (100 x 100 x 24): constant velocity
  (0.3, -0.2), H = diag(1.0, 0.5), kappa = 0.3, 2,000 observations per step,
  noise sd 0.05 (reference ``spdes/advection_diffusion2D.py``).
"""
from __future__ import annotations

import numpy as np

from .grids import Grid


def fourier_velocity(M, N, modes=16, amplitude=0.5, wl=(20.0, 80.0), seed=1):
    """Divergence-free smooth velocity (we, wn) at cell centres from a stream
    function of `modes` random plane waves; RMS speed ~ `amplitude`."""
    rng = np.random.default_rng(seed)
    X, Y = np.meshgrid(np.arange(M, dtype=float), np.arange(N, dtype=float))
    we = np.zeros_like(X)
    wn = np.zeros_like(X)
    a = amplitude * np.sqrt(2.0 / modes)
    for _ in range(modes):
        lam = rng.uniform(*wl)
        ang = rng.uniform(0, 2 * np.pi)
        ph = rng.uniform(0, 2 * np.pi)
        kx, ky = 2 * np.pi / lam * np.cos(ang), 2 * np.pi / lam * np.sin(ang)
        s = np.sin(kx * X + ky * Y + ph)
        kn = np.hypot(kx, ky)
        we += a * (-ky / kn) * s
        wn += a * (kx / kn) * s
    return we.ravel(), wn.ravel()


class Workload:
    def __init__(self, name, grid, family, diff, bc, par, idx, noise_sd, ww=None, mod0_par=None):
        self.name, self.grid, self.family, self.diff, self.bc = name, grid, family, diff, bc
        self.par, self.idx, self.noise_sd, self.ww, self.mod0_par = par, idx, noise_sd, ww, mod0_par
        self.y = None


def nonstationary_advection_diffusion(M=200, N=200, T=24, Nbs=5, seed=1, obs_frac=0.01, bc=3):
    grid = Grid(np.arange(M, dtype=float), np.arange(N, dtype=float), np.arange(T, dtype=float), None, Nbs)
    we, wn = fourier_velocity(M, N, seed=seed)
    ww = grid.assimilate_adv(we, wn)
    rng = np.random.default_rng(seed)
    nb2 = Nbs * Nbs
    vx = rng.normal(0.0, 0.3, nb2)
    vy = rng.normal(0.0, 0.3, nb2)
    mod0 = np.array([np.log(0.3), np.log(0.5), np.sqrt(0.5), 0.0])
    par = np.hstack([np.full(nb2, np.log(0.3)), np.full(nb2, np.log(0.5)), vx, vy, 1.0, 0.0, mod0,
                     np.log(1.0 / 0.1 ** 2)])
    idx = np.sort(rng.choice(M * N * T, int(round(obs_frac * M * N * T)), replace=False))
    return Workload(f"nonstationary advection-diffusion {M}x{N}x{T}", grid, "cov-advection-var-diffusion", "ani", bc,
                    par, idx, 0.1, ww=ww, mod0_par=mod0)


def stationary_advection_diffusion(M=100, N=100, T=24, seed=0, obs_per_step=2000, bc=1):
    grid = Grid(np.arange(M, dtype=float), np.arange(N, dtype=float), np.arange(T, dtype=float), None, 3)
    mod0 = np.array([np.log(0.3), np.log(0.5), np.sqrt(0.5), 0.0])
    par = np.hstack([np.log(0.3), np.log(0.5), np.sqrt(0.5), 0.0, 0.3, -0.2, 0.0, mod0, np.log(1 / 0.05 ** 2)])
    idx = []
    for t in range(T):
        r = np.random.default_rng(seed + t)
        idx.append(t * M * N + np.sort(r.choice(M * N, obs_per_step, replace=False)))
    return Workload(f"stationary advection-diffusion {M}x{N}x{T}", grid, "advection-diffusion", "ani", bc, par,
                    np.concatenate(idx), 0.05, mod0_par=mod0)


def sensor_track(M, N, T, steps_per_t=2000, seed=3):
    """Node indices of a 1-cell-wide random walk (4-neighbour moves, reflected at
    the border) sampled `steps_per_t` times per time step and continued across
    time steps; revisited cells give repeated observations."""
    rng = np.random.default_rng(seed)
    x, y = int(rng.integers(M)), int(rng.integers(N))
    moves = np.array([(1, 0), (-1, 0), (0, 1), (0, -1)])
    out = []
    for t in range(T):
        for _ in range(steps_per_t):
            dx, dy = moves[rng.integers(4)]
            x = x + dx if 0 <= x + dx < M else x - dx
            y = y + dy if 0 <= y + dy < N else y - dy
            out.append(t * M * N + y * M + x)
    return np.asarray(out, dtype=np.int64)


def sensor_track_advection_diffusion(M=150, N=150, T=36, seed=3, obs_frac=0.005, steps_per_t=2000):
    """The non-stationary generator (seed 3) observed at 0.5 % of nodes at random
    plus a simulated sensor track of 2,000 points per time step, noise sd 0.05."""
    w = nonstationary_advection_diffusion(M, N, T, seed=seed, obs_frac=obs_frac)
    track = sensor_track(M, N, T, steps_per_t, seed=seed + 100)
    w.idx = np.sort(np.concatenate([w.idx, track]))
    w.noise_sd = 0.05
    w.par = w.par.copy()
    w.par[-1] = np.log(1.0 / 0.05 ** 2)
    w.name = f"nonstationary advection-diffusion {M}x{N}x{T} with sensor track"
    return w


def build_model(w: Workload, precision="mixed"):
    """GPU model object for a workload (observations attached, data simulated)."""
    from .spdes import _CLASSES
    mod0 = _CLASSES[("whittle-matern", "ani")](grid=w.grid.spatial(), bc=w.bc, precision=precision)
    mod0.setPars(np.hstack([w.mod0_par, 0.0]))
    mod = _CLASSES[(w.family, w.diff)](grid=w.grid, bc=w.bc, mod0=mod0, ww=w.ww, precision=precision)
    mod.setPars(w.par)
    return mod


def simulate(mod, w: Workload, seed=2):
    """y = S x + noise with x ~ N(0, Q(theta*)^-1), drawn on the GPU."""
    import torch
    mod._assemble(w.par)
    mod.plan.factor(False, 0.0)
    z = torch.as_tensor(np.random.default_rng(seed).normal(size=w.grid.n))
    x = mod.plan.sample(z).cpu().numpy()
    nodes = w.grid.obs_nodes(w.idx)
    y = x[nodes] + w.noise_sd * np.random.default_rng(seed + 1).normal(size=nodes.size)
    w.y = y
    mod.initFit(y, idx=w.idx)
    return y
