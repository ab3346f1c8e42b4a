"""Generate the golden vectors in tests/golden/*.npz from the reference itself.

Run in a container that has the reference tree (after ``make -C oracle``):

    python tests/golden/make_golden.py

Every number in the fixtures comes from the reference's own Python classes and
its own compiled stencils (see ``ref_harness.py`` for how they are imported).
The fixtures pin both the oracle (``oracle/spde_oracle.py``) and, through it,
the CUDA path.  Cases:

* ``stencil_*``  raw COO triplets (with the ``row == M*N`` sentinel) of the four
  stencil families ``AcH/AH/Acw/Aw`` for bc 1 and 3 and every ``diff`` mode
  (reference ``spdes/ccode/*.cpp``).
* ``model_*``    one model object each: the precision Q (CSR), the objective
  ``logLike(par, grad=False)`` and the Hutchinson gradient
  ``logLike(par, nh1, grad=True)`` with ``np.random.seed`` fixed before the call
  (reference e.g. ``spdes/advection_diffusion2D.py:187-223``).
* ``facade_wm``  ``Model.update`` conditional mean (reference ``model.py:120-127``).
* ``separable_*`` separable space-time models Q = Qt (x) Qs, as the ``model_*``
  cases (reference ``spdes/seperable_spatial_temporal2D.py`` and
  ``seperable_spatial_temporal_idiffusion2D.py``).  They pin the oracle and,
  through ``tests/test_gpu_separable.py``, the CUDA path's 75-slot plans; they
  carry their own prefix because their parameter layout differs.

* ``facade_cov``  ``Model.setModel(useCov=True)`` and two ``update`` calls, with
  covariate + intercept and with intercept only (reference ``model.py:120-150``).
* ``facade_tau``  ``Model.update`` twice with different ``tau`` (the reference
  accumulates Q += tau_k S_k^T S_k, ``model.py:120-127``), without and with fixed
  effects.
* ``grid_adv``  face velocities on extended grids: ``assimilate_adv`` (with the
  ``advBound`` ramp into the padding cells) and ``evalAdv`` of the B-spline
  velocity, plus the bases on the extended grid
  (``grids/spat2Dtemp_regular_mesh.py:102-117,157-391``).
* ``model_*_ext2``  model objects on a grid extended by two cells
  (``extend=2``): the velocity field and the observations go through the
  padding (``n2e``).
* ``grid_getS``  the observation matrix with fixed-effect columns: ``Grid.getS``
  after ``addInt`` / ``addCov`` (with and without intercept and scaling) on a
  padded space-time grid (reference ``grids/spat2Dtemp_regular_mesh.py:35-68``).

* ``optim``  the reference's ``Optimize.fit`` (``optim/__init__.py``) with each of
  its step rules (``adam``, ``rmsprop``, ``sgd``, ``adagrad``, ``adadelta``;
  ``optim/*.py``) on a fixed smooth objective: the trajectory, the Polyak
  average and the last objective, also with a learning-rate schedule, a ``fix``
  mask and non-default step settings.

``python tests/golden/make_golden.py --only separable [name ...]`` regenerates just
the separable cases, ``--only getS`` the grid_getS fixture, ``--only facade_cov`` the
facade_cov fixture, ``--only facade_tau`` the facade_tau fixture, ``--only plumbing``
the grid_adv and extended-grid model fixtures, ``--only optim`` the optim fixture.
"""
from __future__ import annotations

import ctypes
import os
import sys

import numpy as np
from scipy import sparse

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)
import ref_harness  # noqa: E402

OUT = HERE
NH1 = 20
SEED_V = 1234


def _stencil_cases():
    lib_dir = ref_harness.REF_LIBS
    M, N, hx, hy = 7, 6, 1.3, 0.8
    rng = np.random.default_rng(7)
    H = rng.normal(size=(M * N, 4, 2, 2))
    H = H + H.transpose(0, 1, 3, 2)  # symmetric per face, as the models build them
    Hc = np.array([[1.3, 0.4], [0.4, 0.7]])
    G = rng.normal(size=(M * N, 4))
    G[3, 1] = 0.0  # exercise the G/|G| = NaN path of the derivative modes
    dG = rng.normal(size=(M * N, 4))
    Gc = np.array([0.3, -0.2])
    out = {}
    c_int, c_dbl = ctypes.c_int, ctypes.c_double
    for bc in (1, 3):
        for fam in ("AcH", "AH"):
            lib = ctypes.cdll.LoadLibrary(os.path.join(lib_dir, f"lib_{fam}_2D_b{bc}.so"))
            lib.AH_new.restype = ctypes.c_void_p
            for f in ("AH_Row", "AH_Col", "AH_Val"):
                getattr(lib, f).argtypes = [ctypes.c_void_p]
            lib.AH_Row.restype = np.ctypeslib.ndpointer(dtype=np.int32, shape=(9 * M * N,))
            lib.AH_Col.restype = np.ctypeslib.ndpointer(dtype=np.int32, shape=(9 * M * N,))
            lib.AH_Val.restype = np.ctypeslib.ndpointer(dtype=np.float64, shape=(9 * M * N,))
            lib.AH_delete.argtypes = [ctypes.c_void_p]
            Hin = np.ascontiguousarray(Hc if fam == "AcH" else H.copy())
            lib.AH_new.argtypes = [c_int, c_int, np.ctypeslib.ndpointer(dtype=np.float64, shape=Hin.shape),
                                   c_dbl, c_dbl]
            obj = lib.AH_new(M, N, Hin, hx, hy)
            key = f"{fam}_b{bc}"
            out[key + "_row"] = lib.AH_Row(obj).copy()
            out[key + "_col"] = lib.AH_Col(obj).copy()
            out[key + "_val"] = lib.AH_Val(obj).copy()
            lib.AH_delete(obj)
        for fam in ("Acw", "Aw"):
            lib = ctypes.cdll.LoadLibrary(os.path.join(lib_dir, f"lib_{fam}_2D_b{bc}.so"))
            lib.Aw_new.restype = ctypes.c_void_p
            for f in ("Aw_Row", "Aw_Col", "Aw_Val"):
                getattr(lib, f).argtypes = [ctypes.c_void_p]
            lib.Aw_Row.restype = np.ctypeslib.ndpointer(dtype=np.int32, shape=(5 * M * N,))
            lib.Aw_Col.restype = np.ctypeslib.ndpointer(dtype=np.int32, shape=(5 * M * N,))
            lib.Aw_Val.restype = np.ctypeslib.ndpointer(dtype=np.float64, shape=(5 * M * N,))
            lib.Aw_delete.argtypes = [ctypes.c_void_p]
            for diff in (1, 2, 3):
                if fam == "Acw":
                    Gin = np.ascontiguousarray(Gc)
                    lib.Aw_new.argtypes = [c_int, c_int, np.ctypeslib.ndpointer(dtype=np.float64, shape=(2,)),
                                           c_dbl, c_dbl, c_int]
                    obj = lib.Aw_new(M, N, Gin, hx, hy, diff)
                else:
                    Gin = np.ascontiguousarray(G.copy())
                    dGin = np.ascontiguousarray(dG.copy())
                    nd = np.ctypeslib.ndpointer(dtype=np.float64, shape=(M * N, 4))
                    lib.Aw_new.argtypes = [c_int, c_int, nd, c_dbl, c_dbl, c_int, nd]
                    obj = lib.Aw_new(M, N, Gin, hx, hy, diff, dGin)
                key = f"{fam}_b{bc}_d{diff}"
                out[key + "_row"] = lib.Aw_Row(obj).copy()
                out[key + "_col"] = lib.Aw_Col(obj).copy()
                out[key + "_val"] = lib.Aw_Val(obj).copy()
                lib.Aw_delete(obj)
    np.savez_compressed(os.path.join(OUT, "stencils.npz"), M=M, N=N, hx=hx, hy=hy, H=H, Hc=Hc, G=G, dG=dG,
                        Gc=Gc, **out)


def _csr(Q):
    Q = sparse.csr_matrix(Q)
    Q.sort_indices()
    return dict(Q_data=Q.data, Q_indices=Q.indices.astype(np.int32), Q_indptr=Q.indptr.astype(np.int64))


def _simulate(Q, S, noise_sd, seed):
    rng = np.random.default_rng(seed)
    L = np.linalg.cholesky(Q.toarray())
    import scipy.linalg as sla
    x = sla.solve_triangular(L.T, rng.normal(size=Q.shape[0]), lower=False)
    return S @ x + noise_sd * rng.normal(size=S.shape[0])


def _model_case(name, mod, par, idx, noise_sd, gridinfo, extra=None, prefix="model"):
    Q = mod.Q if mod.Q is not None else mod.makeQ(par, grad=False)[0]
    S = mod.grid.getS(idx)
    y = _simulate(Q, S, noise_sd, seed=11)
    mod.initFit(y, idx=idx)
    f = mod.logLike(par, grad=False)
    np.random.seed(SEED_V)
    fg, jac = mod.logLike(par, nh1=NH1, grad=True)
    rec = dict(par=np.asarray(par, float), idx=np.asarray(idx, np.int64), y=y, f=f, f_grad=fg, jac=jac,
               nh1=NH1, seed_v=SEED_V, **_csr(Q), **gridinfo)
    if extra:
        rec.update(extra)
    np.savez_compressed(os.path.join(OUT, f"{prefix}_{name}.npz"), **rec)
    print(f"{name}: n={Q.shape[0]} nnz={Q.nnz} f={f:.12g} |jac|={np.linalg.norm(jac):.6g}")


def _st_grid(sp, M, N, T, Nbs=3, extend=None):
    g = sp.grid(x=np.arange(M, dtype=float), y=np.arange(N, dtype=float), t=np.arange(T, dtype=float),
                extend=extend, Nbs=Nbs)
    return g, dict(M=M, N=N, T=T, Nbs=Nbs, extend=-1 if extend is None else extend)


def _sp_grid(sp, M, N, Nbs=3):
    g = sp.grid(x=np.arange(M, dtype=float), y=np.arange(N, dtype=float), Nbs=Nbs)
    return g, dict(M=M, N=N, T=1, Nbs=Nbs, extend=-1)


def _mod0(sp, M, N, ani, ha, bc):
    g0 = sp.grid(x=np.arange(M, dtype=float), y=np.arange(N, dtype=float))
    return sp.spde_init(model="whittle-matern", grid=g0, ani=ani, ha=ha, bc=bc)


def _smooth_ww(grid, seed):
    rng = np.random.default_rng(seed)
    M, N = grid.M, grid.N
    X, Y = np.meshgrid(np.arange(M), np.arange(N))
    we = np.zeros(M * N)
    wn = np.zeros(M * N)
    for _ in range(4):
        kx, ky = rng.uniform(0.2, 0.8, size=2)
        ph = rng.uniform(0, 2 * np.pi, size=2)
        we += 0.5 * np.cos(kx * X + ky * Y + ph[0]).ravel()
        wn += 0.5 * np.sin(kx * X - ky * Y + ph[1]).ravel()
    return grid.assimilate_adv(we, wn)


def main():
    sp = ref_harness.load_reference()
    _stencil_cases()

    # config-1 shape: stationary anisotropic Whittle-Matern, 40x40, Neumann
    g, gi = _sp_grid(sp, 40, 40)
    par = np.array([-0.7, 0.0, 0.0, np.sqrt(np.exp(0.3) - 1.0), 1.0])
    mod = sp.spde_init(model="whittle-matern", grid=g, parameters=par, ani=True, ha=False, bc=1)
    idx = np.random.default_rng(0).choice(1600, 200, replace=False)
    _model_case("wm_ani_bc1", mod, par, idx, 0.1, dict(gi, bc=1, family="whittle-matern", ani=1, ha=0))

    g, gi = _sp_grid(sp, 15, 12)
    par = np.array([-0.5, 0.2, 1.5])
    mod = sp.spde_init(model="whittle-matern", grid=g, parameters=par, ani=False, ha=False, bc=3)
    idx = np.random.default_rng(1).choice(180, 60, replace=False)
    _model_case("wm_iso_bc3", mod, par, idx, 0.2, dict(gi, bc=3, family="whittle-matern", ani=0, ha=0))

    g, gi = _sp_grid(sp, 14, 13)
    par = np.array([-0.4, -0.2, 0.3, -0.5, 1.2])
    mod = sp.spde_init(model="whittle-matern", grid=g, parameters=par, ani=True, ha=True, bc=3)
    idx = np.random.default_rng(2).choice(182, 70, replace=False)
    _model_case("wm_ha_bc3", mod, par, idx, 0.2, dict(gi, bc=3, family="whittle-matern", ani=1, ha=1))

    g, gi = _sp_grid(sp, 12, 11)
    rng = np.random.default_rng(3)
    par = np.hstack([-0.5 + 0.2 * rng.normal(size=9), 0.1 * rng.normal(size=9), 0.3 * rng.normal(size=9),
                     0.3 * rng.normal(size=9), 1.0])
    mod = sp.spde_init(model="var-whittle-matern", grid=g, parameters=par, ani=True, ha=False, bc=1)
    idx = np.random.default_rng(4).choice(132, 50, replace=False)
    _model_case("varwm_ani_bc1", mod, par, idx, 0.2, dict(gi, bc=1, family="var-whittle-matern", ani=1, ha=0))

    # config-2 shape (reduced): stationary advection-diffusion with a fitted initial field
    for bc in (1, 3):
        M, N, T = 12, 10, 5
        g, gi = _st_grid(sp, M, N, T)
        par = np.array([np.log(0.3), np.log(0.5), np.sqrt(0.5), 0.0, 0.3, -0.2, 0.0,
                        np.log(0.3), np.log(0.5), np.sqrt(0.5), 0.0, np.log(1 / 0.05 ** 2)])
        mod0 = _mod0(sp, M, N, True, False, bc)
        mod = sp.spde_init(model="advection-diffusion", grid=g, parameters=par, ani=True, ha=False, bc=bc, mod0=mod0)
        idx = np.random.default_rng(5).choice(M * N * T, 150, replace=False)
        _model_case(f"advdiff_ani_bc{bc}", mod, par, idx, 0.05,
                    dict(gi, bc=bc, family="advection-diffusion", ani=1, ha=0))

    M, N, T = 10, 9, 4
    g, gi = _st_grid(sp, M, N, T)
    par = np.array([np.log(0.4), np.log(0.6), 0.4, -0.3, -0.25, 0.15, 0.2, np.log(0.5), np.log(0.7), 0.2, 0.1,
                    np.log(200.0)])
    mod0 = _mod0(sp, M, N, True, True, 3)
    mod = sp.spde_init(model="advection-diffusion", grid=g, parameters=par, ani=True, ha=True, bc=3, mod0=mod0)
    idx = np.random.default_rng(6).choice(M * N * T, 100, replace=False)
    _model_case("advdiff_ha_bc3", mod, par, idx, 0.1, dict(gi, bc=3, family="advection-diffusion", ani=1, ha=1))

    M, N, T = 9, 8, 4
    g, gi = _st_grid(sp, M, N, T)
    par = np.array([np.log(0.5), np.log(0.8), 0.35, -0.15, 0.1, np.log(0.5), np.log(0.9), np.log(150.0)])
    mod0 = _mod0(sp, M, N, False, False, 1)
    mod = sp.spde_init(model="advection-diffusion", grid=g, parameters=par, ani=False, ha=False, bc=1, mod0=mod0)
    idx = np.random.default_rng(7).choice(M * N * T, 90, replace=False)
    _model_case("advdiff_iso_bc1", mod, par, idx, 0.1, dict(gi, bc=1, family="advection-diffusion", ani=0, ha=0))

    # config-3 family at Nbs=3: spatially varying diffusion, given velocity field scaled by lambda
    from spdepy.spdes.cov_advection_var_diffusion2D import CovAdvectionVarDiffusion2D
    for bc in (1, 3):
        M, N, T = 11, 10, 4
        g, gi = _st_grid(sp, M, N, T)
        ww = _smooth_ww(g, seed=21)
        rng = np.random.default_rng(22)
        par = np.hstack([np.log(0.4) + 0.1 * rng.normal(size=9), np.log(0.6) + 0.1 * rng.normal(size=9),
                         0.3 * rng.normal(size=9), 0.3 * rng.normal(size=9), 0.8, 0.1,
                         np.log(0.4), np.log(0.6), 0.3, 0.0, np.log(100.0)])
        mod0 = _mod0(sp, M, N, True, False, bc)
        mod = CovAdvectionVarDiffusion2D(grid=g, mod0=mod0, par=par, bc=bc, ww=ww)
        mod.setQ(par)
        idx = np.random.default_rng(23).choice(M * N * T, 120, replace=False)
        _model_case(f"covadv_vardiff_bc{bc}", mod, par, idx, 0.1,
                    dict(gi, bc=bc, family="cov-advection-var-diffusion", ani=1, ha=0), extra=dict(ww=ww))

    M, N, T = 10, 9, 4
    g, gi = _st_grid(sp, M, N, T)
    rng = np.random.default_rng(31)
    par = np.hstack([np.log(0.4) + 0.1 * rng.normal(size=9), np.log(0.6) + 0.1 * rng.normal(size=9),
                     0.3 * rng.normal(size=9), 0.3 * rng.normal(size=9), 0.2 * rng.normal(size=9),
                     0.2 * rng.normal(size=9), 0.1, np.log(0.4), np.log(0.6), 0.3, 0.0, np.log(100.0)])
    mod0 = _mod0(sp, M, N, True, False, 1)
    mod = sp.spde_init(model="var-advection-var-diffusion", grid=g, parameters=par, ani=True, ha=False, bc=1,
                       mod0=mod0)
    idx = np.random.default_rng(32).choice(M * N * T, 100, replace=False)
    _model_case("varadv_vardiff_bc1", mod, par, idx, 0.1,
                dict(gi, bc=1, family="var-advection-var-diffusion", ani=1, ha=0))

    # facade: Model.update conditional mean on a small stationary field
    g, gi = _sp_grid(sp, 16, 14)
    par = np.array([-0.6, 0.1, 0.2, 0.4, 2.0])
    model = sp.Model(spde="whittle-matern", grid=g, parameters=par, ani=True, ha=False, bc=3)
    model.setModel()
    idx = np.random.default_rng(41).choice(16 * 14, 40, replace=False)
    yobs = np.random.default_rng(42).normal(size=40)
    Q0 = model.Q.copy()
    model.update(yobs, idx)
    np.savez_compressed(os.path.join(OUT, "facade_wm.npz"), par=par, idx=idx, y=yobs, mu=model.mu,
                        tau=model.tau, **_csr(Q0), **dict(gi, bc=3))
    print("facade_wm: mu norm", np.linalg.norm(model.mu))


def facade_cov_case(sp=None):
    """Model.setModel(useCov=True) and two updates on a stationary Whittle-Matern
    field: the covariate form (two sigmas: intercept + scaled covariate, prior
    mean of the covariate coefficient max(cov)) and the intercept-only form (one
    sigma) (reference model.py:120-150)."""
    sp = sp or ref_harness.load_reference()
    M, N = 16, 14
    par = np.array([-0.6, 0.1, 0.2, 0.4, 2.0])
    rng = np.random.default_rng(71)
    cov = 1.0 + rng.uniform(0.0, 2.0, size=M * N)
    idx1 = np.sort(rng.choice(M * N, 30, replace=False))
    idx2 = np.sort(rng.choice(M * N, 25, replace=False))
    y1 = rng.normal(size=30) + 2.0
    y2 = rng.normal(size=25) + 2.0
    out = dict(M=M, N=N, par=par, cov=cov, idx1=idx1, idx2=idx2, y1=y1, y2=y2)
    for name, sig in (("cov", np.log(np.array([0.01, 140.0]))), ("int", np.log(0.5))):
        g = sp.grid(x=np.arange(M, dtype=float), y=np.arange(N, dtype=float))
        model = sp.Model(spde="whittle-matern", grid=g, parameters=par, ani=True, ha=False, bc=3)
        model.setModel(mu=cov, sigmas=sig, useCov=True, scale=True)
        out[f"{name}_sigmas"] = np.atleast_1d(sig)
        out[f"{name}_mu0"] = model.mu.copy()
        out[f"{name}_tau"] = float(model.tau)
        model.update(y1, idx1)
        out[f"{name}_mu1"] = model.mu.copy()
        model.update(y2, idx2)
        out[f"{name}_mu2"] = model.mu.copy()
    np.savez_compressed(os.path.join(OUT, "facade_cov.npz"), **out)
    print("facade_cov:", {k: out[k].shape for k in out if k.endswith("_mu2")})


def facade_tau_case(sp=None):
    """Model.update twice with different noise precisions: plain, and with the
    covariate + intercept fixed effects (reference model.py:120-150)."""
    sp = sp or ref_harness.load_reference()
    M, N = 16, 14
    par = np.array([-0.6, 0.1, 0.2, 0.4, 2.0])
    rng = np.random.default_rng(81)
    cov = 1.0 + rng.uniform(0.0, 2.0, size=M * N)
    idx1 = np.sort(rng.choice(M * N, 30, replace=False))
    idx2 = np.sort(rng.choice(M * N, 25, replace=False))
    y1 = rng.normal(size=30) + 2.0
    y2 = rng.normal(size=25) + 2.0
    tau1, tau2 = 20.0, 3.5
    out = dict(M=M, N=N, par=par, cov=cov, idx1=idx1, idx2=idx2, y1=y1, y2=y2, tau1=tau1, tau2=tau2)
    for name in ("plain", "cov"):
        g = sp.grid(x=np.arange(M, dtype=float), y=np.arange(N, dtype=float))
        model = sp.Model(spde="whittle-matern", grid=g, parameters=par, ani=True, ha=False, bc=3)
        if name == "cov":
            model.setModel(mu=cov, sigmas=np.log(np.array([0.01, 140.0])), useCov=True, scale=True)
        else:
            model.setModel()
        model.update(y1, idx1, tau=tau1)
        out[f"{name}_mu1"] = model.mu.copy()
        model.update(y2, idx2, tau=tau2)
        out[f"{name}_mu2"] = model.mu.copy()
        if name == "plain":
            out.update({f"plain_{k}": v for k, v in _csr(model.Q).items()})
    np.savez_compressed(os.path.join(OUT, "facade_tau.npz"), **out)
    print("facade_tau:", {k: float(np.linalg.norm(out[k])) for k in out if k.endswith("_mu2")})


def optim_objective(x):
    """A smooth, anisotropic objective with its gradient (no reference code)."""
    a = np.array([1.0, 3.0, 0.5, 2.0, 0.25])
    c = np.array([0.3, -0.7, 1.1, 0.0, -1.5])
    d = x - c
    f = float(np.sum(a * d ** 2) + 0.1 * np.sum(d ** 4) + 0.05 * np.sum(np.sin(x)))
    g = 2 * a * d + 0.4 * d ** 3 + 0.05 * np.cos(x)
    return f, g


# The reference's fit reads the step's learning rate from a schedule only (a
# scalar lr leaves it unset), so every run passes one.
OPTIM_RUNS = [
    ("adam", dict(lr=[0.05] * 40, pol=10)),
    ("adam", dict(lr=list(np.linspace(0.2, 0.01, 30)), pol=5, beta1=0.8, beta2=0.99)),
    ("rmsprop", dict(lr=[0.02] * 40, pol=10)),
    ("rmsprop", dict(lr=[0.02] * 30, pol=3, decay=0.5, memory=0.7)),
    ("sgd", dict(lr=[0.01] * 40, pol=10)),
    ("sgd", dict(lr=[0.02] * 25, pol=4, decay=0.3, fix=[1, 3])),
    ("adagrad", dict(lr=[0.3] * 40, pol=10)),
    ("adadelta", dict(lr=[1.0] * 40, pol=10)),
    ("adadelta", dict(lr=[1.0] * 30, pol=6, rho=0.8, epsilon=1e-4)),
]


def optim_cases():
    """Optimize.fit of the reference on optim_objective for each step rule."""
    ref_harness.load_reference()
    import importlib
    ropt = importlib.import_module("spdepy.optim")
    import io
    import contextlib
    out = {"nruns": len(OPTIM_RUNS)}
    x0 = np.array([1.0, 1.0, -1.0, 0.5, 0.0])
    for i, (step, kw) in enumerate(OPTIM_RUNS):
        opt = ropt.Optimize(fun=optim_objective)
        kw = dict(kw)
        if "lr" in kw and isinstance(kw["lr"], list):
            kw["lr"] = np.array(kw["lr"])
        if "fix" in kw:
            kw["fix"] = np.array(kw["fix"])
        if step == "sgd":
            # the reference's SGD lacks the printInit that Optimize.fit calls, so
            # its step object drives the same loop here (fit's body, line for
            # line: evaluate, step with the scheduled rate, restore fixed entries)
            sgd = ropt.SGD()
            sgd.settings(**kw)
            x = x0.copy()
            histX, histF = [], []
            for lr in kw["lr"]:
                f, g = optim_objective(x)
                histF.append(f)
                keep = x[kw["fix"]] if "fix" in kw else None
                x = sgd(x, f, g, lr)
                if keep is not None:
                    x[kw["fix"]] = keep
                histX.append(x)
            res = {"x": np.array(histX).T[:, -kw["pol"]:].mean(axis=1), "fun": f}
            opt.histX, opt.histF = histX, histF
        else:
            with contextlib.redirect_stdout(io.StringIO()):
                res = opt.fit(x0=x0.copy(), stepType=step, **kw)
        out[f"r{i}_step"] = np.array(step)
        out[f"r{i}_x"] = np.asarray(res["x"], dtype=float)
        out[f"r{i}_fun"] = np.array(res["fun"], dtype=float)
        out[f"r{i}_hist"] = np.array(opt.histX, dtype=float)
        out[f"r{i}_histf"] = np.array(opt.histF, dtype=float)
    out["x0"] = x0
    np.savez_compressed(os.path.join(OUT, "optim.npz"), **out)
    print("optim:", {k: out[k].tolist() for k in out if k.endswith("_fun")})


def plumbing_cases(sp=None):
    """Face velocities and bases on extended grids, and two model objects on a
    grid extended by two cells (reference grids/spat2Dtemp_regular_mesh.py:
    102-117 extend, 157-275 bases, 277-391 assimilate_adv / advBound)."""
    sp = sp or ref_harness.load_reference()
    M, N, T = 9, 7, 3
    rng = np.random.default_rng(91)
    we = rng.normal(size=M * N)
    wn = rng.normal(size=M * N)
    par_adv = 0.3 * rng.normal(size=18)
    out = dict(M=M, N=N, T=T, we=we, wn=wn, par_adv=par_adv)
    for ext in (0, 1, 2, 3):
        g = sp.grid(x=np.arange(M, dtype=float), y=np.arange(N, dtype=float), t=np.arange(T, dtype=float),
                    extend=ext if ext else None)
        out[f"ww_e{ext}"] = g.assimilate_adv(we, wn)
        out[f"adv_e{ext}"] = g.evalAdv(par_adv)
        out[f"bs_e{ext}"] = g.bs
        out[f"bsH_e{ext}"] = g.bsH
    np.savez_compressed(os.path.join(OUT, "grid_adv.npz"), **out)
    print("grid_adv:", {k: out[k].shape for k in out if k.startswith("ww_")})

    from spdepy.spdes.cov_advection_var_diffusion2D import CovAdvectionVarDiffusion2D
    M, N, T = 9, 8, 4
    g, gi = _st_grid(sp, M, N, T, extend=2)
    rng = np.random.default_rng(92)
    ww = _smooth_ww(g, seed=93)
    par = np.hstack([np.log(0.4) + 0.1 * rng.normal(size=9), np.log(0.6) + 0.1 * rng.normal(size=9),
                     0.3 * rng.normal(size=9), 0.3 * rng.normal(size=9), 0.8, 0.1,
                     np.log(0.4), np.log(0.6), 0.3, 0.0, np.log(100.0)])
    mod0 = sp.spde_init(model="whittle-matern", grid=sp.grid(x=np.arange(M, dtype=float),
                        y=np.arange(N, dtype=float), extend=2), ani=True, ha=False, bc=3)
    mod = CovAdvectionVarDiffusion2D(grid=g, mod0=mod0, par=par, bc=3, ww=ww)
    mod.setQ(par)
    idx = np.random.default_rng(94).choice(M * N * T, 100, replace=False)
    _model_case("covadv_vardiff_bc3_ext2", mod, par, idx, 0.1,
                dict(gi, bc=3, family="cov-advection-var-diffusion", ani=1, ha=0), extra=dict(ww=ww))

    M, N, T = 8, 8, 4
    g, gi = _st_grid(sp, M, N, T, extend=2)
    rng = np.random.default_rng(95)
    par = np.hstack([np.log(0.4) + 0.1 * rng.normal(size=9), np.log(0.6) + 0.1 * rng.normal(size=9),
                     0.3 * rng.normal(size=9), 0.3 * rng.normal(size=9), 0.2 * rng.normal(size=9),
                     0.2 * rng.normal(size=9), 0.1, np.log(0.4), np.log(0.6), 0.3, 0.0, np.log(100.0)])
    mod0 = sp.spde_init(model="whittle-matern", grid=sp.grid(x=np.arange(M, dtype=float),
                        y=np.arange(N, dtype=float), extend=2), ani=True, ha=False, bc=3)
    mod = sp.spde_init(model="var-advection-var-diffusion", grid=g, parameters=par, ani=True, ha=False, bc=3,
                       mod0=mod0)
    idx = np.random.default_rng(96).choice(M * N * T, 90, replace=False)
    _model_case("varadv_vardiff_bc3_ext2", mod, par, idx, 0.1,
                dict(gi, bc=3, family="var-advection-var-diffusion", ani=1, ha=0))


def getS_cases(sp=None):
    """Grid.getS with fixed-effect columns on a padded space-time grid."""
    sp = sp or ref_harness.load_reference()
    M, N, T, ext = 6, 5, 3, 1
    rng = np.random.default_rng(61)
    cov = rng.uniform(0.5, 3.0, size=M * N * T)
    idx = np.sort(rng.choice(M * N * T, 25, replace=False))
    out = dict(M=M, N=N, T=T, extend=ext, cov=cov, idx=idx)
    variants = {"plain": None, "int": "int", "cov_int": (True, False), "cov_int_scale": (True, True),
                "cov": (False, False)}
    for name, how in variants.items():
        g = sp.grid(x=np.arange(M, dtype=float), y=np.arange(N, dtype=float), t=np.arange(T, dtype=float),
                    extend=ext)
        if how == "int":
            g.addInt()
        elif how is not None:
            g.addCov(cov, inter=how[0], scale=how[1])
        for tag, ii in (("sub", idx), ("all", None)):
            S = sparse.csr_matrix(g.getS(ii))
            S.sort_indices()
            out[f"{name}_{tag}_data"] = S.data
            out[f"{name}_{tag}_indices"] = S.indices.astype(np.int32)
            out[f"{name}_{tag}_indptr"] = S.indptr.astype(np.int64)
            out[f"{name}_{tag}_shape"] = np.array(S.shape, np.int64)
    np.savez_compressed(os.path.join(OUT, "grid_getS.npz"), **out)
    print("grid_getS:", {k: tuple(out[k]) for k in out if k.endswith("_all_shape")})


def separable_cases(sp=None, only=None):
    """Separable space-time fixtures: the rho form (anisotropic, bc 1 and 3) and
    the (a, sigma) form (isotropic and half-angle; those reference classes need
    T = 10).  `only`: names to (re)generate, all when None."""
    sp = sp or ref_harness.load_reference()
    from spdepy.spdes.seperable_spatial_temporal2D import SeperableSpatialTemporal2D
    from spdepy.spdes.seperable_spatial_temporal_ha2D import SeperableSpatialTemporalHa2D
    from spdepy.spdes.seperable_spatial_temporal_idiffusion2D import SeperableSpatialTemporalIDiffusion2D
    want = (lambda name: only is None or name in only)
    for bc in (1, 3):
        if not want(f"ani_bc{bc}"):
            continue
        M, N, T = 10, 9, 5
        g, gi = _st_grid(sp, M, N, T)
        rng = np.random.default_rng(50 + bc)
        par = np.hstack([np.log(0.5) + 0.1 * rng.normal(size=9), np.log(0.6) + 0.1 * rng.normal(size=9),
                         0.3 * rng.normal(size=9), 0.3 * rng.normal(size=9), np.log(0.6), np.log(100.0)])
        mod = SeperableSpatialTemporal2D(grid=g, par=par, bc=bc)
        idx = np.random.default_rng(53 + bc).choice(M * N * T, 120, replace=False)
        _model_case(f"ani_bc{bc}", mod, par, idx, 0.1,
                    dict(gi, bc=bc, family="seperable-spatial-temporal", ani=1, ha=0, temporal="rho"),
                    prefix="separable")
    if want("ha_bc1"):
        M, N, T = 8, 7, 10
        g, gi = _st_grid(sp, M, N, T)
        rng = np.random.default_rng(59)
        par = np.hstack([np.log(0.5) + 0.1 * rng.normal(size=9), np.log(0.6) + 0.1 * rng.normal(size=9),
                         0.3 * rng.normal(size=9), 0.3 * rng.normal(size=9), 0.4, np.log(1.5), np.log(100.0)])
        mod = SeperableSpatialTemporalHa2D(grid=g, par=par, bc=1)
        idx = np.random.default_rng(60).choice(M * N * T, 110, replace=False)
        _model_case("ha_bc1", mod, par, idx, 0.1,
                    dict(gi, bc=1, family="seperable-spatial-temporal", ani=1, ha=1, temporal="a-sigma"),
                    prefix="separable")
    if not want("iso_bc3"):
        return
    M, N, T = 8, 7, 10
    g, gi = _st_grid(sp, M, N, T)
    rng = np.random.default_rng(57)
    par = np.hstack([np.log(0.5) + 0.1 * rng.normal(size=9), np.log(0.6) + 0.1 * rng.normal(size=9), 0.5,
                     np.log(2.0), np.log(100.0)])
    mod = SeperableSpatialTemporalIDiffusion2D(grid=g, par=par, bc=3)
    idx = np.random.default_rng(58).choice(M * N * T, 110, replace=False)
    _model_case("iso_bc3", mod, par, idx, 0.1,
                dict(gi, bc=3, family="seperable-spatial-temporal", ani=0, ha=0, temporal="a-sigma"),
                prefix="separable")


if __name__ == "__main__":
    if len(sys.argv) > 2 and sys.argv[1] == "--only" and sys.argv[2] == "separable":
        separable_cases(only=sys.argv[3:] or None)
    elif len(sys.argv) > 2 and sys.argv[1] == "--only" and sys.argv[2] == "getS":
        getS_cases()
    elif len(sys.argv) > 2 and sys.argv[1] == "--only" and sys.argv[2] == "facade_cov":
        facade_cov_case()
    elif len(sys.argv) > 2 and sys.argv[1] == "--only" and sys.argv[2] == "facade_tau":
        facade_tau_case()
    elif len(sys.argv) > 2 and sys.argv[1] == "--only" and sys.argv[2] == "plumbing":
        plumbing_cases()
    elif len(sys.argv) > 2 and sys.argv[1] == "--only" and sys.argv[2] == "optim":
        optim_cases()
    else:
        main()
        separable_cases()
        getS_cases()
        facade_cov_case()
        facade_tau_case()
        plumbing_cases()
        optim_cases()
