"""The tensor-core path against the oracle at a size where it runs.

The reference fixtures are at most 1,600 nodes, where no front reaches the
tensor-core product (k >= 128).  Here the benchmark's own generator (the
non-stationary advection-diffusion model of
spdes/cov_advection_var_diffusion2D.py:87-121, Nbs = 5, a lambda-scaled Fourier
velocity) runs at 30 x 30 x 24 (21,600 nodes): the top separators are ~1,400
columns wide, so the mixed plan's Schur updates and inverse products go through
the tcgen05 3xTF32 kernel.  Both plans are compared with the oracle's
logLike (spdes/cov_advection_var_diffusion2D.py:187-223; SuperLU stands in for
CHOLMOD) on the same inputs: the objective, and the reference's Hutchinson
gradient with the same seeded probes.
"""
import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

M, N, T = 30, 30, 24
NH1 = 16
SEED_V = 3
TOL_F = {"fp64": 1e-10, "mixed": 1e-6}
# Hutchinson gradient: its solves are refined in FP64 to 1e-10 relative residual
# on both plans, so the two agree with the oracle far below the estimator's own noise
TOL_G = {"fp64": 1e-8, "mixed": 1e-7}


@pytest.fixture(scope="module")
def case():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from oracle.spde_oracle import OracleGrid, OracleModel
    from spdepy_gb300 import build
    from spdepy_gb300.workloads import fourier_velocity, nonstationary_advection_diffusion
    build.build()
    w = nonstationary_advection_diffusion(M=M, N=N, T=T)
    w.y = np.random.default_rng(0).normal(size=w.idx.size)
    og = OracleGrid(np.arange(float(M)), np.arange(float(N)), np.arange(float(T)), None, 5)
    ww = og.assimilate_adv(*fourier_velocity(M, N, seed=1))
    assert np.array_equal(ww, w.ww)
    om = OracleModel(og, "cov-advection-var-diffusion", "ani", w.bc, ww=ww)
    f0, j0 = om.loglike(w.par, w.y, w.idx, grad=True, nh1=NH1, seed=SEED_V)
    return w, f0, j0


def _model(w, precision):
    from spdepy_gb300.workloads import build_model
    mod = build_model(w, precision)
    mod.initFit(w.y, idx=w.idx)
    return mod


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_objective_vs_oracle(case, precision):
    from spdepy_gb300 import _native as nat
    w, f0, _ = case
    mod = _model(w, precision)
    info = mod.plan.info()
    assert info.max_front >= 1024
    L = nat.lib()
    L.spde_plan_read_profile(mod.plan.h, None, None, None, 1)
    nat.check(L.spde_plan_set_profiling(mod.plan.h, 2), mod.plan.h)
    try:
        f = mod.logLike(w.par, grad=False)
    finally:
        cnt = np.zeros(10, dtype=np.int64)
        L.spde_plan_read_profile(mod.plan.h, None, None, cnt.ctypes.data, 1)
        L.spde_plan_set_profiling(mod.plan.h, 0)
    assert abs(f - f0) <= TOL_F[precision] * abs(f0), (f, f0, abs(f - f0) / abs(f0))
    if precision == "mixed":
        assert cnt[9] > 0, "no tensor-core product ran"
    else:
        assert cnt[9] == 0


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_hutchinson_gradient_vs_oracle(case, precision):
    w, f0, j0 = case
    mod = _model(w, precision)
    np.random.seed(SEED_V)
    f, jac = mod.logLike(w.par, nh1=NH1, grad=True, grad_mode="hutchinson")
    assert abs(f - f0) <= TOL_F[precision] * abs(f0)
    scale = np.abs(j0).max()
    err = np.abs(jac - j0).max() / scale
    assert err <= TOL_G[precision], err
