"""Failure detection on the GPU path, made on the host side (no kernel is made to
fault): invalid parameters, a matrix that is not positive definite, a PCG that
runs out of iterations.  Each must come back as the C ABI's status code and the
Python error the reference raises in the same place (CHOLMOD's
CholmodNotPositiveDefiniteError for a non-SPD factorisation), and leave the
plan usable for the next call."""
import numpy as np
import pytest

from golden_cases import load
from gpu_cases import gpu_model

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _cuda():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from spdepy_gb300 import build
    build.build()


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_nan_parameter_is_an_argument_error(precision):
    from spdepy_gb300 import _native as nat
    g = load("advdiff_ani_bc3")
    mod = gpu_model(g, precision)
    par = np.array(g["par"], float)
    bad = par.copy()
    bad[1] = np.nan
    with pytest.raises(nat.SpdeError, match="invalid argument.*non-finite"):
        mod.logLike(bad, grad=True)
    canon = mod.canonical(bad)
    assert nat.lib().spde_assemble(mod.plan.h, canon.ctypes.data, canon.size) == 1
    f = mod.logLike(par, grad=False)  # the plan still works
    assert abs(f - float(g["f"])) <= 1e-6 * abs(float(g["f"]))


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_indefinite_matrix_raises_not_positive_definite(precision):
    """Q + tau S^T S with a large negative tau has negative diagonal entries: the
    factorisation reports SPDE_ERR_NOT_SPD, which the Python layer raises as
    NotPositiveDefiniteError, and the next factorisation succeeds."""
    import ctypes
    from spdepy_gb300 import _native as nat
    g = load("advdiff_ani_bc3")
    mod = gpu_model(g, precision)
    mod._assemble(g["par"])
    plan = mod.plan
    plan.set_obs(mod.grid.obs_nodes(g["idx"]))
    ld = ctypes.c_double()
    assert nat.lib().spde_factor(plan.h, 1, -1e6, ctypes.byref(ld)) == 3
    assert b"not positive definite" in nat.lib().spde_last_error(plan.h)
    with pytest.raises(nat.NotPositiveDefiniteError):
        plan.factor(True, -1e6)
    ld_ok = plan.factor(True, 400.0)
    assert np.isfinite(ld_ok)


def test_pcg_iteration_cap_reports_not_converged():
    """PCG that reaches maxit before the tolerance returns SPDE_ERR_NOT_CONVERGED
    with the iterations run and the residual reached."""
    import ctypes
    from spdepy_gb300 import _native as nat
    g = load("advdiff_ani_bc3")
    mod = gpu_model(g, "fp64")
    mod._assemble(g["par"])
    plan = mod.plan
    n = mod.grid.n
    b = torch.randn(n, dtype=torch.float64, generator=torch.Generator().manual_seed(0)).cuda()
    x = torch.empty_like(b)
    it, rel = ctypes.c_int(), ctypes.c_double()
    rc = nat.lib().spde_pcg(plan.h, 0, 0.0, 1, None, b.data_ptr(), x.data_ptr(), 1, 1e-12, 3, ctypes.byref(it),
                            ctypes.byref(rel))
    assert rc == 6
    assert it.value == 3 and rel.value > 1e-12
    with pytest.raises(nat.SpdeError, match="not converged"):
        plan.pcg(b, precond="jacobi", tol=1e-12, maxit=3, check=True)
    x2, its, rel2 = plan.pcg(b, precond="jacobi", tol=1e-8, maxit=5000)
    assert rel2 <= 1e-8


def test_bad_observation_index_and_weights():
    from spdepy_gb300 import _native as nat
    g = load("advdiff_ani_bc3")
    mod = gpu_model(g, "fp64")
    plan = mod.plan
    n = mod.grid.n
    with pytest.raises(nat.SpdeError, match="out of range"):
        plan.set_obs(np.array([0, n], dtype=np.int64))
    plan._obs = None
    with pytest.raises(nat.SpdeError, match="finite and non-negative"):
        plan.set_obs(np.array([0, 1], dtype=np.int64), weights=np.array([1.0, -2.0]))
    plan._obs = None
    plan.set_obs(np.array([0, 1], dtype=np.int64), weights=np.array([1.0, 2.0]))


def test_tensor_core_wait_limit_returns_an_error_and_the_plan_recovers():
    """Every wait inside the tensor-core kernels (single-CTA and cluster-pair) is
    bounded.  With the limit lowered to 1 ns the waits run out: each CTA records
    the error, waits for its issued tensor-core work (with the normal limit),
    frees its tensor memory and returns; the factorisation reports SPDE_ERR_CUDA,
    and with the default limit restored the same plan factors to the same
    log-determinant as before."""
    import ctypes
    from spdepy_gb300 import _native as nat
    from spdepy_gb300.workloads import build_model, nonstationary_advection_diffusion
    w = nonstationary_advection_diffusion(M=48, N=48, T=12)
    mod = build_model(w, "mixed")
    mod._assemble(w.par)
    plan = mod.plan
    L = nat.lib()
    ld0 = plan.factor(False, 0.0)
    prof = np.zeros(10, dtype=np.int64)
    L.spde_plan_read_profile(plan.h, None, None, None, 1)
    nat.check(L.spde_plan_set_profiling(plan.h, 2), plan.h)
    nat.check(L.spde_plan_set_wait_limit(plan.h, 1), plan.h)
    ld = ctypes.c_double()
    try:
        rc = L.spde_factor(plan.h, 0, 0.0, ctypes.byref(ld))
    finally:
        nat.check(L.spde_plan_set_wait_limit(plan.h, 0), plan.h)
        L.spde_plan_read_profile(plan.h, None, None, prof.ctypes.data, 1)
        L.spde_plan_set_profiling(plan.h, 0)
    assert prof[9] > 0  # tensor-core products ran (and gave up)
    assert rc == 2
    assert b"timed out" in L.spde_last_error(plan.h)
    with pytest.raises(nat.SpdeError):
        plan.solve(torch.zeros(w.grid.n, dtype=torch.float64))  # no valid factor
    ld1 = plan.factor(False, 0.0)
    assert ld1 == ld0


def test_sweep_wait_limit_returns_an_error_and_the_plan_recovers():
    """The one-right-hand-side sweeps wait on per-block completion flags with the
    plan's wait limit.  With the limit lowered to 1 ns the waits give up, the
    solve reports a timed-out sweep, and with the default limit restored the
    same factor solves to the refinement tolerance."""
    from spdepy_gb300 import _native as nat
    from spdepy_gb300.workloads import build_model, nonstationary_advection_diffusion
    w = nonstationary_advection_diffusion(M=48, N=48, T=12)
    mod = build_model(w, "mixed")
    mod._assemble(w.par)
    plan = mod.plan
    plan.factor(False, 0.0)
    L = nat.lib()
    b = torch.randn(w.grid.n, dtype=torch.float64, generator=torch.Generator().manual_seed(3))
    nat.check(L.spde_plan_set_wait_limit(plan.h, 1), plan.h)
    try:
        with pytest.raises(nat.SpdeError, match="timed out"):
            plan.solve(b, refine=0)
    finally:
        nat.check(L.spde_plan_set_wait_limit(plan.h, 0), plan.h)
    x, res = plan.solve(b, refine=10, tol=1e-12)
    assert res < 1e-10
    assert torch.allclose(plan.spmv(x).cpu(), b, rtol=0, atol=1e-9 * b.abs().max())
