"""GPU parity: every step of the hot path through the C ABI against the
reference's golden fixtures and the oracle (FP64 restatement)."""
import ctypes

import numpy as np
import pytest
from scipy import sparse

from golden_cases import load, model_cases, oracle_model
from gpu_cases import gpu_model

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

# tolerances: FP64 path is pinned to rounding; the mixed path (FP32 factor with
# FP64 pivots and FP64 iterative refinement) to 1e-6 relative, the mixed plan's accuracy bound
TOL_F = {"fp64": 1e-11, "mixed": 1e-6}
TOL_G = {"fp64": 1e-8, "mixed": 1e-4}


@pytest.fixture(scope="module", autouse=True)
def _cuda():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from spdepy_gb300 import build
    build.build()


def test_triplets_bit_exact():
    from spdepy_gb300 import _native as nat
    g = load("stencils.npz")
    M, N, hx, hy = int(g["M"]), int(g["N"]), float(g["hx"]), float(g["hy"])
    L = nat.lib()
    for bc in (1, 3):
        for fam, field in (("AcH", 0), ("AH", 1)):
            H = torch.as_tensor(g["H"] if field else g["Hc"]).cuda().contiguous()
            row = torch.empty(9 * M * N, dtype=torch.int32, device="cuda")
            col = torch.empty_like(row)
            val = torch.empty(9 * M * N, dtype=torch.float64, device="cuda")
            nat.check(L.spde_diffusion_triplets(M, N, H.data_ptr(), field, hx, hy, bc, row.data_ptr(), col.data_ptr(),
                                                val.data_ptr(), None))
            torch.cuda.synchronize()
            k = f"{fam}_b{bc}"
            assert np.array_equal(row.cpu().numpy(), g[k + "_row"])
            assert np.array_equal(col.cpu().numpy(), g[k + "_col"])
            assert np.array_equal(val.cpu().numpy(), g[k + "_val"])
        for fam, field in (("Acw", 0), ("Aw", 1)):
            for diff in (1, 2, 3):
                G = torch.as_tensor(g["G"] if field else g["Gc"]).cuda().contiguous()
                dG = torch.as_tensor(g["dG"]).cuda().contiguous()
                row = torch.empty(5 * M * N, dtype=torch.int32, device="cuda")
                col = torch.empty_like(row)
                val = torch.empty(5 * M * N, dtype=torch.float64, device="cuda")
                nat.check(L.spde_advection_triplets(M, N, G.data_ptr(), dG.data_ptr() if field else None, field, hx, hy,
                                                    bc, diff, row.data_ptr(), col.data_ptr(), val.data_ptr(), None))
                torch.cuda.synchronize()
                k = f"{fam}_b{bc}_d{diff}"
                assert np.array_equal(row.cpu().numpy(), g[k + "_row"])
                assert np.array_equal(col.cpu().numpy(), g[k + "_col"])
                assert np.array_equal(val.cpu().numpy(), g[k + "_val"], equal_nan=True)


@pytest.mark.parametrize("name", model_cases())
def test_q_assembly(name):
    g = load(name)
    mod = gpu_model(g)
    Q = mod.makeQ(g["par"])[0].to_scipy()
    Qg = sparse.csr_matrix((g["Q_data"], g["Q_indices"], g["Q_indptr"]), shape=Q.shape)
    assert abs(Q - Qg).max() <= 1e-12 * abs(Qg).max()


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
@pytest.mark.parametrize("name", model_cases())
def test_loglike_value(name, precision):
    g = load(name)
    mod = gpu_model(g, precision)
    f = mod.logLike(g["par"], grad=False)
    assert abs(f - float(g["f"])) <= TOL_F[precision] * max(1.0, abs(float(g["f"])))


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
@pytest.mark.parametrize("name", model_cases())
def test_exact_gradient_vs_oracle(name, precision):
    g = load(name)
    om = oracle_model(g)
    om.derivative = "true"
    f0, jex = om.loglike(g["par"], g["y"], g["idx"], grad=True, exact=True)
    mod = gpu_model(g, precision)
    f, jac = mod.logLike(g["par"], grad=True)
    assert abs(f - f0) <= TOL_F[precision] * max(1.0, abs(f0))
    scale = np.abs(jex).max()
    assert np.allclose(jac, jex, rtol=TOL_G[precision], atol=TOL_G[precision] * scale), np.abs(jac - jex).max() / scale


@pytest.mark.parametrize("name", model_cases())
def test_hutchinson_replica(name):
    """Same probes as the reference (np.random seeded), same estimator."""
    g = load(name)
    mod = gpu_model(g, "fp64")
    np.random.seed(int(g["seed_v"]))
    f, jac = mod.logLike(g["par"], nh1=int(g["nh1"]), grad=True, grad_mode="hutchinson")
    om = oracle_model(g)
    om.derivative = "true"
    f0, jref = om.loglike(g["par"], g["y"], g["idx"], grad=True, nh1=int(g["nh1"]), seed=int(g["seed_v"]))
    assert abs(f - float(g["f"])) <= 1e-11 * max(1.0, abs(float(g["f"])))
    scale = np.abs(jref).max()
    assert np.allclose(jac, jref, rtol=1e-8, atol=1e-9 * scale)
    # where the reference's derivative stencils are exact derivatives, equal to its own output;
    # with bc = 1 its velocity derivatives are not (constant velocity: the boundary term
    # keeps -|w|h/2; B-spline velocity: G/|G| = NaN on zeroed faces drops the other face)
    quirk = int(g["bc"]) == 1 and str(g["family"]) in ("advection-diffusion", "advection-var-diffusion",
                                                         "var-advection-diffusion", "var-advection-var-diffusion")
    if not quirk:
        assert np.allclose(jac, g["jac"], rtol=1e-8, atol=1e-9 * scale)


def test_solve_refinement_and_sample_identity():
    g = load("advdiff_ani_bc3")
    for precision in ("fp64", "mixed"):
        mod = gpu_model(g, precision)
        mod._assemble(g["par"])
        plan = mod.plan
        plan.factor(False, 0.0)
        n = mod.grid.n
        b = torch.randn(n, 5, dtype=torch.float64, generator=torch.Generator().manual_seed(0))
        x, res = plan.solve(b, refine=10, tol=1e-12)
        assert res < 1e-10
        Qb = plan.spmv(x)
        assert torch.allclose(Qb.cpu(), b, rtol=0, atol=1e-9 * b.abs().max())
        z = torch.randn(n, 4, dtype=torch.float64, generator=torch.Generator().manual_seed(1))
        xs = plan.sample(z)
        quad = (xs * plan.spmv(xs)).sum(0).cpu()
        rel = ((quad - (z ** 2).sum(0)).abs() / (z ** 2).sum(0)).max().item()
        assert rel < (1e-10 if precision == "fp64" else 1e-4)


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
@pytest.mark.parametrize("nrhs", [1, 2, 8])
def test_narrow_solves(precision, nrhs):
    """Solves with at most 8 right-hand sides run on the narrow products (the
    one-column kernel for nrhs = 1): Q x = b to the refinement tolerance, and
    each column equals the same solve done alone."""
    g = load("advdiff_ani_bc3")
    mod = gpu_model(g, precision)
    mod._assemble(g["par"])
    plan = mod.plan
    plan.factor(False, 0.0)
    n = mod.grid.n
    b = torch.randn(n, nrhs, dtype=torch.float64, generator=torch.Generator().manual_seed(nrhs))
    x, res = plan.solve(b, refine=10, tol=1e-12)
    assert res < 1e-10
    assert torch.allclose(plan.spmv(x).cpu(), b, rtol=0, atol=1e-9 * b.abs().max())
    x1, _ = plan.solve(b[:, -1:].contiguous(), refine=10, tol=1e-12)
    assert torch.allclose(x[:, -1:].cpu(), x1.cpu(), rtol=0, atol=1e-9 * x1.abs().max().item())


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_selected_inverse_vs_dense(precision):
    g = load("covadv_vardiff_bc1")
    mod = gpu_model(g, precision)
    Q = mod.makeQ(g["par"])[0].to_scipy()
    mod._assemble(g["par"])
    mod.plan.factor(False, 0.0)
    zq = mod.plan.selinv().cpu().numpy()
    Z = np.linalg.inv(Q.toarray())
    from spdepy_gb300.spdes import stencil_to_csr
    Zs = stencil_to_csr(mod.grid, zq)
    mask = (stencil_to_csr(mod.grid, np.ones_like(zq)) != 0).toarray()
    err = np.abs(Zs.toarray() - Z)[mask].max() / np.abs(Z).max()
    assert err < (1e-11 if precision == "fp64" else 1e-4)


def test_facade_update_golden():
    import spdepy_gb300 as sp
    g = load("facade_wm.npz")
    grid = sp.grid(x=np.arange(int(g["M"]), dtype=float), y=np.arange(int(g["N"]), dtype=float))
    m = sp.Model(spde="whittle-matern", grid=grid, parameters=g["par"], ani=True, ha=False, bc=3, precision="fp64")
    m.setModel()
    m.update(g["y"], g["idx"])
    assert np.allclose(m.mu, g["mu"], rtol=1e-10, atol=1e-12)


@pytest.mark.parametrize("name", ["cov", "int"])
def test_facade_fixed_effects_golden(name):
    """Model.setModel(useCov=True) and two updates on the GPU factor, with the
    fixed-effect border eliminated on the host, against the reference's
    augmented Cholesky solves (covariate + intercept, and intercept alone)."""
    import spdepy_gb300 as sp
    g = load("facade_cov.npz")
    M, N = int(g["M"]), int(g["N"])
    grid = sp.grid(x=np.arange(M, dtype=float), y=np.arange(N, dtype=float))
    m = sp.Model(spde="whittle-matern", grid=grid, parameters=g["par"], ani=True, ha=False, bc=3, precision="fp64")
    sig = g["cov_sigmas"] if name == "cov" else float(g["int_sigmas"][0])
    m.setModel(mu=g["cov"], sigmas=sig, useCov=True, scale=True)
    assert np.allclose(m.mu, g[f"{name}_mu0"], rtol=1e-14, atol=0)
    for k in (1, 2):
        m.update(g[f"y{k}"], g[f"idx{k}"])
        ref = g[f"{name}_mu{k}"]
        assert np.allclose(m.mu, ref, rtol=1e-9, atol=1e-11 * np.abs(ref).max()), k
    draws = m.sample(n=8, simple=True, seed=3)
    assert draws.shape == (M * N, 8) and np.isfinite(draws).all()


def test_factor_handle_survives_other_factorisations():
    """makeQ's factor handle (the reference's cholesky(Q)) keeps solving with Q
    after the plan has factored Q + tau S^T S and run a log-likelihood, and
    apply_Pt(solve_Lt(z)) draws from N(0, Q^-1) as the reference's sampler does."""
    g = load("advdiff_ani_bc3")
    mod = gpu_model(g, "fp64")
    Q, fac, _ = mod.makeQ(g["par"])
    b = np.random.default_rng(1).normal(size=mod.grid.n)
    x0 = fac.solve_A(b)
    mod.logLike(g["par"], grad=True)          # refactors and inverts internally
    mod.plan.factor(True, 25.0)
    x1 = fac.solve_A(b)
    np.testing.assert_allclose(x1, x0, rtol=1e-12, atol=1e-12 * np.abs(x0).max())
    Qs = Q.to_scipy()
    np.testing.assert_allclose(Qs @ x1, b, rtol=0, atol=1e-9 * np.abs(b).max())
    z = np.random.default_rng(2).normal(size=(mod.grid.n, 2000))
    xs = fac.apply_Pt(fac.solve_Lt(z))
    # E[x x^T] = Q^-1: check the quadratic form of the empirical covariance
    v = np.random.default_rng(3).normal(size=mod.grid.n)
    emp = np.mean((v @ xs) ** 2)
    assert emp == pytest.approx(v @ fac.solve_A(v), rel=0.15)


@pytest.mark.parametrize("M,N,T,leaf", [(7, 5, 3, 16), (33, 17, 9, 64), (41, 29, 6, 128)])
def test_device_ordering_on_odd_lattices(M, N, T, leaf):
    """The plan's permutation comes from the device nested-dissection kernel and
    is checked against the symbolic analysis when the plan is built; on lattices
    with odd extents and small leaves the factor then solves Q x = b to the
    refinement tolerance through that permutation, in both precisions."""
    from spdepy_gb300.spdes import GPUPlan
    from spdepy_gb300.workloads import build_model, nonstationary_advection_diffusion
    w = nonstationary_advection_diffusion(M=M, N=N, T=T)
    for precision in ("fp64", "mixed"):
        mod = build_model(w, precision)
        mod._plan = GPUPlan(w.grid, precision, leaf)
        mod._model_key = None
        mod._assemble(w.par)
        plan = mod.plan
        assert plan.info().n == M * N * T
        plan.factor(False, 0.0)
        b = torch.randn(w.grid.n, 2, dtype=torch.float64, generator=torch.Generator().manual_seed(M))
        for rhs in (b[:, :1].contiguous(), b):
            x, res = plan.solve(rhs, refine=10, tol=1e-12)
            assert res < 1e-10, (precision, rhs.shape, res)
            assert torch.allclose(plan.spmv(x).cpu(), rhs, rtol=0, atol=1e-9 * rhs.abs().max())
