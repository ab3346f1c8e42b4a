"""The benchmarked workload at full size, where the oracle cannot run: the
non-stationary advection-diffusion model of
spdes/cov_advection_var_diffusion2D.py:87-121 on 200 x 200 x 24 (960,000 nodes,
1 % observed, data simulated at the generating parameters), mixed plan.  The
checks are properties that hold at any size:

- repeated evaluations give bit-identical objectives and gradients;
- the conditional mean solves (Q + tau S^T S) mu = tau S^T y, checked with the
  FP64 stencil product;
- x = P L^-T z satisfies x^T Q x = z^T z (the sampling identity);
- the selected inverse's diagonal equals e_i^T A^-1 e_i from refined solves;
- the exact gradient equals the central difference of the objective along the
  gradient direction.
"""
import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

M, N, T = 200, 200, 24
DIAG_SLOT = 21  # (0, 0, 0) in the 43-slot layout: 9 slots at dt = -1, then (dx, dy) over -2..2


@pytest.fixture(scope="module")
def full():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from spdepy_gb300 import build
    from spdepy_gb300.workloads import build_model, nonstationary_advection_diffusion, simulate
    build.build()
    w = nonstationary_advection_diffusion(M=M, N=N, T=T)
    mod = build_model(w, "mixed")
    simulate(mod, w)
    mod.initFit(w.y, idx=w.idx)
    return w, mod


def test_repeated_evaluations_are_identical(full):
    w, mod = full
    f1, j1 = mod.logLike(w.par, grad=True)
    f2, j2 = mod.logLike(w.par, grad=True)
    assert np.isfinite(f1) and np.isfinite(j1).all()
    assert f1 == f2
    assert np.array_equal(j1, j2)


def test_conditional_mean_residual(full):
    w, mod = full
    plan = mod.plan
    mod._assemble(w.par)
    tau = float(np.exp(w.par[-1]))
    nodes = w.grid.obs_nodes(w.idx)
    plan.set_obs(nodes)
    plan.factor(True, tau)
    b = torch.zeros(w.grid.n, dtype=torch.float64)
    b.index_add_(0, torch.as_tensor(nodes), torch.as_tensor(tau * w.y))
    mu, res = plan.solve(b, refine=10, tol=1e-12)
    assert res < 1e-10
    r = plan.spmv(mu, with_obs=True, tau=tau).cpu() - b
    assert (r.norm() / b.norm()).item() < 1e-10


def test_sampling_identity(full):
    w, mod = full
    plan = mod.plan
    mod._assemble(w.par)
    plan.factor(False, 0.0)
    z = torch.randn(w.grid.n, 8, dtype=torch.float64, generator=torch.Generator().manual_seed(5))
    x = plan.sample(z)
    quad = (x * plan.spmv(x)).sum(0).cpu()
    zz = (z ** 2).sum(0)
    rel = ((quad - zz).abs() / zz).max().item()
    assert rel < 1e-4, rel  # the FP32 factor's error, as on the small fixtures


def test_selected_inverse_diagonal_vs_solves(full):
    w, mod = full
    plan = mod.plan
    mod._assemble(w.par)
    plan.factor(False, 0.0)
    rng = np.random.default_rng(11)
    picks = np.concatenate([[0, w.grid.n - 1], rng.choice(w.grid.n, 6, replace=False)])
    E = torch.zeros(w.grid.n, picks.size, dtype=torch.float64)
    E[torch.as_tensor(picks), torch.arange(picks.size)] = 1.0
    X, res = plan.solve(E, refine=10, tol=1e-12)
    assert res < 1e-10
    ref = X.cpu()[torch.as_tensor(picks), torch.arange(picks.size)].numpy()
    zq = plan.selinv().cpu().numpy()
    got = zq[picks, DIAG_SLOT]
    rel = np.abs(got / ref - 1).max()
    assert rel < 1e-4, rel  # selected inverse from the FP32 factor; the solves are refined in FP64


def test_gradient_vs_central_difference_along_gradient(full):
    """Central difference with h = 1e-2 along d = jac / |jac|.  The mixed
    objective's rounding error (about 4e-7 relative to |f| < 1) contributes at
    most 4e-5 / |jac| and the h^2 truncation about 2e-5 relative."""
    w, mod = full
    par = np.array(w.par, float)
    f0, jac = mod.logLike(par, grad=True)
    g = np.linalg.norm(jac)
    d = jac / g
    h = 1e-2
    fp = mod.logLike(par + h * d, grad=False)
    fm = mod.logLike(par - h * d, grad=False)
    fd = (fp - fm) / (2 * h)
    assert abs(fd - g) <= 1e-3 * g, (fd, g)
