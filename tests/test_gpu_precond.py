"""Learned preconditioner and PCG on the GPU: network forward, training loss and
gradient against the oracle (csrc/pcg.cu vs oracle/precond_oracle.py), PCG
against the Cholesky solve, and what training gains over Jacobi and plain CG."""
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


def _golden_system(precision="fp64", tau=25.0):
    g = load("advdiff_ani_bc3")
    mod = gpu_model(g, precision)
    mod._assemble(g["par"])
    mod.plan.set_obs(mod.grid.obs_nodes(g["idx"]))
    return g, mod, tau


def test_weights_loss_and_gradient_match_oracle():
    from oracle import precond_oracle as po
    from spdepy_gb300.spdes import stencil_to_csr
    g, mod, tau = _golden_system()
    plan, grid = mod.plan, mod.grid
    prm = np.random.default_rng(0).normal(0.0, 0.2, po.NPARAMS).astype(np.float32)
    p_dev = torch.as_tensor(prm).cuda()
    w, act = plan.precond_weights(p_dev, True, tau, keep_activations=True)
    z = np.random.default_rng(1).choice([-1.0, 1.0], size=(grid.n, 3))
    loss, gr = plan.precond_grad(p_dev, w, act, torch.as_tensor(z), True, tau)
    A = stencil_to_csr(grid, plan.export_q(True, tau).cpu().numpy())
    l_ref, g_ref, w_ref = po.loss_grad(prm.astype(np.float64), A, grid.Mx, grid.Ny, grid.T, z)
    # FP32 network and weights against the FP64 restatement
    np.testing.assert_allclose(w.view(27, grid.n).T.cpu().numpy(), w_ref, rtol=2e-5, atol=2e-6 * np.abs(w_ref).max())
    assert loss == pytest.approx(l_ref, rel=1e-4)
    gd = gr.cpu().numpy()
    assert np.abs(gd - g_ref).max() <= 2e-4 * np.abs(g_ref).max()


def test_pcg_matches_cholesky_solve():
    from spdepy_gb300.precond import LearnedPreconditioner
    g, mod, tau = _golden_system()
    plan = mod.plan
    b = torch.as_tensor(np.random.default_rng(2).normal(size=(mod.grid.n, 2)))
    plan.factor(True, tau)
    x_ref, _ = plan.solve(b)
    x_ref = x_ref.cpu().numpy()
    lp = LearnedPreconditioner(seed=3)
    w = lp.weights(plan, True, tau)
    for kind in ("none", "jacobi", "learned", "ic0"):
        x, it, rel = plan.pcg(b, True, tau, kind, w=w, tol=1e-11, maxit=5000)
        assert rel <= 1e-11 and it > 0
        assert np.abs(x.cpu().numpy() - x_ref).max() <= 1e-8 * np.abs(x_ref).max()


def test_iterative_plan_has_no_factor():
    import spdepy_gb300._native as nat
    from spdepy_gb300.workloads import build_model, nonstationary_advection_diffusion
    w = nonstationary_advection_diffusion(M=20, N=20, T=4)
    mod = build_model(w, "iterative")
    mod._assemble(w.par)
    with pytest.raises(nat.SpdeError):
        mod.plan.factor(False, 0.0)
    b = torch.ones(w.grid.n, dtype=torch.float64)
    x, it, rel = mod.plan.pcg(b, False, 0.0, "jacobi", tol=1e-9)
    assert rel <= 1e-9


def test_training_beats_jacobi_and_plain_cg():
    """Train on systems drawn from the prior at 24 x 24 x 8, evaluate PCG on
    held-out parameters at 32 x 32 x 8."""
    from spdepy_gb300.precond import LearnedPreconditioner, prior_sample, system_maker
    from spdepy_gb300.workloads import build_model, nonstationary_advection_diffusion
    wt = nonstationary_advection_diffusion(M=24, N=24, T=8)
    mt = build_model(wt, "iterative")
    lp = LearnedPreconditioner(seed=0)
    hist = lp.train(system_maker(wt, mt), steps=400, probes=4, lr=3e-3, seed=1)
    assert np.mean(hist[-40:]) < 0.95 * np.mean(hist[:10])
    we = nonstationary_advection_diffusion(M=32, N=32, T=8, seed=5)
    me = build_model(we, "iterative")
    make = system_maker(we, me)
    rng = np.random.default_rng(123)
    its = {"none": [], "jacobi": [], "learned": []}
    for _ in range(3):
        plan, wo, tau = make(rng)
        b = torch.as_tensor(rng.normal(size=we.grid.n))
        wts = lp.weights(plan, wo, tau)
        for kind in its:
            _, it, rel = plan.pcg(b, wo, tau, kind, w=wts, tol=1e-8, maxit=20000)
            assert rel <= 1e-8
            its[kind].append(it)
    print("PCG iterations on held-out systems", its)
    assert sum(its["learned"]) < 0.9 * sum(its["jacobi"]) < sum(its["none"])


def test_hutchinson_gradient_by_pcg_matches_cholesky():
    """The Hutchinson gradient with every solve by PCG (plain, Jacobi, learned)
    equals the one with Cholesky solves on the same probes."""
    from spdepy_gb300.precond import LearnedPreconditioner
    from spdepy_gb300.workloads import build_model, nonstationary_advection_diffusion, simulate
    w = nonstationary_advection_diffusion(M=24, N=22, T=6)
    mod = build_model(w, "fp64")
    simulate(mod, w)
    np.random.seed(7)
    _, j_chol = mod.logLike(w.par, nh1=32, grad=True, grad_mode="hutchinson")
    lp = LearnedPreconditioner(seed=1)
    for pc in ("none", "jacobi", lp):
        np.random.seed(7)
        j_pcg, its = mod.logLikeGradPCG(w.par, precond=pc, nh1=32, tol=1e-11)
        assert its > 0
        np.testing.assert_allclose(j_pcg, j_chol, rtol=1e-7, atol=1e-8 * np.abs(j_chol).max())


@pytest.mark.parametrize("name", ["advdiff_ani_bc3", "covadv_vardiff_bc1", "wm_ani_bc1"])
def test_square_root_of_q(name):
    """B^T B x == Q x for the square root used by the factor-free samplers."""
    g = load(name)
    mod = gpu_model(g, "fp64")
    mod._assemble(g["par"])
    plan = mod.plan
    x = torch.as_tensor(np.random.default_rng(3).normal(size=(mod.grid.n, 3)))
    qx = plan.spmv(x).cpu().numpy()
    btbx = plan.qsqrt(plan.qsqrt(x), transpose=True).cpu().numpy()
    np.testing.assert_allclose(btbx, qx, rtol=0, atol=1e-12 * np.abs(qx).max())
    # the transpose is the adjoint
    z = torch.as_tensor(np.random.default_rng(4).normal(size=(mod.grid.n, 3))).cuda()
    lhs = (plan.qsqrt(x) * z).sum().item()
    rhs = (x.cuda() * plan.qsqrt(z, transpose=True)).sum().item()
    assert lhs == pytest.approx(rhs, rel=1e-12)


def test_posterior_draws_by_pcg_match_cholesky():
    """Factor-free posterior draws (B^T e1 + sqrt(tau) S^T e2 through PCG) equal
    the Cholesky solve of the same perturbations."""
    g = load("advdiff_ani_bc3")
    mod = gpu_model(g, "fp64")
    x_pcg, its = mod.samplePosteriorPCG(n=4, precond="jacobi", seed=9, tol=1e-12)
    assert its > 0
    plan = mod.plan
    tau = float(np.exp(mod.canonical(mod.par)[-1]))
    rng = np.random.default_rng(9)
    nn = mod.grid.n
    e1 = torch.as_tensor(rng.normal(size=(nn, 4))).cuda()
    nodes = mod.grid.obs_nodes(mod.idx)
    e2 = torch.as_tensor(rng.normal(size=(nodes.size, 4))).cuda()
    rhs = plan.qsqrt(e1, transpose=True)
    rhs.index_add_(0, torch.as_tensor(nodes).cuda(), np.sqrt(tau) * e2)
    b = torch.zeros(nn, dtype=torch.float64, device="cuda")
    b.index_add_(0, torch.as_tensor(nodes).cuda(), tau * torch.as_tensor(np.asarray(g["y"], float)).cuda())
    plan.factor(True, tau)
    mu, _ = plan.solve(b)
    xs, _ = plan.solve(rhs)
    ref = (xs + mu[:, None]).cpu().numpy()
    np.testing.assert_allclose(x_pcg.cpu().numpy(), ref, rtol=0, atol=1e-9 * np.abs(ref).max())


def test_compact_weights_are_the_per_node_operator():
    """The compact weights (one row of G per cell and time class, one per observed
    node) expand to exactly the per-node weights, PCG gives the same solution
    with either, and a solve with another observation setting is refused."""
    import spdepy_gb300._native as nat
    from spdepy_gb300.precond import LearnedPreconditioner
    g, mod, tau = _golden_system()
    plan, grid = mod.plan, mod.grid
    lp = LearnedPreconditioner(seed=3)
    lp.params.add_(torch.randn(lp.params.shape, generator=torch.Generator().manual_seed(4)).cuda() * 0.05)
    wn = lp.weights(plan, True, tau, compact=False).view(27, grid.n).cpu().numpy()
    wc = lp.weights(plan, True, tau)
    raw = wc.data.cpu().numpy()
    n, Ns, T = grid.n, grid.Mx * grid.Ny, grid.T
    obs_nodes = np.unique(grid.obs_nodes(g["idx"]))
    cls = raw[4:4 + 3 * 27 * Ns].reshape(3, 27, Ns)
    orow = raw[4 + 3 * 27 * Ns:].reshape(27, obs_nodes.size)
    k = np.arange(n)
    t, c = np.divmod(k, Ns)
    klass = np.where(t == 0, 0, np.where(t == T - 1, 2, 1))
    full = cls[klass, :, c].T.copy()
    full[:, obs_nodes] = orow
    np.testing.assert_array_equal(full, wn)
    b = torch.as_tensor(np.random.default_rng(2).normal(size=(grid.n, 3)))
    x1, it1, r1 = plan.pcg(b, True, tau, "learned", w=torch.as_tensor(wn.ravel()).cuda(), tol=1e-10)
    x2, it2, r2 = plan.pcg(b, True, tau, "learned", w=wc, tol=1e-10)
    assert r1 <= 1e-10 and r2 <= 1e-10 and abs(it1 - it2) <= 4
    np.testing.assert_allclose(x2.cpu().numpy(), x1.cpu().numpy(), rtol=0, atol=1e-8 * np.abs(x1.cpu().numpy()).max())
    with pytest.raises(nat.SpdeError, match="do not match"):
        plan.pcg(b, False, 0.0, "learned", w=wc, tol=1e-8)


def test_ic0_preconditioner_reduces_iterations():
    """IC(0) in the natural order (the incomplete-Cholesky baseline of the PCG
    comparison) converges in fewer iterations than Jacobi on the non-stationary
    generator, and its solution matches the other preconditioners'."""
    from spdepy_gb300.workloads import build_model, nonstationary_advection_diffusion
    w = nonstationary_advection_diffusion(M=40, N=36, T=10, seed=4)
    mod = build_model(w, "iterative")
    mod._assemble(w.par)
    n = w.grid.n
    idx = np.sort(np.random.default_rng(0).choice(n, n // 50, replace=False))
    mod.plan.set_obs(idx)
    tau = float(np.exp(w.par[-1]))
    b = torch.as_tensor(np.random.default_rng(1).normal(size=n))
    xj, itj, relj = mod.plan.pcg(b, True, tau, "jacobi", tol=1e-9)
    xi, iti, reli = mod.plan.pcg(b, True, tau, "ic0", tol=1e-9)
    assert relj <= 1e-9 and reli <= 1e-9
    assert iti < itj
    np.testing.assert_allclose(xi.cpu().numpy(), xj.cpu().numpy(), rtol=0, atol=1e-7 * np.abs(xj.cpu().numpy()).max())
