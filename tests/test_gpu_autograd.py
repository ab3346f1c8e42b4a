"""The differentiable objective (torch.autograd.Function) against central finite
differences, the mixed-precision path against FP64 on the non-stationary
advection-diffusion generator, and sample moments against the selected inverse."""
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


def _fd(mod, par, i, h=1e-5):
    e = np.zeros_like(par)
    e[i] = h
    return (mod.logLike(par + e, grad=False) - mod.logLike(par - e, grad=False)) / (2 * h)


@pytest.mark.parametrize("name", ["advdiff_ani_bc3", "covadv_vardiff_bc1", "varadv_vardiff_bc1", "wm_ha_bc3"])
def test_autograd_gradient_matches_central_differences(name):
    import spdepy_gb300 as sp
    g = load(name)
    mod = gpu_model(g, "fp64")
    par = np.asarray(g["par"], dtype=np.float64)
    p = torch.tensor(par, requires_grad=True)
    f = sp.loglike(mod, p)
    f.backward()
    ga = p.grad.numpy()
    f_ref, jac = mod.logLike(par, grad=True)
    assert float(f) == pytest.approx(f_ref, rel=1e-14)
    np.testing.assert_allclose(ga, jac, rtol=1e-14, atol=0)
    fd = np.array([_fd(mod, par, i) for i in range(par.size)])
    scale = np.abs(fd).max()
    # central differences with h = 1e-5: truncation ~h^2, rounding ~eps |f| / h
    np.testing.assert_allclose(ga, fd, rtol=1e-5, atol=1e-7 * scale)


def test_autograd_without_grad_request():
    import spdepy_gb300 as sp
    g = load("advdiff_ani_bc3")
    mod = gpu_model(g, "fp64")
    f = sp.loglike(mod, torch.tensor(np.asarray(g["par"], dtype=np.float64)))
    assert not f.requires_grad
    assert float(f) == pytest.approx(mod.logLike(g["par"], grad=False), rel=1e-14)


def _generator_model(precision):
    from spdepy_gb300.workloads import build_model, nonstationary_advection_diffusion, simulate
    w = nonstationary_advection_diffusion(M=30, N=28, T=6)
    mod = build_model(w, precision)
    simulate(mod, w)
    return w, mod


def test_nonstationary_generator_fd_and_mixed_precision():
    """The non-stationary advection-diffusion generator (5 x 5 B-spline anisotropy,
    Fourier velocity field scaled by lambda) on a reduced grid: FP64 gradient vs
    central differences (h = 1e-5) and the mixed path within 1e-6 relative in logL."""
    import spdepy_gb300 as sp
    w, m64 = _generator_model("fp64")
    par = w.par.copy()
    p = torch.tensor(par, requires_grad=True)
    f64 = sp.loglike(m64, p)
    f64.backward()
    g64 = p.grad.numpy()
    lay = m64.layout
    picks = [0, lay.sl["vx"].start + 3, lay.sl["vy"].start + 7, lay.sl["lamb"].start, lay.sl["sigma"].start,
             par.size - 2, par.size - 1]
    fd = np.array([_fd(m64, par, i) for i in picks])
    np.testing.assert_allclose(g64[picks], fd, rtol=1e-5, atol=1e-7 * np.abs(g64).max())
    _, mmx = _generator_model("mixed")
    fm, gm = mmx.logLike(par, grad=True)
    assert abs(fm - float(f64)) <= 1e-6 * abs(float(f64))
    assert np.abs(gm - g64).max() <= 1e-4 * np.abs(g64).max()


def test_sample_variances_match_selected_inverse():
    """Empirical variances of P L^-T z draws against diag(Q^-1) from the selected
    inverse (4,000 draws: relative standard error sqrt(2/4000) = 2.2 %)."""
    g = load("advdiff_ani_bc3")
    mod = gpu_model(g, "fp64")
    mod._assemble(g["par"])
    plan = mod.plan
    plan.factor(False, 0.0)
    ns = 4000
    z = torch.as_tensor(np.random.default_rng(11).normal(size=(mod.grid.n, ns)))
    x = plan.sample(z).cpu().numpy()
    plan.factor(False, 0.0)
    zq = plan.selinv().cpu().numpy()
    var = zq[:, 21]
    emp = (x * x).mean(axis=1)
    rel = emp / var - 1.0
    assert np.abs(rel).max() < 6 * np.sqrt(2.0 / ns)
    assert abs(rel.mean()) < 4 * np.sqrt(2.0 / ns / mod.grid.n) + 0.01


def test_lbfgs_fit_reaches_a_stationary_point():
    """L-BFGS on the exact gradients (the maximum-likelihood fit driver) on the
    sensor-track generator: lambda, log sigma and log tau free from a perturbed
    start, everything else held at the truth."""
    from spdepy_gb300.optim import Optimize
    from spdepy_gb300.workloads import build_model, sensor_track_advection_diffusion, simulate
    w = sensor_track_advection_diffusion(M=32, N=30, T=8, steps_per_t=300)
    mod = build_model(w, "fp64")
    simulate(mod, w, seed=4)
    truth = w.par.copy()
    nb2 = w.grid.Nbs2
    free = np.array([4 * nb2, 4 * nb2 + 1, truth.size - 1])
    fix = np.setdiff1d(np.arange(truth.size), free)
    x0 = truth.copy()
    x0[free] += np.array([0.4, -0.3, 0.5])
    res = Optimize(mod.logLike).fit(x0=x0, stepType="lbfgs", max_steps=50, fix=fix)
    assert np.array_equal(res["x"][fix], truth[fix])
    assert res["fun"] < mod.logLike(x0, grad=False)
    assert np.abs(np.asarray(res["jac"])[free]).max() < 1e-5
    # the estimates move towards the truth
    assert np.abs(res["x"][free] - truth[free]).max() < np.abs(x0[free] - truth[free]).max()
