"""The mixed-precision plan on a grid large enough that its fronts go through
the tensor-core tiled product (3xTF32, k >= 128), against the FP64 plan on the
same inputs: log-likelihood, exact gradient, selected inverse, solves, samples."""
import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def pair():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from spdepy_gb300 import build
    from spdepy_gb300.workloads import build_model, nonstationary_advection_diffusion, simulate
    build.build()
    w = nonstationary_advection_diffusion(M=48, N=48, T=12)
    m64 = build_model(w, "fp64")
    simulate(m64, w)
    mmx = build_model(w, "mixed")
    mmx.initFit(w.y, idx=w.idx)
    return w, m64, mmx


def test_fronts_reach_tensor_core_sizes(pair):
    w, m64, mmx = pair
    info = mmx.plan.info()
    assert info.max_front >= 512


def test_loglike_and_gradient_mixed_vs_fp64(pair):
    w, m64, mmx = pair
    f64, g64 = m64.logLike(w.par, grad=True)
    fmx, gmx = mmx.logLike(w.par, grad=True)
    assert abs(fmx - f64) <= 1e-6 * abs(f64)
    # the selected inverse of an FP32 factor carries ~cond(Q) * 2^-24 relative
    # error; the gradient (traces of Z_Q - Z_Qc) is held to 1e-3 of its largest entry
    assert np.abs(gmx - g64).max() <= 1e-3 * np.abs(g64).max()


def test_selinv_solve_sample_mixed_vs_fp64(pair):
    w, m64, mmx = pair
    out = {}
    for name, m in (("fp64", m64), ("mixed", mmx)):
        m._assemble(w.par)
        p = m.plan
        ld = p.factor(False, 0.0)
        z = torch.as_tensor(np.random.default_rng(3).normal(size=(w.grid.n, 8)))
        x = p.sample(z).cpu().numpy()
        b = torch.as_tensor(np.random.default_rng(4).normal(size=(w.grid.n, 4)))
        s, res = p.solve(b)
        p.factor(False, 0.0)
        zq = p.selinv().cpu().numpy()
        out[name] = (ld, x, s.cpu().numpy(), res, zq)
    ld64, x64, s64, _, z64 = out["fp64"]
    ldm, xm, sm, resm, zm = out["mixed"]
    assert abs(ldm - ld64) <= 1e-7 * abs(ld64)
    assert resm <= 1e-10
    assert np.abs(sm - s64).max() <= 1e-9 * np.abs(s64).max()
    assert np.abs(xm - x64).max() <= 1e-4 * np.abs(x64).max()
    mask = z64 != 0
    assert np.abs(zm - z64)[mask].max() <= 1e-4 * np.abs(z64).max()


def test_one_and_two_pipelines_agree(pair):
    """spde_loglike with the Q and Q + tau S^T S pipelines on two streams gives the
    same numbers as with both on one (the kernels are deterministic)."""
    from spdepy_gb300 import _native as nat
    w, m64, mmx = pair
    f2, g2 = mmx.logLike(w.par, grad=True)
    nat.check(nat.lib().spde_plan_set_pipelines(mmx.plan.h, 1), mmx.plan.h)
    try:
        f1, g1 = mmx.logLike(w.par, grad=True)
    finally:
        nat.check(nat.lib().spde_plan_set_pipelines(mmx.plan.h, 2), mmx.plan.h)
    assert f1 == f2
    np.testing.assert_array_equal(g1, g2)
