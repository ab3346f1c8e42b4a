"""GPU parity of the separable space-time models Q = Qt (x) Qs (75-slot plans)
against the reference's golden fixtures and the oracle."""
import numpy as np
import pytest
from scipy import sparse

from golden_cases import diff_form, grid_args, load, separable_cases, separable_oracle

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

TOL_F = {"fp64": 1e-11, "mixed": 1e-6}
TOL_G = {"fp64": 1e-8, "mixed": 1e-4}


@pytest.fixture(scope="module", autouse=True)
def _cuda():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from spdepy_gb300 import build
    build.build()


def sep_model(g, precision="fp64"):
    from spdepy_gb300.grids import Grid
    from spdepy_gb300.spdes import spde_init
    ga = grid_args(g)
    grid = Grid(ga["x"], ga["y"], ga["t"], ga["extend"], ga["Nbs"])
    d = diff_form(g)
    mod = spde_init("seperable-spatial-temporal", grid, ani=d != "iso", ha=d == "ha", bc=int(g["bc"]),
                    precision=precision)
    mod.setPars(g["par"])
    mod.initFit(g["y"], idx=g["idx"])
    return mod


@pytest.mark.parametrize("name", separable_cases())
def test_separable_q_assembly(name):
    g = load(name)
    mod = sep_model(g)
    Q = mod.makeQ(g["par"])[0].to_scipy()
    Qg = sparse.csr_matrix((g["Q_data"], g["Q_indices"], g["Q_indptr"]), shape=Q.shape)
    assert abs(Q - Qg).max() <= 1e-12 * abs(Qg).max()
    x = np.random.default_rng(0).normal(size=(Q.shape[0], 3))
    y = mod.plan.spmv(torch.as_tensor(x)).cpu().numpy()
    assert np.allclose(y, Qg @ x, rtol=0, atol=1e-12 * np.abs(Qg @ x).max())


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
@pytest.mark.parametrize("name", separable_cases())
def test_separable_loglike_and_exact_gradient(name, precision):
    g = load(name)
    mod = sep_model(g, precision)
    f = mod.logLike(g["par"], grad=False)
    assert abs(f - float(g["f"])) <= TOL_F[precision] * max(1.0, abs(float(g["f"])))
    f0, jex = separable_oracle(g).loglike(g["par"], g["y"], g["idx"], grad=True, exact=True)
    f1, jac = mod.logLike(g["par"], grad=True)
    assert abs(f1 - f0) <= TOL_F[precision] * max(1.0, abs(f0))
    scale = np.abs(jex).max()
    assert np.allclose(jac, jex, rtol=TOL_G[precision], atol=TOL_G[precision] * scale), np.abs(jac - jex).max() / scale


@pytest.mark.parametrize("name", separable_cases())
def test_separable_hutchinson_replica(name):
    """The reference's estimator with its own seeded probes."""
    g = load(name)
    mod = sep_model(g, "fp64")
    np.random.seed(int(g["seed_v"]))
    f, jac = mod.logLike(g["par"], nh1=int(g["nh1"]), grad=True, grad_mode="hutchinson")
    assert abs(f - float(g["f_grad"])) <= 1e-11 * max(1.0, abs(float(g["f_grad"])))
    assert np.allclose(jac, g["jac"], rtol=1e-8, atol=1e-9 * np.abs(g["jac"]).max())
