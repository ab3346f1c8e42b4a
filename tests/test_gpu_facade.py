"""The Model facade on the GPU (reference model.py:73-150): marginal variances
(qinv) against dense inverses, updates with different noise precisions and with
fixed effects against the reference's own results, and the prediction loop of
examples/advection_diffusion_example/results.py:9-32 (setModel, update, qinv per
time step) against dense FP64 algebra on the oracle's Q."""
import numpy as np
import pytest
from scipy import sparse

from golden_cases import load, oracle_model, separable_oracle
from gpu_cases import gpu_model, separable_gpu_model

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

# qinv returns float32 as the reference does; the mixed plan's selected inverse
# carries the FP32 factor's error (about cond(Q) 2^-24 relative)
TOL_V = {"fp64": 2e-6, "mixed": 1e-4}


@pytest.fixture(scope="module", autouse=True)
def _cuda():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from spdepy_gb300 import build
    build.build()


def _wm_facade(g, precision):
    import spdepy_gb300 as sp
    from oracle.spde_oracle import OracleGrid, OracleModel
    M, N = int(g["M"]), int(g["N"])
    grid = sp.grid(x=np.arange(M, dtype=float), y=np.arange(N, dtype=float))
    m = sp.Model(spde="whittle-matern", grid=grid, parameters=g["par"], ani=True, ha=False, bc=3,
                 precision=precision)
    Q = OracleModel(OracleGrid(np.arange(M, dtype=float), np.arange(N, dtype=float)), "whittle-matern", "ani",
                    3).makeQ(g["par"]).toarray()
    return m, Q


def _facade(name, precision):
    """A Model around a golden case, and the oracle's dense Q of the same model."""
    from spdepy_gb300.model import Model
    if name == "facade_wm":
        return _wm_facade(load("facade_wm.npz"), precision)
    g = load(name)
    if name.startswith("separable_"):
        mod = separable_gpu_model(g, precision)
        Q = separable_oracle(g).makeQ(g["par"]).toarray()
    else:
        mod = gpu_model(g, precision)
        Q = oracle_model(g).makeQ(g["par"]).toarray()
    mod.setQ(par=g["par"])
    m = Model(grid=mod.grid, precision=precision)
    m.mod = mod
    return m, Q


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
@pytest.mark.parametrize("name", ["facade_wm", "advdiff_ani_bc3", "separable_ani_bc1"])
def test_qinv_matches_dense_inverse_before_and_after_update(name, precision):
    m, Q = _facade(name, precision)
    m.setModel()
    v0 = m.qinv()
    assert v0.dtype == np.float32
    ref = np.diag(np.linalg.inv(Q))
    assert np.allclose(v0, ref, rtol=TOL_V[precision], atol=0), np.abs(v0 / ref - 1).max()
    rng = np.random.default_rng(3)
    g = m.grid
    idx = np.sort(rng.choice(g.M * g.N * g.T, 25, replace=False))
    y = rng.normal(size=idx.size)
    tau = 40.0
    m.update(y, idx, tau=tau)
    A = Q.copy()
    nodes = g.obs_nodes(idx)
    np.add.at(A, (nodes, nodes), tau)
    v1 = m.qinv()
    ref1 = np.diag(np.linalg.inv(A))
    assert np.allclose(v1, ref1, rtol=TOL_V[precision], atol=0), np.abs(v1 / ref1 - 1).max()
    assert (v1 <= v0 * (1 + TOL_V[precision])).all()  # observations only remove variance


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_updates_with_different_tau_golden(precision):
    """Model.update twice with tau 20 and 3.5: the reference accumulates
    Q += tau_k S_k^T S_k (model.py:122), here per-observation weights on the
    GPU factor; conditional means against the reference's, plain and with the
    covariate + intercept fixed effects."""
    g = load("facade_tau.npz")
    tol = 1e-9 if precision == "fp64" else 1e-8
    for name in ("plain", "cov"):
        m, _ = _wm_facade(g, precision)
        if name == "cov":
            m.setModel(mu=g["cov"], sigmas=np.log(np.array([0.01, 140.0])), useCov=True, scale=True)
        else:
            m.setModel()
        for k, tau in ((1, float(g["tau1"])), (2, float(g["tau2"]))):
            m.update(g[f"y{k}"], g[f"idx{k}"], tau=tau)
            ref = g[f"{name}_mu{k}"]
            assert np.allclose(m.mu, ref, rtol=tol, atol=tol * np.abs(ref).max()), (name, k)


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_qinv_with_fixed_effects(precision):
    """The reference's qinv with fixed effects: diag((S Q_aug S^T)^-1) with
    S = getS() = [I | X] (model.py:108-117), returned in an (n + p)-vector; here
    against dense FP64 algebra after two updates with different precisions."""
    g = load("facade_tau.npz")
    m, Q = _wm_facade(g, precision)
    m.setModel(mu=g["cov"], sigmas=np.log(np.array([0.01, 140.0])), useCov=True, scale=True)
    n = Q.shape[0]
    X = m.grid._fixed_effects()
    Qaug = sparse.block_diag([Q, np.diag(np.array([0.01, 140.0]))]).toarray()
    for k, tau in ((1, float(g["tau1"])), (2, float(g["tau2"]))):
        m.update(g[f"y{k}"], g[f"idx{k}"], tau=tau)
        Sk = np.hstack([np.eye(n)[g[f"idx{k}"]], X[g[f"idx{k}"]]])
        Qaug += tau * Sk.T @ Sk
    v = m.qinv()
    S = np.hstack([np.eye(n), X])
    ref = np.diag(np.linalg.inv(S @ Qaug @ S.T))
    assert v.dtype == np.float32 and v.shape == (n + 2,)
    assert np.allclose(v[:n], ref, rtol=TOL_V[precision], atol=0), np.abs(v[:n] / ref - 1).max()
    assert (v[n:] == 0).all()


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_prediction_loop(precision):
    """The paper's prediction loop (results.py:9-32) on a small space-time grid:
    for each time step, reset the model, observe that step's slice except the
    held-out positions, and predict with the conditional mean and the marginal
    variances; both against dense FP64 algebra on the oracle's Q at every step."""
    m, Q = _facade("advdiff_ani_bc3", precision)
    g = m.grid
    npos = g.M * g.N * g.T
    rng = np.random.default_rng(8)
    data = rng.normal(size=npos)
    held = np.sort(rng.choice(npos, npos // 10, replace=False))
    tau = m.mod.par[-1]
    tau = float(np.exp(tau))
    nidx = np.arange(npos)
    Qinv_diag = None
    for t in range(g.T):
        m.setModel()
        uidx = np.zeros(npos, dtype=bool)
        uidx[t * g.M * g.N:(t + 1) * g.M * g.N] = True
        uidx[held] = False
        m.update(y=data[uidx], idx=nidx[uidx])
        nodes = g.obs_nodes(nidx[uidx])
        A = Q.copy()
        np.add.at(A, (nodes, nodes), tau)
        b = np.zeros(g.n)
        np.add.at(b, nodes, tau * data[uidx])
        mu_ref = np.linalg.solve(A, b)
        assert np.allclose(m.mu, mu_ref, rtol=1e-8, atol=1e-9 * np.abs(mu_ref).max()), t
        mvar = m.qinv()
        Qinv_diag = np.diag(np.linalg.inv(A))
        assert np.allclose(mvar, Qinv_diag, rtol=TOL_V[precision], atol=0), t
        # the scores the loop reports: squared error and CRPS-type spread terms are finite
        z = (data - g.getS() @ m.mu) / np.sqrt(mvar[: npos] if g.Ne == 0 else g.getS() @ mvar)
        assert np.isfinite(z).all()
