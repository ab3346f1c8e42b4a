"""The preconditioner oracle pinned by central finite differences of its own
training loss, plus the Jacobi start and the CPU PCG it uses."""
import numpy as np
import pytest
from scipy import sparse

from golden_cases import load


def _system():
    g = load("advdiff_ani_bc3")
    M, N, T = int(g["M"]), int(g["N"]), int(g["T"])
    assert int(g["extend"]) < 0
    n = M * N * T
    Q = sparse.csc_matrix((g["Q_data"], g["Q_indices"], g["Q_indptr"]), shape=(n, n)).tocsr()
    tau = 25.0
    d = np.zeros(n)
    np.add.at(d, g["idx"], tau)
    return Q + sparse.diags(d), M, N, T


def _params(seed, scale=0.2):
    from oracle import precond_oracle as po
    rng = np.random.default_rng(seed)
    return rng.normal(0.0, scale, po.NPARAMS)


def test_loss_gradient_matches_central_differences():
    from oracle import precond_oracle as po
    A, M, N, T = _system()
    prm = _params(0)
    z = np.random.default_rng(1).choice([-1.0, 1.0], size=(A.shape[0], 2))
    loss, grad, _ = po.loss_grad(prm, A, M, N, T, z)
    assert loss > 0
    rng = np.random.default_rng(2)
    picks = np.concatenate([rng.choice(po.NPARAMS, 24, replace=False), [po.NPARAMS - 1, 0]])
    h = 1e-6
    for i in picks:
        e = np.zeros_like(prm)
        e[i] = h
        fd = (po.loss_grad(prm + e, A, M, N, T, z)[0] - po.loss_grad(prm - e, A, M, N, T, z)[0]) / (2 * h)
        assert fd == pytest.approx(grad[i], rel=1e-5, abs=1e-9 * np.abs(grad).max())


def test_zero_last_layer_is_jacobi():
    from oracle import precond_oracle as po
    A, M, N, T = _system()
    prm = _params(3)
    P = po.unpack(prm)
    P["W3"][:] = 0.0
    P["b3"][:] = 0.0
    prm = po.pack(P)
    f, s = po.features(po.stencil43(A, M, N, T))
    _, _, out = po.forward(prm, f)
    w = po.weights(out, s, M, N, T)
    v = np.random.default_rng(4).normal(size=A.shape[0])
    np.testing.assert_allclose(po.apply_G(w, v, M, N, T), v / np.sqrt(A.diagonal()), rtol=1e-14)
    np.testing.assert_allclose(po.apply_G(w, v, M, N, T, transpose=True), v / np.sqrt(A.diagonal()), rtol=1e-14)


def test_apply_transpose_is_adjoint():
    from oracle import precond_oracle as po
    A, M, N, T = _system()
    f, s = po.features(po.stencil43(A, M, N, T))
    _, _, out = po.forward(_params(5), f)
    w = po.weights(out, s, M, N, T)
    rng = np.random.default_rng(6)
    a, b = rng.normal(size=A.shape[0]), rng.normal(size=A.shape[0])
    assert po.apply_G(w, a, M, N, T) @ b == pytest.approx(a @ po.apply_G(w, b, M, N, T, transpose=True), rel=1e-12)


def test_oracle_pcg_converges():
    from oracle import precond_oracle as po
    A, *_ = _system()
    b = np.random.default_rng(7).normal(size=A.shape[0])
    d = A.diagonal()
    x, it, rel = po.pcg(A, b, lambda r: r / d, tol=1e-10)
    assert rel <= 1e-10 and it > 0
