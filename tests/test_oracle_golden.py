"""Pin the oracle against fixtures produced by the reference itself (CPU only)."""
import numpy as np
import pytest
from scipy import sparse

from golden_cases import load, model_cases, oracle_model, separable_cases, separable_oracle
from oracle import stencils as S


def test_stencils_bit_exact():
    g = load("stencils.npz")
    M, N, hx, hy = int(g["M"]), int(g["N"]), float(g["hx"]), float(g["hy"])
    for bc in (1, 3):
        for fam, field in (("AcH", False), ("AH", True)):
            r, c, v = S.diffusion_triplets(M, N, g["H"] if field else g["Hc"], hx, hy, bc, field)
            k = f"{fam}_b{bc}"
            assert np.array_equal(r, g[k + "_row"]) and np.array_equal(c, g[k + "_col"])
            assert np.array_equal(v, g[k + "_val"])
        for diff in (1, 2, 3):
            r, c, v = S.advection_const_triplets(M, N, g["Gc"], hx, hy, bc, diff)
            k = f"Acw_b{bc}_d{diff}"
            assert np.array_equal(r, g[k + "_row"]) and np.array_equal(c, g[k + "_col"])
            assert np.array_equal(v, g[k + "_val"], equal_nan=True)
            r, c, v = S.advection_field_triplets(M, N, g["G"], hx, hy, bc, diff, g["dG"])
            k = f"Aw_b{bc}_d{diff}"
            assert np.array_equal(r, g[k + "_row"]) and np.array_equal(c, g[k + "_col"])
            assert np.array_equal(v, g[k + "_val"], equal_nan=True)


@pytest.mark.parametrize("name", model_cases())
def test_model_golden(name):
    g = load(name)
    mod = oracle_model(g)
    par = g["par"]
    Q = mod.makeQ(par)
    Qg = sparse.csr_matrix((g["Q_data"], g["Q_indices"], g["Q_indptr"]), shape=Q.shape)
    assert abs(Q - Qg).max() <= 1e-13 * abs(Qg).max()
    f = mod.loglike(par, g["y"], g["idx"], grad=False)
    assert abs(f - float(g["f"])) <= 1e-12 * abs(float(g["f"]))
    fg, jac = mod.loglike(par, g["y"], g["idx"], grad=True, nh1=int(g["nh1"]), seed=int(g["seed_v"]))
    assert np.allclose(jac, g["jac"], rtol=1e-10, atol=1e-12 * np.abs(g["jac"]).max())


@pytest.mark.parametrize("name", separable_cases())
def test_separable_golden(name):
    """Q = Qt (x) Qs, the objective and the Hutchinson gradient of the reference's
    separable space-time classes."""
    g = load(name)
    mod = separable_oracle(g)
    par = g["par"]
    Q = mod.makeQ(par)
    Qg = sparse.csr_matrix((g["Q_data"], g["Q_indices"], g["Q_indptr"]), shape=Q.shape)
    assert abs(Q - Qg).max() <= 1e-13 * abs(Qg).max()
    assert len(mod.dQ_list(par)) == par.size - 1
    f = mod.loglike(par, g["y"], g["idx"], grad=False)
    assert abs(f - float(g["f"])) <= 1e-12 * abs(float(g["f"]))
    fg, jac = mod.loglike(par, g["y"], g["idx"], grad=True, nh1=int(g["nh1"]), seed=int(g["seed_v"]))
    assert np.allclose(jac, g["jac"], rtol=1e-10, atol=1e-12 * np.abs(g["jac"]).max())


def test_separable_derivatives_by_differences():
    """The analytic dQ list of the separable oracle against central differences of
    its own Q (this also checks the temporal derivatives, which the golden
    Hutchinson gradient only sees through a random projection)."""
    for name in separable_cases():
        g = load(name)
        mod = separable_oracle(g)
        par = np.asarray(g["par"], float)
        dQ = mod.dQ_list(par)
        for i in range(par.size - 1):
            h = 1e-6 * max(1.0, abs(par[i]))
            pp, pm = par.copy(), par.copy()
            pp[i] += h
            pm[i] -= h
            fd = (mod.makeQ(pp) - mod.makeQ(pm)) / (2 * h)
            assert abs(fd - dQ[i]).max() <= 1e-6 * max(abs(dQ[i]).max(), 1e-8), (name, i)


def test_facade_update_golden():
    from oracle.spde_oracle import OracleGrid, OracleModel
    g = load("facade_wm.npz")
    grid = OracleGrid(np.arange(int(g["M"]), dtype=float), np.arange(int(g["N"]), dtype=float))
    mod = OracleModel(grid, "whittle-matern", "ani", int(g["bc"]))
    Q = mod.makeQ(g["par"])
    Qg = sparse.csr_matrix((g["Q_data"], g["Q_indices"], g["Q_indptr"]), shape=Q.shape)
    assert abs(Q - Qg).max() <= 1e-13 * abs(Qg).max()
    mu = mod.conditional_mean(g["par"], g["y"], g["idx"], tau=float(g["tau"]))
    assert np.allclose(mu, g["mu"], rtol=1e-11, atol=1e-13)


def test_getS_fixed_effect_columns():
    """Grid.getS after addInt / addCov matches the reference's S bit for bit
    (selected identity rows on a padded grid, then [1, cov], [1, cov / max],
    [cov] or [1])."""
    from spdepy_gb300.grids import Grid
    g = load("grid_getS.npz")
    M, N, T, ext = (int(g[k]) for k in ("M", "N", "T", "extend"))
    for name in ("plain", "int", "cov_int", "cov_int_scale", "cov"):
        grid = Grid(np.arange(M, dtype=float), np.arange(N, dtype=float), np.arange(T, dtype=float), extend=ext)
        if name == "int":
            grid.addInt()
        elif name != "plain":
            grid.addCov(g["cov"], inter=name.startswith("cov_int"), scale=name.endswith("scale"))
        for tag, idx in (("sub", g["idx"]), ("all", None)):
            ref = sparse.csr_matrix((g[f"{name}_{tag}_data"], g[f"{name}_{tag}_indices"], g[f"{name}_{tag}_indptr"]),
                                    shape=tuple(g[f"{name}_{tag}_shape"]))
            S = grid.getS(idx)
            assert S.shape == ref.shape, (name, tag)
            assert abs(S - ref).max() == 0.0, (name, tag)


def _fixed_effect_setup(g, name):
    """Grid with the fixture's fixed-effect columns and the reference's initial mu (model.py:129-150)."""
    from spdepy_gb300.grids import Grid
    M, N = int(g["M"]), int(g["N"])
    grid = Grid(np.arange(M, dtype=float), np.arange(N, dtype=float))
    cov = g["cov"]
    n = grid.n
    if name == "cov":
        grid.addCov(cov, scale=True)
        mu = np.zeros(n + 2)
        mu[-2:] = [0.0, cov.max()]
    else:
        grid.addInt()
        S = grid.getS()
        mu = np.zeros(n + 1)
        mu[:-1] = S[:, :-1].T @ cov
    return grid, mu


@pytest.mark.parametrize("name", ["cov", "int"])
def test_fixed_effect_updates_by_block_elimination(name):
    """Model.update with fixed effects (intercept and covariate coefficients) by
    block elimination on the sparse part matches the reference's augmented
    Cholesky solves (dense exact solves stand in for the GPU factor here)."""
    from oracle.spde_oracle import OracleGrid, OracleModel
    from spdepy_gb300.fixed_effects import Border, update_step
    g = load("facade_cov.npz")
    M, N = int(g["M"]), int(g["N"])
    Q = OracleModel(OracleGrid(np.arange(M, dtype=float), np.arange(N, dtype=float)), "whittle-matern", "ani",
                    3).makeQ(g["par"]).toarray()
    grid, mu = _fixed_effect_setup(g, name)
    assert np.allclose(mu, g[f"{name}_mu0"], rtol=1e-14, atol=0)
    tau = float(g[f"{name}_tau"])
    border = Border(grid.n, np.exp(g[f"{name}_sigmas"]))
    A = Q.copy()
    F = grid._fixed_effects()
    for k in (1, 2):
        idx, y = g[f"idx{k}"], g[f"y{k}"]
        nodes = grid.obs_nodes(idx)
        np.add.at(A, (nodes, nodes), tau)
        mu = update_step(border, lambda R: np.linalg.solve(A, R), mu, nodes, F[idx], y, tau)
        ref = g[f"{name}_mu{k}"]
        assert np.allclose(mu, ref, rtol=1e-10, atol=1e-12 * np.abs(ref).max()), k


def test_fixed_effect_draws_have_the_augmented_covariance():
    """Border.sample: x = (P L^-T z_n - A^-1 B x_b, L_Sc^-T z_b) has covariance
    exactly Q_aug^-1, checked with the draw's linear map on a small dense case."""
    from spdepy_gb300.fixed_effects import Border
    rng = np.random.default_rng(5)
    n, p = 30, 2
    R = rng.normal(size=(n, n))
    A0 = R @ R.T + n * np.eye(n)
    border = Border(n, [0.5, 2.0])
    nodes = rng.choice(n, 12, replace=False)
    X = rng.normal(size=(12, p))
    border.add(nodes, X, 3.0)
    A = A0.copy()
    np.add.at(A, (nodes, nodes), 3.0)
    L = np.linalg.cholesky(A)
    import scipy.linalg as sla
    Zn, Zb = np.eye(n + p)[:n], np.eye(n + p)[n:]  # the map applied to the identity
    xn, xb = border.sample(lambda Z: sla.solve_triangular(L.T, Z, lower=False), lambda R: np.linalg.solve(A, R),
                           Zn, Zb)
    G = np.vstack([xn, xb])  # x = G z
    Qaug = np.block([[A, border.B], [border.B.T, border.C]])
    assert np.allclose(G @ G.T, np.linalg.inv(Qaug), rtol=1e-9, atol=1e-12)


@pytest.mark.parametrize("name", separable_cases())
def test_separable_host_mapping(name):
    """Host side of the separable GPU models (no device needed): the reference's
    dispatch, the parameter vector <-> canonical vector round trip, the default
    start vector and the 75-slot stencil export against the oracle's Q."""
    from golden_cases import diff_form, grid_args
    from spdepy_gb300.grids import Grid
    from spdepy_gb300.spdes import SeparableModel, spde_init, stencil_offsets, stencil_to_csr
    g = load(name)
    ga = grid_args(g)
    grid = Grid(ga["x"], ga["y"], ga["t"], ga["extend"], ga["Nbs"])
    d = diff_form(g)
    mod = spde_init("seperable-spatial-temporal", grid, ani=d != "iso", ha=d == "ha", bc=int(g["bc"]))
    assert isinstance(mod, SeparableModel) and mod.diff == d
    par = np.asarray(g["par"], float)
    assert mod.initFit(g["y"], idx=g["idx"]).size == par.size
    c = mod.canonical(par)
    assert c.size == mod.layout.ncanon
    assert np.array_equal(mod.from_canonical_grad(c, par), par)
    Q = separable_oracle(g).makeQ(par).tocsr()
    n, Mx, Ny, T = Q.shape[0], grid.Mx, grid.Ny, grid.T
    k = np.arange(n)
    t, r = np.divmod(k, Mx * Ny)
    y, x = np.divmod(r, Mx)
    qv = np.zeros((n, 75))
    for s, (dx, dy, dt) in enumerate(stencil_offsets(T, 75)):
        ok = (x + dx >= 0) & (x + dx < Mx) & (y + dy >= 0) & (y + dy < Ny) & (t + dt >= 0) & (t + dt < T)
        qv[ok, s] = np.asarray(Q[k[ok], (((t + dt) * Ny + y + dy) * Mx + x + dx)[ok]]).ravel()
    assert abs(stencil_to_csr(grid, qv) - Q).max() == 0.0


@pytest.mark.parametrize("ext", [0, 1, 2, 3])
def test_grid_plumbing_on_extended_grids(ext):
    """Face velocities and bases on grids padded by `ext` cells against the
    reference's own output: assimilate_adv with the advBound ramp into the
    padding, evalAdv of a B-spline velocity (through the extended bsA), and the
    centre / face bases (grids/spat2Dtemp_regular_mesh.py:102-117,157-391)."""
    from oracle.spde_oracle import OracleGrid
    from spdepy_gb300.grids import Grid
    g = load("grid_adv.npz")
    M, N, T = (int(g[k]) for k in ("M", "N", "T"))
    args = (np.arange(M, dtype=float), np.arange(N, dtype=float), np.arange(T, dtype=float), ext or None)
    p = g["par_adv"]
    nb = p.size // 2
    for grid in (Grid(*args), OracleGrid(*args)):
        ww = grid.assimilate_adv(g["we"], g["wn"])
        assert np.allclose(ww, g[f"ww_e{ext}"], rtol=1e-14, atol=1e-15), type(grid)
        assert np.allclose(grid.bs, g[f"bs_e{ext}"], rtol=1e-12, atol=1e-14), type(grid)
        assert np.allclose(grid.bsH, g[f"bsH_e{ext}"], rtol=1e-12, atol=1e-14), type(grid)
    grid = Grid(*args)
    A = grid.bsA
    adv = np.stack([A[:, 0] @ p[:nb], A[:, 1] @ p[nb:], A[:, 2] @ p[:nb], A[:, 3] @ p[nb:]], axis=1)
    assert np.allclose(adv, g[f"adv_e{ext}"], rtol=1e-12, atol=1e-14)
    assert np.allclose(OracleGrid(*args).evalAdv(p), g[f"adv_e{ext}"], rtol=1e-12, atol=1e-14)


def test_updates_with_different_tau():
    """Two Model.update calls with different noise precisions accumulate
    Q += tau_k S_k^T S_k (reference model.py:120-127): the conditional means of
    the reference, without fixed effects (dense solves of the accumulated
    precision) and with them (block elimination through the border)."""
    from oracle.spde_oracle import OracleGrid, OracleModel
    from spdepy_gb300.fixed_effects import Border, update_step
    g = load("facade_tau.npz")
    M, N = int(g["M"]), int(g["N"])
    Q = OracleModel(OracleGrid(np.arange(M, dtype=float), np.arange(N, dtype=float)), "whittle-matern", "ani",
                    3).makeQ(g["par"]).toarray()
    taus = (float(g["tau1"]), float(g["tau2"]))
    A = Q.copy()
    mu = np.zeros(M * N)
    for k, tau in zip((1, 2), taus):
        idx, y = g[f"idx{k}"], g[f"y{k}"]
        np.add.at(A, (idx, idx), tau)
        b = np.zeros(M * N)
        np.add.at(b, idx, tau * (y - mu[idx]))
        mu = mu + np.linalg.solve(A, b)
        assert np.allclose(mu, g[f"plain_mu{k}"], rtol=1e-10, atol=1e-12 * np.abs(mu).max()), k
    Qref = sparse.csr_matrix((g["plain_Q_data"], g["plain_Q_indices"], g["plain_Q_indptr"]), shape=A.shape)
    assert abs(Qref - sparse.csr_matrix(A)).max() <= 1e-12 * abs(Qref).max()
    grid, mu = _fixed_effect_setup(dict(M=M, N=N, cov=g["cov"]), "cov")
    border = Border(grid.n, np.exp(np.log(np.array([0.01, 140.0]))))
    A = Q.copy()
    F = grid._fixed_effects()
    for k, tau in zip((1, 2), taus):
        idx, y = g[f"idx{k}"], g[f"y{k}"]
        nodes = grid.obs_nodes(idx)
        np.add.at(A, (nodes, nodes), tau)
        mu = update_step(border, lambda R: np.linalg.solve(A, R), mu, nodes, F[idx], y, tau)
        ref = g[f"cov_mu{k}"]
        assert np.allclose(mu, ref, rtol=1e-10, atol=1e-12 * np.abs(ref).max()), k


def test_fixed_effect_marginal_variances_formula():
    """The reference's qinv with fixed effects returns diag((S Q_aug S^T)^-1) for
    S = getS() = [I | X] (model.py:108-117); the facade computes it as the
    selected inverse of the lattice block A plus a Woodbury correction for the
    border.  Here both sides are dense on a small case."""
    from spdepy_gb300.fixed_effects import Border
    rng = np.random.default_rng(9)
    n, p = 40, 2
    R = rng.normal(size=(n, n))
    A0 = R @ R.T + n * np.eye(n)
    X = np.column_stack([np.ones(n), rng.uniform(0.5, 2.0, n)])
    border = Border(n, [0.3, 4.0])
    nodes = rng.choice(n, 15, replace=False)
    border.add(nodes, X[nodes], 7.0)
    A = A0.copy()
    np.add.at(A, (nodes, nodes), 7.0)
    Qaug = np.block([[A, border.B], [border.B.T, border.C]])
    S = np.hstack([np.eye(n), X])
    ref = np.diag(np.linalg.inv(S @ Qaug @ S.T))
    U = np.hstack([X, border.B])
    Y = np.linalg.solve(A, U)
    Winv = np.block([[np.zeros((p, p)), np.eye(p)], [np.eye(p), -border.C]])
    K = np.linalg.inv(Winv + U.T @ Y)
    got = np.diag(np.linalg.inv(A)) - np.einsum("ij,ij->i", Y @ K, Y)
    assert np.allclose(got, ref, rtol=1e-10, atol=0)
