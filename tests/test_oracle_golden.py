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
