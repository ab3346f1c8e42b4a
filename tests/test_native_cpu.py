"""CPU-only checks of the native library (loads, exports, symbolic analysis) and host logic."""
import os
import re

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def lib():
    from spdepy_gb300 import build, _native
    build.build()
    return _native.lib()


def test_exports_every_declared_symbol(lib):
    hdr = open(os.path.join(ROOT, "include", "spde_gb300.h")).read()
    names = set(re.findall(r"^\s*(?:int|const char\*)\s+(spde_\w+)\(", hdr, re.M))
    assert len(names) >= 18
    for n in names:
        assert hasattr(lib, n), n
    from spdepy_gb300._native import SIGNATURES
    assert names == set(SIGNATURES)


@pytest.mark.parametrize("dims", [(40, 40, 1), (12, 10, 5), (30, 28, 6), (7, 40, 3)])
def test_symbolic_structure(lib, dims):
    from spdepy_gb300 import _native
    perm, ns, nb, par = _native.symbolic_export(*dims, leaf_max=64)
    n = dims[0] * dims[1] * dims[2]
    assert np.array_equal(np.sort(perm), np.arange(n))
    assert ns.sum() == n
    roots = np.where(par < 0)[0]
    assert roots.size == 1 and nb[roots[0]] == 0
    assert np.all(par[par >= 0] > np.arange(par.size)[par >= 0])   # post-order


def test_symbolic_counts_config3(lib):
    from spdepy_gb300 import _native
    info = _native.symbolic_info(200, 200, 24)
    assert info.n == 960000
    assert 1e13 < info.factor_flops < 2e13
    assert info.max_front == 14400


def test_grid_bases_match_oracle():
    from oracle.spde_oracle import OracleGrid
    from spdepy_gb300.grids import Grid
    for args in [(np.arange(12.), np.arange(9.), np.arange(4.), None, 3), (np.arange(8.), np.arange(7.), np.arange(3.), 2, 3),
                 (np.arange(10.), np.arange(10.), None, None, 5)]:
        o = OracleGrid(*args)
        g = Grid(*args)
        assert np.allclose(g.bs, o.bs, atol=1e-14)
        assert np.allclose(g.bsH, o.bsH, atol=1e-14)
        if g.T > 1:
            c = np.random.default_rng(0).normal(size=2 * g.Nbs2)
            w_ref = o.evalAdv(c)
            w = np.stack([g.bsA[:, f, :] @ (c[:g.Nbs2] if f % 2 == 0 else c[g.Nbs2:]) for f in range(4)], axis=1)
            assert np.allclose(w, w_ref, atol=1e-13)


def test_layout_roundtrip():
    """Reference parameter vector -> canonical ABI vector -> back is the identity."""
    from golden_cases import diff_form, grid_args, load, model_cases
    from spdepy_gb300.grids import Grid
    from spdepy_gb300.spdes import _CLASSES
    for name in model_cases():
        g = load(name)
        ga = grid_args(g)
        grid = Grid(ga["x"], ga["y"], ga["t"], ga["extend"], ga["Nbs"])
        d = diff_form(g)
        mod0 = _CLASSES[("whittle-matern", d)](grid=grid.spatial(), bc=int(g["bc"])) if grid.T > 1 else None
        mod = _CLASSES[(str(g["family"]), d)](grid=grid, bc=int(g["bc"]), mod0=mod0,
                                              ww=g["ww"] if "ww" in g.files else None)
        par = g["par"]
        back = mod.from_canonical_grad(mod.canonical(par), par)
        assert np.array_equal(back, par), name


def test_oracle_exact_gradient_matches_fd():
    """The oracle's exact-trace gradient (true derivatives) is the derivative of its objective."""
    from golden_cases import load, oracle_model
    for name in ("advdiff_ani_bc1", "covadv_vardiff_bc3", "wm_ha_bc3", "varadv_vardiff_bc1"):
        g = load(name)
        om = oracle_model(g)
        om.derivative = "true"
        par = g["par"].astype(float)
        _, jac = om.loglike(par, g["y"], g["idx"], grad=True, exact=True)
        h = 1e-5
        for i in range(par.size):
            e = np.zeros_like(par); e[i] = h
            fd = (om.loglike(par + e, g["y"], g["idx"], grad=False) - om.loglike(par - e, g["y"], g["idx"], grad=False)) / (2 * h)
            assert abs(fd - jac[i]) <= 1e-6 * max(1.0, np.abs(jac).max()), (name, i, fd, jac[i])


def _descent_perm(Mx, Ny, T, leaf_max):
    """The device ordering's per-node descent (engine.cu, nd_perm_kernel),
    vectorised over nodes in numpy: every node follows the dissection tree by box
    arithmetic alone (cheapest thickness-2 cut across x or y, thickness-1 across
    t; children numbered first, then the separator; x fastest in a box)."""
    k = np.arange(Mx * Ny * T, dtype=np.int64)
    x, y, t = k % Mx, (k // Mx) % Ny, k // (Mx * Ny)
    box = np.tile(np.array([0, Mx, 0, Ny, 0, T], dtype=np.int64), (k.size, 1))
    base = np.zeros(k.size, dtype=np.int64)
    active = np.ones(k.size, dtype=bool)
    inf = np.iinfo(np.int64).max
    for _ in range(256):
        if not active.any():
            break
        b = box[active]
        a_, b_, c_ = b[:, 1] - b[:, 0], b[:, 3] - b[:, 2], b[:, 5] - b[:, 4]
        vol = a_ * b_ * c_
        cx = np.where(a_ >= 4, 2 * b_ * c_, inf)
        cy = np.where(b_ >= 4, 2 * a_ * c_, inf)
        ct = np.where((T > 1) & (c_ >= 3), a_ * b_, inf)
        cmin = np.minimum(cx, np.minimum(cy, ct))
        leaf = (vol <= leaf_max) | (cmin == inf)
        idx = np.where(active)[0]
        stop = idx[leaf]
        active[stop] = False
        go = ~leaf
        idx, b = idx[go], b[go]
        a_, b_, c_, cx, cy, cmin = a_[go], b_[go], c_[go], cx[go], cy[go], cmin[go]
        k1, k2, sp = b.copy(), b.copy(), b.copy()
        ax = cmin == cx
        ay = (~ax) & (cmin == cy)
        at = (~ax) & (~ay)
        m = b[:, 0] + (a_ - 2) // 2
        k1[ax, 1], sp[ax, 0], sp[ax, 1], k2[ax, 0] = m[ax], m[ax], m[ax] + 2, m[ax] + 2
        m = b[:, 2] + (b_ - 2) // 2
        k1[ay, 3], sp[ay, 2], sp[ay, 3], k2[ay, 2] = m[ay], m[ay], m[ay] + 2, m[ay] + 2
        m = b[:, 4] + (c_ - 1) // 2
        k1[at, 5], sp[at, 4], sp[at, 5], k2[at, 4] = m[at], m[at], m[at] + 1, m[at] + 1

        def inside(q, j):
            return ((x[j] >= q[:, 0]) & (x[j] < q[:, 1]) & (y[j] >= q[:, 2]) & (y[j] < q[:, 3]) &
                    (t[j] >= q[:, 4]) & (t[j] < q[:, 5]))
        v1 = (k1[:, 1] - k1[:, 0]) * (k1[:, 3] - k1[:, 2]) * (k1[:, 5] - k1[:, 4])
        v2 = (k2[:, 1] - k2[:, 0]) * (k2[:, 3] - k2[:, 2]) * (k2[:, 5] - k2[:, 4])
        in1, in2 = inside(k1, idx), inside(k2, idx)
        sep = ~(in1 | in2)
        box[idx[in1]] = k1[in1]
        base[idx[in2]] += v1[in2]
        box[idx[in2]] = k2[in2]
        base[idx[sep]] += v1[sep] + v2[sep]
        box[idx[sep]] = sp[sep]
        active[idx[sep]] = False
    wa, wb = box[:, 1] - box[:, 0], box[:, 3] - box[:, 2]
    return base + ((t - box[:, 4]) * wb + (y - box[:, 2])) * wa + (x - box[:, 0])


@pytest.mark.parametrize("dims,leaf", [((40, 40, 1), 64), ((12, 10, 5), 64), ((7, 5, 3), 16), ((33, 17, 9), 64),
                                       ((41, 29, 6), 128), ((64, 48, 12), 128), ((5, 4, 2), 8)])
def test_device_ordering_rule_matches_symbolic_analysis(lib, dims, leaf):
    """The per-node descent the device ordering kernel performs reproduces the
    host symbolic analysis's permutation exactly (the plan also compares the two
    on the device whenever it is built)."""
    from spdepy_gb300 import _native
    perm, _, _, _ = _native.symbolic_export(*dims, leaf_max=leaf)
    assert np.array_equal(_descent_perm(*dims, leaf), perm)
