"""Oracle (test infrastructure only): CPU FP64 restatement of spdepy's inference path.

It restates, in numpy/scipy, what the reference computes for one model object:
grid geometry and B-spline bases, theta -> fields, the stencils, the precision
Q(theta), its analytic derivatives dQ_i, the log-likelihood with the reference's
Hutchinson gradient (and the exact-trace gradient it estimates), sampling and the
conditional mean.  Parity of this restatement is pinned against fixtures that the
reference itself produced (``tests/golden/make_golden.py``).

Reference files followed (paths inside the reference project):
  grids/spat2Dtemp_regular_mesh.py:35-58,86-95,102-275,277-391   Grid
  grids/spatial2D_regular_mesh.py                                spatial Grid
  spdes/whittle_matern*2D.py, spdes/var_whittle_matern*2D.py      spatial models
  spdes/{,var_,cov_}advection_{,var_}{,i,ha_}diffusion2D.py       spatio-temporal models
  spdes/seperable_spatial_temporal{,_idiffusion}2D.py              separable space-time models
  model.py:73-87,120-127                                          sample / update

Only tests/, ``__graft_entry__.smoke()`` and ``bench.py``'s CPU-baseline leg
import this module.  It is test infrastructure, never the product path.
"""
from __future__ import annotations

import numpy as np
import scipy.linalg as sla
from scipy import sparse
from scipy.sparse import linalg as spla

from . import stencils as st


# ----------------------------------------------------------------------------- grid
class OracleGrid:
    """Regular 2-D (or 2-D x time) grid with the reference's degree-2 B-spline bases.

    Restates ``grids/spat2Dtemp_regular_mesh.py:119-275`` (``setGrid``, ``basis``,
    ``basisN/H/A``, ``evalB/BH/Adv``) and ``:86-117`` (``n2e``, ``extend``).
    """

    def __init__(self, x, y, t=None, extend=None, Nbs=3):
        self.x = np.asarray(x, dtype=float)
        self.y = np.asarray(y, dtype=float)
        self.temporal = t is not None
        self.t = np.asarray(t, dtype=float) if t is not None else np.zeros(1)
        self.M, self.N = self.x.size, self.y.size
        self.T = self.t.size
        self.hx = (self.x.max() - self.x.min()) / (self.M - 1)   # Q12
        self.hy = (self.y.max() - self.y.min()) / (self.N - 1)
        self.dt = (self.t.max() - self.t.min()) / (self.T - 1) if self.T > 1 else 1.0
        self.V = self.hx * self.hy
        sx, sy = np.meshgrid(self.x, self.y)
        self.sx, self.sy = sx.ravel(), sy.ravel()
        self.Nbs = Nbs
        self.Nbs2 = Nbs * Nbs
        self.Ne = 0
        self.isExtended = False
        self.bs = self._basisN()
        self.bsH = self._basis_faces((0, 1, 2, 3))
        # basisA is computed once, before any extension (spat2Dtemp_regular_mesh.py:142-149)
        self.bsA = self._basis_faces((1, 3, 0, 2)) if self.temporal else None
        if extend is not None:
            self._extend(extend)
        self.Mx, self.Ny = self.M + 2 * self.Ne, self.N + 2 * self.Ne
        self.Ns = self.Mx * self.Ny
        self.n = self.Ns * self.T
        self._Ae = None

    # spat2Dtemp_regular_mesh.py:102-117
    def _extend(self, e):
        self.xe = np.hstack([np.linspace(self.x[0] - e * self.hx, self.x[0], e + 1)[:-1], self.x,
                             np.linspace(self.x[-1], self.x[-1] + e * self.hx, e + 1)[1:]])
        self.ye = np.hstack([np.linspace(self.y[0] - e * self.hy, self.y[0], e + 1)[:-1], self.y,
                             np.linspace(self.y[-1], self.y[-1] + e * self.hy, e + 1)[1:]])
        sxe, sye = np.meshgrid(self.xe, self.ye)
        self.sxe, self.sye = sxe.ravel(), sye.ravel()
        self.isExtended = True
        self.Ne = e
        self.bs = self._basisN()
        self.bsH = self._basis_faces((0, 1, 2, 3))

    # spat2Dtemp_regular_mesh.py:157-187
    def _basis1d(self, dx=0.0, dy=0.0, d=2):
        if self.isExtended:
            tx, ty = self.sxe + dx, self.sye + dy
        else:
            tx, ty = self.sx + dx, self.sy + dy
        if dx != 0 or dy != 0:
            xmin, xmax = self.sx.min() - self.hx / 2, self.sx.max() + self.hx / 2
            ymin, ymax = self.sy.min() - self.hy / 2, self.sy.max() + self.hy / 2
        else:
            xmin, xmax, ymin, ymax = self.sx.min(), self.sx.max(), self.sy.min(), self.sy.max()
        nb = self.Nbs
        kx = np.linspace(xmin - 2 * (xmax - xmin) / nb, xmax + 2 * (xmax - xmin) / nb, nb + 5)
        ky = np.linspace(ymin - 2 * (ymax - ymin) / nb, ymax + 2 * (ymax - ymin) / nb, nb + 5)

        def cox_de_boor(tv, kv):
            last = kv.size - 2
            B = np.stack([(((tv >= kv[i]) & (tv < kv[i + 1])) |
                           ((tv >= kv[i]) & (tv <= kv[i + 1]) & (i == last))) * 1.0
                          for i in range(kv.size - 1)], axis=1)
            for r in range(1, d + 1):
                Bn = np.zeros((tv.size, kv.size - r - 1))
                for i in range(kv.size - r - 1):
                    Bn[:, i] = ((tv - kv[i]) / (kv[i + r] - kv[i]) * B[:, i]
                                + (kv[i + r + 1] - tv) / (kv[i + r + 1] - kv[i + 1]) * B[:, i + 1])
                B = Bn
            # merged end functions (spat2Dtemp_regular_mesh.py:185-186)
            return np.hstack([(B[:, 0] + B[:, 1])[:, None], B[:, 2:-2], (B[:, -2] + B[:, -1])[:, None]])

        return cox_de_boor(tx, kx), cox_de_boor(ty, ky)

    def _basisN(self):
        bx, by = self._basis1d()
        nb = self.Nbs
        bs = np.zeros((bx.shape[0], nb * nb))
        for i in range(nb):
            for j in range(nb):
                bs[:, i * nb + j] = bx[:, j] * by[:, i]
        return bs

    def _basis_faces(self, order):
        """Face bases; ``order[f]`` says which shift face f uses
        (0: -hx/2, 1: +hx/2, 2: -hy/2, 3: +hy/2).  basisH uses (0,1,2,3) = W,E,S,N
        and basisA uses (1,3,0,2) so its faces are E,N,W,S (:201-249)."""
        shifts = {0: (-self.hx / 2, 0.0), 1: (self.hx / 2, 0.0), 2: (0.0, -self.hy / 2), 3: (0.0, self.hy / 2)}
        nb = self.Nbs
        out = None
        for f, s in enumerate(order):
            bx, by = self._basis1d(*shifts[s])
            if out is None:
                out = np.zeros((bx.shape[0], 4, nb * nb))
            for i in range(nb):
                for j in range(nb):
                    out[:, f, i * nb + j] = bx[:, j] * by[:, i]
        return out

    # spat2Dtemp_regular_mesh.py:251-275
    def evalB(self, par):
        return self.bs @ par

    def evalBH(self, par):
        return self.bsH @ par

    def evalAdv(self, par):
        nb2 = self.Nbs2
        b = self.bsA
        res = np.stack([b[:, 0, :] @ par[:nb2], b[:, 1, :] @ par[nb2:], b[:, 2, :] @ par[:nb2],
                        b[:, 3, :] @ par[nb2:]], axis=1)
        return self.advBound(res)

    # spat2Dtemp_regular_mesh.py:347-391
    def _ae(self):
        if self._Ae is None:
            M, N, Ne = self.M, self.N, self.Ne
            Ae = np.zeros((self.Ns, M * N))
            for i in range(M + 2 * Ne):
                for j in range(N + 2 * Ne):
                    k = i + j * (M + 2 * Ne)
                    if i < Ne and j < Ne:
                        Ae[k, 0] = j / Ne if i >= j else i / Ne
                        continue
                    if i >= M + Ne and j >= N + Ne:
                        Ae[k, M * N - 1] = ((N + 2 * Ne - 1 - j) / Ne if N - j <= M - i
                                            else (M + 2 * Ne - 1 - i) / Ne)
                        continue
                    if i >= M + Ne and j < Ne:
                        Ae[k, M - 1] = (M + 2 * Ne - 1 - i) / Ne if M + 2 * Ne - 1 - i <= j else j / Ne
                        continue
                    if i < Ne and j >= N + Ne:
                        Ae[k, M * (N - 1)] = i / Ne if i <= N + 2 * Ne - 1 - j else (N + 2 * Ne - 1 - j) / Ne
                        continue
                    if i < Ne:
                        Ae[k, (j - Ne) * M] = i / Ne
                    elif i >= M + Ne:
                        Ae[k, M - 1 + (j - Ne) * M] = (M + 2 * Ne - 1 - i) / Ne
                    if j < Ne:
                        Ae[k, i - Ne] = j / Ne
                    elif j >= N + Ne:
                        Ae[k, i - Ne + (N - 1) * M] = (N + 2 * Ne - 1 - j) / Ne
                    if Ne <= i < M + Ne and Ne <= j < N + Ne:
                        Ae[k, (i - Ne) + (j - Ne) * M] = 1
            self._Ae = Ae
        return self._Ae

    def advBound(self, ww):
        return self._ae() @ ww if self.isExtended else ww

    # spat2Dtemp_regular_mesh.py:277-344
    def assimilate_adv(self, we, wn):
        M, N = self.M, self.N
        k = np.arange(M * N)
        j, i = np.divmod(k, M)
        e_idx = np.where(i + 1 == M, k, k + 1)
        w_idx = np.where(i == 0, k, k - 1)
        n_idx = np.where(j + 1 == N, k, k + M)
        s_idx = np.where(j == 0, k, k - M)
        ww = np.zeros((M * N, 4))
        ww[:, 0] = (we + we[e_idx]) / 2
        ww[:, 1] = (wn + wn[n_idx]) / 2
        ww[:, 2] = (we + we[w_idx]) / 2
        ww[:, 3] = (wn + wn[s_idx]) / 2
        return self._ae() @ ww if self.isExtended else ww

    # spat2Dtemp_regular_mesh.py:86-95
    def n2e(self, idx):
        idx = np.asarray(idx, dtype=np.int64)
        M, N, Ne = self.M, self.N, self.Ne
        t, r = np.divmod(idx, M * N)
        j, i = np.divmod(r, M)
        return (i + Ne) + (j + Ne) * (M + 2 * Ne) + t * (M + 2 * Ne) * (N + 2 * Ne)

    def getS(self, idx=None):
        """Observation matrix: selected identity rows (:35-58)."""
        if idx is None:
            idx = np.arange(self.M * self.N * self.T)
        cols = self.n2e(idx)
        m = cols.size
        return sparse.csc_matrix((np.ones(m), (np.arange(m), cols)), shape=(m, self.n))


# ------------------------------------------------------------------ model families
FAMILIES = ("whittle-matern", "var-whittle-matern", "advection-diffusion", "advection-var-diffusion",
            "var-advection-diffusion", "var-advection-var-diffusion", "cov-advection-diffusion",
            "cov-advection-var-diffusion")


class Family:
    """Parameter layout of one reference model class (its ``setPars``).

    kappa/gamma/v are constant ("c") or B-spline fields ("v"); advection is "none",
    constant ("c"), B-spline field ("v") or a given field scaled by lambda ("cov").
    ``diff`` is "iso" (gamma I), "ani" (gamma I + v v^T) or "ha" (half-angle form).
    """

    def __init__(self, name, diff, Nbs2=9):
        if name not in FAMILIES:
            raise ValueError(f"unknown family {name}")
        if diff not in ("iso", "ani", "ha"):
            raise ValueError(f"unknown diffusion form {diff}")
        self.name, self.diff = name, diff
        self.spatial = name in ("whittle-matern", "var-whittle-matern")
        varH = name in ("var-whittle-matern", "advection-var-diffusion", "var-advection-var-diffusion",
                        "cov-advection-var-diffusion")
        self.varH = varH
        if self.spatial:
            self.adv = "none"
        elif name.startswith("cov-"):
            self.adv = "cov"
        elif name.startswith("var-advection"):
            self.adv = "v"
        else:
            self.adv = "c"
        np_ = Nbs2 if varH else 1
        self.np_h = np_
        npw = Nbs2 if self.adv == "v" else 1
        sl = {}
        o = 0
        for key in ("kappa", "gamma") + (() if diff == "iso" else ("vx", "vy")):
            sl[key] = slice(o, o + np_)
            o += np_
        if self.adv == "c" or self.adv == "v":
            sl["wx"] = slice(o, o + npw); o += npw
            sl["wy"] = slice(o, o + npw); o += npw
        elif self.adv == "cov":
            sl["lamb"] = slice(o, o + 1); o += 1
        if not self.spatial:
            sl["sigma"] = slice(o, o + 1); o += 1
        self.sl = sl
        self.nself = o          # parameters before tau (and before mod0's)
        self.nbase = o + 1      # with tau


def h_tensor(diff, gamma, vx, vy):
    """H = gamma I, gamma I + v v^T, or the half-angle form
    gamma (cosh|v| I + sinh|v|/|v| [[vx, vy], [vy, -vx]]) (whittle_matern_ha2D.py:73-82).
    Arrays broadcast; returns (..., 2, 2)."""
    gamma, vx, vy = np.broadcast_arrays(np.asarray(gamma, float), np.asarray(vx, float), np.asarray(vy, float))
    H = np.zeros(gamma.shape + (2, 2))
    if diff == "iso":
        H[..., 0, 0] = gamma
        H[..., 1, 1] = gamma
    elif diff == "ani":
        H[..., 0, 0] = gamma + vx * vx
        H[..., 0, 1] = vx * vy
        H[..., 1, 0] = vx * vy
        H[..., 1, 1] = gamma + vy * vy
    else:
        aV = np.sqrt(vx ** 2 + vy ** 2)
        ch = (np.exp(aV) + np.exp(-aV)) / 2
        sh = (np.exp(aV) - np.exp(-aV)) / 2
        r = sh / aV
        H[..., 0, 0] = gamma * (ch + r * vx)
        H[..., 0, 1] = gamma * r * vy
        H[..., 1, 0] = gamma * r * vy
        H[..., 1, 1] = gamma * (ch - r * vx)
    return H


def h_dtensor(diff, gamma, vx, vy, which):
    """Reference analytic dH for 'gamma' (per log gamma), 'vx', 'vy'
    (whittle_matern_anisotropic2D.py:85-101, whittle_matern_ha2D.py:89-101)."""
    gamma, vx, vy = np.broadcast_arrays(np.asarray(gamma, float), np.asarray(vx, float), np.asarray(vy, float))
    if which == "gamma":
        if diff == "ha":
            return h_tensor(diff, gamma, vx, vy)
        dH = np.zeros(gamma.shape + (2, 2))
        dH[..., 0, 0] = gamma
        dH[..., 1, 1] = gamma
        return dH
    if diff == "ani":
        dH = np.zeros(gamma.shape + (2, 2))
        if which == "vx":
            dH[..., 0, 0] = 2 * vx
            dH[..., 0, 1] = vy
            dH[..., 1, 0] = vy
        else:
            dH[..., 1, 1] = 2 * vy
            dH[..., 0, 1] = vx
            dH[..., 1, 0] = vx
        return dH
    # half-angle
    aV = np.sqrt(vx ** 2 + vy ** 2)
    ch = (np.exp(aV) + np.exp(-aV)) / 2
    sh = (np.exp(aV) - np.exp(-aV)) / 2
    mV = np.zeros(gamma.shape + (2, 2))
    mV[..., 0, 0] = vx
    mV[..., 0, 1] = vy
    mV[..., 1, 0] = vy
    mV[..., 1, 1] = -vx
    comp = vx if which == "vx" else vy
    E = np.zeros(gamma.shape + (2, 2))
    if which == "vx":
        E[..., 0, 0] = 1.0
        E[..., 1, 1] = -1.0
    else:
        E[..., 0, 1] = 1.0
        E[..., 1, 0] = 1.0
    I2 = np.zeros(gamma.shape + (2, 2))
    I2[..., 0, 0] = 1.0
    I2[..., 1, 1] = 1.0
    g = (gamma / aV)[..., None, None]
    return g * ((comp * sh)[..., None, None] * I2 + (comp / aV * (ch - sh / aV))[..., None, None] * mV
                + sh[..., None, None] * E)


class OracleModel:
    """One SPDE model object restated on CPU (FP64).

    ``mod0_diff`` is the diffusion form of the Whittle-Matern initial-field model
    of spatio-temporal families; ``mod0_par`` its default parameters (used when
    ``par`` does not carry them, as in the reference's ``mod0.Q`` branch).
    """

    def __init__(self, grid: OracleGrid, family, diff, bc, ww=None, mod0_diff=None, mod0_par=None):
        self.grid = grid
        self.fam = Family(family, diff, grid.Nbs2)
        self.bc = bc
        self.ww = None if ww is None else np.asarray(ww, dtype=float)
        if not self.fam.spatial:
            self.mod0 = Family("whittle-matern", mod0_diff or diff)
            # default initial-field parameters (whittle_matern2D.py:24, whittle_matern_anisotropic2D.py:24)
            default0 = ([-1.0, -1.0, np.log(100)] if self.mod0.diff == "iso"
                        else [-1.0, -1.0, 0.1, 0.1, np.log(100)])
            self.mod0_par = np.asarray(mod0_par if mod0_par is not None else default0, dtype=float)
        self.derivative = "reference"

    # ------------------------------------------------------------ theta -> fields
    def split(self, par):
        par = np.asarray(par, dtype=float)
        f = self.fam
        p = {k: par[s] for k, s in f.sl.items()}
        p["tau"] = par[-1]
        p0 = None
        if not f.spatial:
            if par.size > f.nbase:
                p0 = par[f.nself:]
            else:
                p0 = self.mod0_par
        return p, p0

    def fields(self, par):
        """kappa per cell, H per cell and face (or one 2x2), w per face (or 2)."""
        g, f = self.grid, self.fam
        p, _ = self.split(par)
        if f.varH:
            kappa = np.exp(g.evalB(p["kappa"]))
            gamma = np.exp(g.evalBH(p["gamma"]))
            vx = g.evalBH(p["vx"]) if "vx" in p else np.zeros_like(gamma)
            vy = g.evalBH(p["vy"]) if "vy" in p else np.zeros_like(gamma)
        else:
            kappa = np.exp(p["kappa"][0])
            gamma = np.exp(p["gamma"][0])
            vx = p["vx"][0] if "vx" in p else 0.0
            vy = p["vy"][0] if "vy" in p else 0.0
        H = h_tensor(f.diff, gamma, vx, vy)
        w = None
        if f.adv == "c":
            w = np.array([p["wx"][0], p["wy"][0]])
        elif f.adv == "v":
            w = g.evalAdv(np.hstack([p["wx"], p["wy"]]))
        elif f.adv == "cov":
            w = p["lamb"][0] * self.ww
        return dict(kappa=kappa, gamma=gamma, vx=vx, vy=vy, H=H, w=w)

    # ------------------------------------------------------------------ stencils
    def Ah(self, H):
        g = self.grid
        r, c, v = st.diffusion_triplets(g.Mx, g.Ny, H, g.hx, g.hy, self.bc, field=self.fam.varH)
        return st.to_csc(g.Mx, g.Ny, r, c, v)

    def Aw(self, w, diff=3, dw=None):
        g = self.grid
        if self.fam.adv == "c":
            r, c, v = st.advection_const_triplets(g.Mx, g.Ny, w, g.hx, g.hy, self.bc, diff)
            return st.to_csc(g.Mx, g.Ny, r, c, v)
        safe = getattr(self, "derivative", "reference") == "true"
        r, c, v = st.advection_field_triplets(g.Mx, g.Ny, w, g.hx, g.hy, self.bc, diff, dw, safe_sign=safe)
        return st.to_csc(g.Mx, g.Ny, r, c, v, nan_to_zero=(self.fam.adv == "v"))

    # ---------------------------------------------------------------- precision
    def _wm_Q(self, fam, par):
        """Spatial Whittle-Matern precision Q = A^T V^-1 A, A = V kappa - A_H
        (whittle_matern_anisotropic2D.py:59-75)."""
        sub = OracleModel.__new__(OracleModel)
        sub.grid, sub.fam, sub.bc, sub.ww = self.grid, fam, self.bc, None
        fl = sub.fields(par)
        g = self.grid
        Dk = sparse.diags(np.broadcast_to(fl["kappa"], (g.Ns,)).astype(float))
        A = (g.V * Dk - sub.Ah(fl["H"])).tocsc()
        return (A.T @ A / g.V).tocsc(), A, fl, sub

    def parts(self, par):
        """Spatial building blocks (A, Qs, Q0, sigma) of a spatio-temporal model
        (advection_diffusion2D.py:86-110, var_advection_var_diffusion2D.py:83-109)."""
        g, f = self.grid, self.fam
        p, p0 = self.split(par)
        fl = self.fields(par)
        kap = np.broadcast_to(fl["kappa"], (g.Ns,)).astype(float)
        Dk = sparse.diags(kap)
        As = g.V * Dk
        Qs = (As.T @ As / g.V).tocsc()
        A = g.V * sparse.eye(g.Ns) + (g.V * Dk - self.Ah(fl["H"])) * g.dt
        if f.adv != "none":
            A = A + self.Aw(fl["w"]) * g.dt
        A = A.tocsc()
        Q0 = self._wm_Q(self.mod0, p0)[0]
        sigma = np.exp(p["sigma"][0])
        return dict(A=A, Qs=Qs, Q0=Q0, sigma=sigma, fields=fl, kappa=kap)

    @staticmethod
    def _stack(g, d0, dmid, dlast, off, scale):
        """Block-tridiagonal assembly of T time blocks (advection_diffusion2D.py:112-116);
        built in one pass (the reference's re-stacking is quadratic in T)."""
        T = g.T
        blocks = [[None] * T for _ in range(T)]
        for t in range(T):
            if t == 0:
                blocks[t][t] = d0
            elif t == T - 1:
                blocks[t][t] = dlast
            else:
                blocks[t][t] = dmid
            if t + 1 < T:
                blocks[t][t + 1] = off
                blocks[t + 1][t] = off.T
        return (sparse.bmat(blocks, format="csc") * scale).tocsc()

    def makeQ(self, par):
        g, f = self.grid, self.fam
        if f.spatial:
            return self._wm_Q(f, np.asarray(par, float))[0]
        pt = self.parts(par)
        A, Qs, Q0, sigma = pt["A"], pt["Qs"], pt["Q0"], pt["sigma"]
        iV = 1.0 / g.V
        QsWA = (Qs @ A * iV).tocsc()
        mid = (A.T @ QsWA * iV).tocsc()
        if g.T == 1:
            raise ValueError("spatio-temporal model needs T >= 2")
        d0 = (sigma * g.dt * Q0 + Qs).tocsc()
        return self._stack(g, d0, mid + Qs, mid, -QsWA, 1.0 / (g.dt * sigma))

    # ------------------------------------------------------- analytic derivatives
    def _dA_list(self, par):
        """(name, dA, dQs) for every self parameter except sigma, tau and mod0,
        mirroring the reference's makeQ(grad=True)."""
        g, f = self.grid, self.fam
        p, _ = self.split(par)
        fl = self.fields(par)
        out = []
        kap = np.broadcast_to(fl["kappa"], (g.Ns,)).astype(float)
        sp_scale = 1.0 if f.spatial else g.dt
        # kappa
        for i in range(f.np_h):
            dk = g.bs[:, i] * kap if f.varH else kap
            dA = g.V * sparse.diags(dk) * sp_scale
            dAs = g.V * sparse.diags(dk)
            dQs = None if f.spatial else ((dAs.T @ (g.V * sparse.diags(kap)) + (g.V * sparse.diags(kap)).T @ dAs)
                                          / g.V).tocsc()
            out.append(("kappa", dA.tocsc(), dQs))
        # gamma, vx, vy
        for key in ("gamma", "vx", "vy"):
            if key not in p:
                continue
            base = h_dtensor(f.diff, fl["gamma"], fl["vx"], fl["vy"], key)
            for i in range(f.np_h):
                dH = base * g.bsH[:, :, i][:, :, None, None] if f.varH else base
                out.append((key, (-self.Ah(dH) * sp_scale).tocsc(), None))
        if f.adv == "c":
            for d, key in ((1, "wx"), (2, "wy")):
                dA = self.Aw(fl["w"], diff=d)
                if self.derivative == "true" and self.bc == 1:
                    dA = self._true_dAcw(fl["w"], d)
                out.append((key, (dA * g.dt).tocsc(), None))
        elif f.adv == "v":
            nb2 = g.Nbs2
            for i in range(2 * nb2):
                e = np.zeros(2 * nb2)
                e[i] = 1.0
                dws = g.evalAdv(e)
                out.append(("wx" if i < nb2 else "wy",
                            (self.Aw(fl["w"], diff=1 if i < nb2 else 2, dw=dws) * g.dt).tocsc(), None))
        elif f.adv == "cov":
            if self.derivative == "true":
                lam = p["lamb"][0]
                dA = self.Aw(np.sign(lam) * self.ww) if lam != 0 else self.Aw(self.ww)
            else:
                dA = self.Aw(self.ww)
            out.append(("lamb", (dA * g.dt).tocsc(), None))
        return out

    def _true_dAcw(self, w, d):
        """d/dw of the constant-velocity bc=1 stencil: the boundary correction
        -|w|h/2 differentiates to -sign(w)h/2 (the reference keeps -|w|h/2)."""
        g = self.grid
        r, c, v = st.advection_const_triplets(g.Mx, g.Ny, w, g.hx, g.hy, 1, d)
        M, N = g.Mx, g.Ny
        i = np.tile(np.arange(M), N)
        j = np.repeat(np.arange(N), M)
        v = v.reshape(-1, 5).copy()
        comp = w[d - 1]
        h = g.hy if d == 1 else g.hx
        bnd = ((i == 0) | (i == M - 1)) if d == 1 else ((j == 0) | (j == N - 1))
        other = ((j == 0) | (j == N - 1)) if d == 1 else ((i == 0) | (i == M - 1))
        wo = w[2 - d]
        # undo the reference's -|w_d|h/2 and -|w_o|h_o/2 and apply the derivative
        v[bnd, 0] += abs(comp) * h / 2 - np.sign(comp) * h / 2
        ho = g.hx if d == 1 else g.hy
        v[other, 0] += abs(wo) * ho / 2
        return st.to_csc(M, N, r, c, v.ravel())

    def dQ_list(self, par):
        """All dQ_i (self parameters, sigma, mod0 parameters), as the reference
        builds them (advection_diffusion2D.py:119-183; spatial: whittle_matern_
        anisotropic2D.py:77-101)."""
        g, f = self.grid, self.fam
        par = np.asarray(par, float)
        if f.spatial:
            Q, A, fl, _ = self._wm_Q(f, par)
            return [(dA.T @ A + A.T @ dA).tocsc() / g.V for _, dA, _ in self._dA_list(par)]
        pt = self.parts(par)
        A, Qs, sigma = pt["A"], pt["Qs"], pt["sigma"]
        iV = 1.0 / g.V
        sc = 1.0 / (g.dt * sigma)
        out = []
        for _, dA, dQs in self._dA_list(par):
            QsWdA = (Qs @ dA * iV).tocsc()
            mid = (dA.T @ (Qs @ A * iV) * iV + A.T @ QsWdA * iV).tocsc()
            if dQs is not None:
                off = -(dQs @ A * iV) - QsWdA
                mid = mid + (A.T @ (dQs @ A * iV) * iV)
                d0, dmid, dlast = dQs, mid + dQs, mid
            else:
                off = -QsWdA
                d0 = sparse.csc_matrix((g.Ns, g.Ns))
                dmid, dlast = mid, mid
            out.append(self._stack(g, d0.tocsc(), dmid.tocsc(), dlast.tocsc(), off.tocsc(), sc))
        # log sigma
        QsWA = (Qs @ A * iV).tocsc()
        midS = (A.T @ QsWA * iV).tocsc()
        out.append(-self._stack(g, Qs, midS + Qs, midS, -QsWA, sc))
        # mod0 parameters, only when par carries them
        if par.size > f.nbase:
            _, p0 = self.split(par)
            sub = OracleModel.__new__(OracleModel)
            sub.grid, sub.fam, sub.bc, sub.ww, sub.derivative = self.grid, self.mod0, self.bc, None, "reference"
            for dQ0 in sub.dQ_list(p0):
                z = sparse.csc_matrix((g.Ns, g.Ns))
                out.append(self._stack(g, dQ0, z, z, z, 1.0))
        return out

    # ----------------------------------------------------------- factor / solve
    @staticmethod
    def factor(Q):
        return DenseOrSparseFactor(Q)

    def loglike(self, par, y, idx, grad=True, nh1=100, seed=None, exact=False):
        """Objective and gradient as in the reference's logLike
        (advection_diffusion2D.py:187-223).  With ``exact=True`` the Hutchinson
        traces are replaced by the exact traces tr(Q^-1 dQ) they estimate."""
        g = self.grid
        par = np.asarray(par, float)
        y = np.asarray(y, float)
        r = 1 if y.ndim == 1 else y.shape[1]
        Y = y.reshape(-1, r)
        tau = np.exp(par[-1])
        S = g.getS(idx)
        m = S.shape[0]
        Q = self.makeQ(par)
        Qc = (Q + (S.T @ S) * tau).tocsc()
        Fq, Fc = self.factor(Q), self.factor(Qc)
        mu = Fc.solve(S.T @ Y * tau)
        like = (0.5 * Fq.logdet() * r + m * r * np.log(tau) / 2 - 0.5 * Fc.logdet() * r
                - 0.5 * (mu * (Q @ mu)).sum() - tau / 2 * ((Y - S @ mu) ** 2).sum())
        f = -like / (m * r)
        if not grad:
            return f
        dQ = self.dQ_list(par)
        gpar = np.zeros(par.size)
        STS = (S.T @ S).tocsc()
        if exact:
            Zq, Zc = Fq.inverse(), Fc.inverse()
            Dz = Zq - Zc
            for i, d in enumerate(dQ):
                gpar[i] = 0.5 * r * (d.multiply(Dz)).sum() - 0.5 * (mu * (d @ mu)).sum()
            gpar[-1] = m * r / 2 - 0.5 * r * tau * (STS.multiply(Zc)).sum() - tau / 2 * ((Y - S @ mu) ** 2).sum()
        else:
            if seed is not None:
                np.random.seed(seed)
            V = (2 * np.random.randint(1, 3, g.n * nh1) - 3).reshape(g.n, nh1)
            TrQ = Fq.solve(V)
            TrQc = Fc.solve(V)
            for i, d in enumerate(dQ):
                gpar[i] = 0.5 * ((TrQ - TrQc) * (d @ V)).sum() * r / nh1 - 0.5 * (mu * (d @ mu)).sum()
            gpar[-1] = (m * r / 2 - 0.5 * (TrQc * (STS * tau @ V)).sum() * r / nh1
                        - tau / 2 * ((Y - S @ mu) ** 2).sum())
        return f, -gpar / (m * r)

    def conditional_mean(self, par, y, idx, tau=None):
        """mu_c = tau Q_c^-1 S^T y (advection_diffusion2D.py:192-194; model.py:120-127 with mu = 0)."""
        g = self.grid
        par = np.asarray(par, float)
        tau = np.exp(par[-1]) if tau is None else tau
        S = g.getS(idx)
        Q = self.makeQ(par)
        Qc = (Q + (S.T @ S) * tau).tocsc()
        return self.factor(Qc).solve(S.T @ np.asarray(y, float) * tau)


class SeparableOracleModel(OracleModel):
    """Separable space-time model Q = Qt (x) Qs, restated on CPU (FP64).

    Qs is the spatially varying Whittle-Matern precision A^T V^-1 A with
    A = V kappa - A_H(H) (the var-Whittle-Matern spatial part,
    spdes/var_whittle_matern_anisotropic2D.py:66-82), with B-spline fields for
    kappa, gamma and, for the anisotropic form, vx and vy (H = gamma I + v v^T per
    face; the isotropic form has H = gamma I).  Qt is a tridiagonal AR(1)
    precision over the T time steps, in one of two parametrisations:

    * ``temporal="rho"`` (spdes/seperable_spatial_temporal2D.py:64-83,186-212):
      rho = exp(par[ns]), Qt_tt = 1 / (1 - rho^2) at both ends and
      (1 + rho^2) / (1 - rho^2) inside, Qt_t,t+1 = -rho / (1 - rho^2);
      parameters kappa, gamma, vx, vy, log rho, log tau.
    * ``temporal="a-sigma"`` (spdes/seperable_spatial_temporal_idiffusion2D.py:
      63-103,166-189): a = par[ns], sigma = exp(par[ns + 1]), Qt_tt = sigma at both
      ends and (1 + a^2) sigma inside, Qt_t,t+1 = -a sigma; parameters kappa,
      gamma, a, log sigma, log tau.  The reference fills Qt in a loop over
      range(10), so its class only works for T = 10; this restatement follows the
      evident formula for any T.

    dQ follows the reference's order: every spatial parameter as Qt (x) dQs_i,
    then the temporal ones (Qt' (x) Qs, and Q itself for log sigma).
    """

    def __init__(self, grid: OracleGrid, diff, bc, temporal="rho"):
        if temporal not in ("rho", "a-sigma"):
            raise ValueError(f"unknown temporal parametrisation {temporal}")
        if grid.T < 2:
            raise ValueError("a separable space-time model needs T >= 2")
        self.grid = grid
        self.fam = Family("var-whittle-matern", diff, grid.Nbs2)  # the spatial parameter layout
        self.bc = bc
        self.ww = None
        self.derivative = "reference"
        self.temporal = temporal
        self.ns = self.fam.nself  # spatial parameters, before the temporal ones

    def _spatial(self, par):
        """The spatial parameters in the var-Whittle-Matern layout (tau last, unused by Qs)."""
        par = np.asarray(par, float)
        return np.hstack([par[:self.ns], par[-1]])

    def qt(self, par, deriv=False):
        """Qt, or its derivative in the first temporal parameter (log rho, or a)."""
        T = self.grid.T
        par = np.asarray(par, float)
        main = np.empty(T)
        if self.temporal == "rho":
            rho = np.exp(par[self.ns])
            q = 1.0 - rho * rho
            if deriv:  # rho d/drho
                main[:] = 4.0 * rho * rho / (q * q)
                main[[0, -1]] = 2.0 * rho * rho / (q * q)
                off = -rho * (1.0 + rho * rho) / (q * q)
            else:
                main[:] = (1.0 + rho * rho) / q
                main[[0, -1]] = 1.0 / q
                off = -rho / q
        else:
            a, sigma = par[self.ns], np.exp(par[self.ns + 1])
            if deriv:  # d/da
                main[:] = 2.0 * a * sigma
                main[[0, -1]] = 0.0
                off = -sigma
            else:
                main[:] = (1.0 + a * a) * sigma
                main[[0, -1]] = sigma
                off = -a * sigma
        return sparse.diags([np.full(T - 1, off), main, np.full(T - 1, off)], [-1, 0, 1], format="csc")

    def makeQ(self, par):
        Qs = self._wm_Q(self.fam, self._spatial(par))[0]
        return sparse.kron(self.qt(par), Qs, format="csc")

    def dQ_list(self, par):
        g = self.grid
        spar = self._spatial(par)
        Qs, A, _, _ = self._wm_Q(self.fam, spar)
        Qt = self.qt(par)
        out = [sparse.kron(Qt, ((dA.T @ A + A.T @ dA) / g.V).tocsc(), format="csc")
               for _, dA, _ in self._dA_list(spar)]
        out.append(sparse.kron(self.qt(par, deriv=True), Qs, format="csc"))
        if self.temporal == "a-sigma":
            out.append(sparse.kron(Qt, Qs, format="csc"))  # d/dlog sigma: Q is linear in sigma
        return out


class DenseOrSparseFactor:
    """FP64 Cholesky: dense LAPACK for n <= 6000, else SuperLU in symmetric mode
    (stand-in for CHOLMOD, which the reference calls and is not installed)."""

    def __init__(self, Q):
        Q = sparse.csc_matrix(Q)
        self.n = Q.shape[0]
        self.dense = self.n <= 6000
        if self.dense:
            self.L = np.linalg.cholesky(Q.toarray())
        else:
            self.lu = spla.splu(Q, permc_spec="MMD_AT_PLUS_A", diag_pivot_thresh=0.0,
                                options=dict(SymmetricMode=True))

    def logdet(self):
        if self.dense:
            return 2.0 * np.log(np.diag(self.L)).sum()
        return np.log(np.abs(self.lu.U.diagonal())).sum()

    def solve(self, b):
        b = b.toarray() if sparse.issparse(b) else np.asarray(b, float)
        if self.dense:
            return sla.cho_solve((self.L, True), b)
        return self.lu.solve(b)

    def inverse(self):
        return self.solve(np.eye(self.n))
