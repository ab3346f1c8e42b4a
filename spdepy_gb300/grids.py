"""Regular 2-D / 2-D x time grids with the B-spline bases of the reference.

Mirrors ``spdepy.grids.grid`` (reference ``grids/__init__.py:3-49``) and the grid
classes ``grids/spatial2D_regular_mesh.py`` / ``grids/spat2Dtemp_regular_mesh.py``:
cell spacing ``hx = (max x - min x)/(M - 1)`` (``:129-132``), degree-2 B-splines
with ``Nbs`` functions per axis whose two end functions are merged (``:157-187``),
evaluated at cell centres (``bs``), at the four faces W,E,S,N (``bsH``) and at the
advection faces E,N,W,S (``bsA``, extended to padding cells as ``advBound`` does,
``:347-391``).  Everything here is one-time set-up on the host; the per-theta
work happens on the GPU.
"""
from __future__ import annotations

import numpy as np
from scipy import sparse


def _bspline2(t, knots):
    """Degree-2 B-splines on `knots` at points t (Cox-de Boor), last interval closed."""
    nk = knots.size
    B = np.zeros((t.size, nk - 1))
    for i in range(nk - 1):
        inside = (t >= knots[i]) & (t < knots[i + 1])
        if i == nk - 2:
            inside |= (t >= knots[i]) & (t <= knots[i + 1])
        B[:, i] = inside
    for r in (1, 2):
        Bn = np.zeros((t.size, nk - r - 1))
        for i in range(nk - r - 1):
            left = (t - knots[i]) / (knots[i + r] - knots[i]) * B[:, i]
            right = (knots[i + r + 1] - t) / (knots[i + r + 1] - knots[i + 1]) * B[:, i + 1]
            Bn[:, i] = left + right
        B = Bn
    return np.hstack([(B[:, 0] + B[:, 1])[:, None], B[:, 2:-2], (B[:, -2] + B[:, -1])[:, None]])


class Grid:
    """Spatial (T == 1) or spatio-temporal grid; cells k = j*M + i, nodes t*Ns + k."""

    def __init__(self, x, y, t=None, extend=None, Nbs=3):
        self.x = np.asarray(x, dtype=np.float64)
        self.y = np.asarray(y, dtype=np.float64)
        self.sdim = 2
        self.type = "gridS" if t is None else "gridST"
        self.t = None if t is None else np.asarray(t, dtype=np.float64)
        self.M, self.N = self.x.size, self.y.size
        self.T = 1 if t is None else self.t.size
        self.hx = (self.x.max() - self.x.min()) / (self.M - 1)
        self.hy = (self.y.max() - self.y.min()) / (self.N - 1)
        self.dt = (self.t.max() - self.t.min()) / (self.T - 1) if self.T > 1 else 1.0
        self.V = self.hx * self.hy
        self.Nbs = int(Nbs)
        self.Nbs2 = self.Nbs ** 2
        self.Ne = int(extend) if extend else 0
        self.Mx, self.Ny = self.M + 2 * self.Ne, self.N + 2 * self.Ne
        self.Ns = self.Mx * self.Ny
        self.n = self.Ns * self.T
        sx, sy = np.meshgrid(self.x, self.y)
        self.sx, self.sy = sx.ravel(), sy.ravel()
        if self.Ne:
            e = self.Ne
            xe = np.hstack([self.x[0] - self.hx * np.arange(e, 0, -1), self.x, self.x[-1] + self.hx * np.arange(1, e + 1)])
            ye = np.hstack([self.y[0] - self.hy * np.arange(e, 0, -1), self.y, self.y[-1] + self.hy * np.arange(1, e + 1)])
            sxe, sye = np.meshgrid(xe, ye)
            self.px, self.py = sxe.ravel(), sye.ravel()
        else:
            self.px, self.py = self.sx, self.sy
        # covariate / intercept columns of S (reference addCov / addInt)
        self.cov = None
        self.inter = False
        self.scale = False
        self.bs = self._basis(self.px, self.py, (0.0, 0.0))
        shifts = {0: (-self.hx / 2, 0.0), 1: (self.hx / 2, 0.0), 2: (0.0, -self.hy / 2), 3: (0.0, self.hy / 2)}
        self.bsH = np.stack([self._basis(self.px, self.py, shifts[f]) for f in range(4)], axis=1)
        if self.T > 1:
            # advection faces E, N, W, S on the unextended cells, then extended
            raw = np.stack([self._basis(self.sx, self.sy, shifts[s]) for s in (1, 3, 0, 2)], axis=1)
            self.bsA = np.einsum("km,mfi->kfi", self._extension(), raw) if self.Ne else raw
        else:
            self.bsA = None
        self._S = None

    @property
    def shape(self):
        return [self.Mx, self.Ny] if self.T == 1 else [self.Mx, self.Ny, self.T]

    def _basis(self, px, py, shift):
        dx, dy = shift
        if dx != 0 or dy != 0:
            xmin, xmax = self.sx.min() - self.hx / 2, self.sx.max() + self.hx / 2
            ymin, ymax = self.sy.min() - self.hy / 2, self.sy.max() + self.hy / 2
        else:
            xmin, xmax, ymin, ymax = self.sx.min(), self.sx.max(), self.sy.min(), self.sy.max()
        nb = self.Nbs
        kx = np.linspace(xmin - 2 * (xmax - xmin) / nb, xmax + 2 * (xmax - xmin) / nb, nb + 5)
        ky = np.linspace(ymin - 2 * (ymax - ymin) / nb, ymax + 2 * (ymax - ymin) / nb, nb + 5)
        bx = _bspline2(px + dx, kx)
        by = _bspline2(py + dy, ky)
        # column i*Nbs + j = bx_j * by_i
        return (by[:, :, None] * bx[:, None, :]).reshape(px.size, nb * nb)

    def _extension(self):
        """Linear ramp of the boundary velocities into the padding cells (advBound)."""
        M, N, Ne = self.M, self.N, self.Ne
        rows, cols, vals = [], [], []

        def put(k, c, v):
            rows.append(k); cols.append(c); vals.append(v)

        for i in range(M + 2 * Ne):
            for j in range(N + 2 * Ne):
                k = i + j * (M + 2 * Ne)
                if i < Ne and j < Ne:
                    put(k, 0, j / Ne if i >= j else i / Ne)
                    continue
                if i >= M + Ne and j >= N + Ne:
                    put(k, M * N - 1, (N + 2 * Ne - 1 - j) / Ne if N - j <= M - i else (M + 2 * Ne - 1 - i) / Ne)
                    continue
                if i >= M + Ne and j < Ne:
                    put(k, M - 1, (M + 2 * Ne - 1 - i) / Ne if M + 2 * Ne - 1 - i <= j else j / Ne)
                    continue
                if i < Ne and j >= N + Ne:
                    put(k, M * (N - 1), i / Ne if i <= N + 2 * Ne - 1 - j else (N + 2 * Ne - 1 - j) / Ne)
                    continue
                if i < Ne:
                    put(k, (j - Ne) * M, i / Ne)
                elif i >= M + Ne:
                    put(k, M - 1 + (j - Ne) * M, (M + 2 * Ne - 1 - i) / Ne)
                if j < Ne:
                    put(k, i - Ne, j / Ne)
                elif j >= N + Ne:
                    put(k, i - Ne + (N - 1) * M, (N + 2 * Ne - 1 - j) / Ne)
                if Ne <= i < M + Ne and Ne <= j < N + Ne:
                    put(k, (i - Ne) + (j - Ne) * M, 1.0)
        Ae = np.zeros((self.Ns, M * N))
        # later writes win, as with the reference's dense assignments
        for k, c, v in zip(rows, cols, vals):
            Ae[k, c] = v
        return Ae

    def assimilate_adv(self, we, wn):
        """Face velocities (E, N, W, S) from cell-centred components
        (reference ``spat2Dtemp_regular_mesh.py:277-344``)."""
        M, N = self.M, self.N
        k = np.arange(M * N)
        j, i = np.divmod(k, M)
        we = np.asarray(we, float)
        wn = np.asarray(wn, float)
        ww = np.stack([(we + we[np.where(i + 1 == M, k, k + 1)]) / 2, (wn + wn[np.where(j + 1 == N, k, k + M)]) / 2,
                       (we + we[np.where(i == 0, k, k - 1)]) / 2, (wn + wn[np.where(j == 0, k, k - M)]) / 2], axis=1)
        return self._extension() @ ww if self.Ne else ww

    def n2e(self, idx):
        """Observation index on the unextended grid -> node on the extended grid (:86-95)."""
        idx = np.asarray(idx, dtype=np.int64)
        t, r = np.divmod(idx, self.M * self.N)
        j, i = np.divmod(r, self.M)
        return (i + self.Ne) + (j + self.Ne) * self.Mx + t * self.Ns

    def obs_nodes(self, idx=None):
        if idx is None:
            idx = np.arange(self.M * self.N * self.T)
        return self.n2e(idx)

    def getS(self, idxs=None):
        """Observation matrix S (reference :35-58): selected identity rows over the
        lattice nodes, followed by the fixed-effect columns when set, in the
        reference's order: [1, cov] (cov / max(cov) with scale) after addCov with
        an intercept, [cov] without one, [1] after addInt alone."""
        cols = self.obs_nodes(idxs)
        m = cols.size
        S = sparse.csc_matrix((np.ones(m), (np.arange(m), cols)), shape=(m, self.n))
        extra = self._fixed_effects()
        if extra is None:
            return S
        rows = np.arange(self.M * self.N * self.T) if idxs is None else np.asarray(idxs, dtype=np.int64)
        return sparse.hstack([S, sparse.csc_matrix(extra[rows])], format="csc")

    def _fixed_effects(self):
        """Dense fixed-effect columns over all M N T observation positions, or None."""
        npos = self.M * self.N * self.T
        if self.cov is not None:
            cov = np.asarray(self.cov, dtype=np.float64).reshape(-1)
            if cov.size != npos:
                raise ValueError(f"covariate has {cov.size} values, the grid {npos} observation positions")
            if self.inter:
                return np.stack([np.ones(npos), cov / cov.max() if self.scale else cov], axis=1)
            return cov.reshape(-1, 1)
        if self.inter:
            return np.ones((npos, 1))
        return None

    def addCov(self, cov, inter=True, scale=False):
        """Covariate (and intercept) columns of S (reference :60-64).  The
        reference's spatial grid ignores `scale` (grids/spatial2D_regular_mesh.py:
        55-58 never stores it), so a spatial grid keeps the unscaled covariate."""
        self.inter = inter
        if self.T > 1:
            self.scale = scale
        self.cov = np.asarray(cov, dtype=np.float64)

    def addInt(self):
        """Intercept column of S (reference :66-68)."""
        self.inter = True

    def spatial(self):
        """The spatial grid of the initial-field model."""
        return Grid(self.x, self.y, None, self.Ne or None, self.Nbs)


def grid(x, y, z=None, t=None, extend=None, Nbs=3):
    """Grid factory with the reference's signature (``grids/__init__.py:3``)."""
    if z is not None:
        raise NotImplementedError("3-D grids have no model in the reference (spdes/__init__.py:104-105)")
    return Grid(x, y, t, extend, Nbs)
