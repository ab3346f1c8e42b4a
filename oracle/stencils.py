"""Oracle (test infrastructure only): numpy restatement of the reference stencils.

Each function returns the raw COO triplets ``(row, col, val)`` exactly as the
reference C++ does, including the ``row == M*N`` sentinel for dropped entries, so
the CUDA stencil kernels can be compared bit for bit.  ``to_csc`` applies the
reference's Python post-processing (drop sentinels, optional NaN -> 0, sum
duplicates into a CSC matrix; e.g. ``spdes/var_advection_var_diffusion2D.py:239-276``).

Entry order inside a cell (offsets in (di, dj)):
0 (0,0)  1 (+1,0)  2 (-1,0)  3 (0,+1)  4 (0,-1)  5 (+1,+1)  6 (-1,-1)  7 (-1,+1)  8 (+1,-1)
for the 9-point diffusion stencil and 0..4 of the same list for the 5-point
advection stencil.  Cells are numbered k = j*M + i (i fastest).

Only this package's tests, ``__graft_entry__.smoke()`` and ``bench.py``'s CPU
baseline import it.
"""
from __future__ import annotations

import numpy as np
from scipy import sparse

DI9 = np.array([0, 1, -1, 0, 0, 1, -1, -1, 1])
DJ9 = np.array([0, 0, 0, 1, -1, 1, -1, 1, -1])


def _ij(M, N):
    j, i = np.divmod(np.arange(M * N), M)
    return i, j


def _cols(M, N, i_n, i_p, j_n, j_p, i, j):
    """Column indices of the nine entries (reference AcH_2D_b1.cpp:122-130)."""
    return np.stack([j * M + i, j * M + i_p, j * M + i_n, j_p * M + i, j_n * M + i,
                     j_p * M + i_p, j_n * M + i_n, j_p * M + i_n, j_n * M + i_p], axis=1)


def _diffusion_vals(hx, hy, W00, E00, N01, S01, N11, S11, E10, W10):
    """The nine 9-point values before boundary folding (AH_2D_b1.cpp:116-124)."""
    return np.stack([
        -hy / hx * (E00 + W00) - hx / hy * (N11 + S11),
        hy / hx * E00 + 0.25 * (N01 - S01),
        hy / hx * W00 - 0.25 * (N01 - S01),
        hx / hy * N11 + 0.25 * (E10 - W10),
        hx / hy * S11 - 0.25 * (E10 - W10),
        0.25 * (N01 + E10),
        0.25 * (S01 + W10),
        -0.25 * (N01 + W10),
        -0.25 * (S01 + E10)], axis=1)


def diffusion_triplets(M, N, H, hx, hy, bc, field):
    """9-point finite-volume operator div(H grad) as COO triplets.

    ``field=False``: constant 2x2 H (reference ``AcH_2D_b{1,3}.cpp``).
    ``field=True``:  per cell and face H of shape (M*N, 4, 2, 2), faces W,E,S,N
    (reference ``AH_2D_b{1,3}.cpp``).  For bc=1 the field version reproduces the
    reference's loop-order quirk (``AH_2D_b1.cpp:34-52``): boundary faces are
    zeroed on the *previous* cell, so only cell 0 sees its own W and S faces
    zeroed; the caller's array is not modified here.
    """
    i, j = _ij(M, N)
    n = M * N
    H = np.asarray(H, dtype=np.float64)
    if field:
        H = H.copy()
        W00, E00 = H[:, 0, 0, 0], H[:, 1, 0, 0]
        N01, S01 = H[:, 3, 0, 1], H[:, 2, 0, 1]
        N11, S11 = H[:, 3, 1, 1], H[:, 2, 1, 1]
        E10, W10 = H[:, 1, 1, 0], H[:, 0, 1, 0]
    else:
        W00 = np.full(n, H[0, 0]); E00 = W00.copy()
        # AcH_2D_b1.cpp:42-49 uses H[1][0] for every cross term; AcH_2D_b3.cpp:41-44
        # reads H[0][1] on the N/S faces and H[1][0] on the E/W faces
        N01 = np.full(n, H[1, 0] if bc == 1 else H[0, 1]); S01 = N01.copy()
        E10 = np.full(n, H[1, 0]); W10 = E10.copy()
        N11 = np.full(n, H[1, 1]); S11 = N11.copy()
    if bc == 1:
        if field:
            # AH_2D_b1.cpp:34-52: the zeroing targets H[k] with k of the previous
            # iteration; only the first iteration (k = 0) hits the current cell.
            if M > 0 and N > 0:
                W00[0] = 0.0; W10[0] = 0.0
                S11[0] = 0.0; S01[0] = 0.0
        else:
            # AcH_2D_b1.cpp:51-68: zero the faces of the current boundary cell.
            left = i == 0
            right = (i == M - 1) & ~left
            bot = j == 0
            top = (j == N - 1) & ~bot
            W00 = np.where(left, 0.0, W00); W10 = np.where(left, 0.0, W10)
            E00 = np.where(right, 0.0, E00); E10 = np.where(right, 0.0, E10)
            S11 = np.where(bot, 0.0, S11); S01 = np.where(bot, 0.0, S01)
            N11 = np.where(top, 0.0, N11); N01 = np.where(top, 0.0, N01)
        i_n = np.where(i == 0, i, i - 1)
        i_p = np.where((i == M - 1) & (i != 0), i, i + 1)
        j_n = np.where(j == 0, j, j - 1)
        j_p = np.where((j == N - 1) & (j != 0), j, j + 1)
        val = _diffusion_vals(hx, hy, W00, E00, N01, S01, N11, S11, E10, W10)
        col = _cols(M, N, i_n, i_p, j_n, j_p, i, j)
        k = j * M + i
        row = np.repeat(k[:, None], 9, axis=1)
        fold = col == k[:, None]
        fold[:, 0] = False
        # AH_2D_b1.cpp:54-101: a folded entry adds its two terms to `rem` (in the
        # C++ association rem = (rem + a) + b) and is dropped
        ha, hb = hy / hx, hx / hy
        terms = [(ha * E00, 0.25 * (N01 - S01)), (ha * W00, -0.25 * (N01 - S01)),
                 (hb * N11, 0.25 * (E10 - W10)), (hb * S11, -0.25 * (E10 - W10)),
                 (0.25 * (N01 + E10), None), (0.25 * (S01 + W10), None),
                 (-0.25 * (N01 + W10), None), (-0.25 * (S01 + E10), None)]
        rem = np.zeros(n)
        for p, (a, b) in enumerate(terms, start=1):
            upd = rem + a if b is None else (rem + a) + b
            rem = np.where(fold[:, p], upd, rem)
        row = np.where(fold, n, row)
        val[:, 0] = val[:, 0] + rem
        return row.astype(np.int32).ravel(), col.astype(np.int32).ravel(), val.ravel()
    if bc == 3:
        val = _diffusion_vals(hx, hy, W00, E00, N01, S01, N11, S11, E10, W10)
        col = _cols(M, N, i - 1, i + 1, j - 1, j + 1, i, j)
        k = j * M + i
        row = np.repeat(k[:, None], 9, axis=1)
        left = i == 0
        right = (i == M - 1) & ~left
        bot = j == 0
        top = (j == N - 1) & ~bot
        for c in (2, 6, 7):
            row[left, c] = n
        for c in (1, 5, 8):
            row[right, c] = n
        for c in (4, 6, 8):
            row[bot, c] = n
        for c in (3, 5, 7):
            row[top, c] = n
        return row.astype(np.int32).ravel(), col.astype(np.int32).ravel(), val.ravel()
    raise ValueError("bc must be 1 (Neumann) or 3 (Dirichlet)")


def advection_const_triplets(M, N, G, hx, hy, bc, diff=3):
    """5-point upwind advection for a constant velocity G = (wx, wy).

    Reference ``Acw_2D_b1.cpp:35-80`` and ``Acw_2D_b3.cpp:39-84``.  ``diff=1,2``
    give the reference's derivative stencils d/dwx, d/dwy; note that for bc=1 the
    boundary correction ``-|G|h/2`` is applied in every mode, as in the reference.
    """
    i, j = _ij(M, N)
    n = M * N
    g0, g1 = float(G[0]), float(G[1])
    with np.errstate(invalid="ignore", divide="ignore"):
        s0 = g0 / abs(g0)
        s1 = g1 / abs(g1)
    if diff == 1:
        v = [s0 * hy, -(s0 - 1.0) * hy / 2, -(s0 + 1.0) * hy / 2, 0.0, 0.0]
    elif diff == 2:
        v = [s1 * hx, 0.0, 0.0, -(s1 - 1.0) * hx / 2, -(s1 + 1.0) * hx / 2]
    else:
        v = [abs(g0) * hy + abs(g1) * hx, -(abs(g0) - g0) * hy / 2, -(abs(g0) + g0) * hy / 2,
             -(abs(g1) - g1) * hx / 2, -(abs(g1) + g1) * hx / 2]
    val = np.tile(np.array(v, dtype=np.float64), (n, 1))
    k = j * M + i
    row = np.repeat(k[:, None], 5, axis=1)
    left = i == 0
    right = (i == M - 1) & ~left
    bot = j == 0
    top = (j == N - 1) & ~bot
    if bc == 1:
        i_n = np.where(left, i, i - 1)
        i_p = np.where(right, i, i + 1)
        j_n = np.where(bot, j, j - 1)
        j_p = np.where(top, j, j + 1)
        val[left, 0] -= abs(g0) * hy / 2
        row[left, 2] = n
        val[right, 0] -= abs(g0) * hy / 2
        row[right, 1] = n
        val[bot, 0] -= abs(g1) * hx / 2
        row[bot, 4] = n
        val[top, 0] -= abs(g1) * hx / 2
        row[top, 3] = n
    elif bc == 3:
        i_n, i_p, j_n, j_p = i - 1, i + 1, j - 1, j + 1
        row[i == M - 1, 1] = n
        row[i == 0, 2] = n
        row[j == N - 1, 3] = n
        row[j == 0, 4] = n
    else:
        raise ValueError("bc must be 1 or 3")
    col = np.stack([k, j * M + i_p, j * M + i_n, j_p * M + i, j_n * M + i], axis=1)
    return row.astype(np.int32).ravel(), col.astype(np.int32).ravel(), val.ravel()


def advection_field_triplets(M, N, G, hx, hy, bc, diff=3, dG=None, safe_sign=False):
    """5-point upwind advection for per-cell face velocities G (M*N, 4).

    Faces are ordered (E, N, W, S) = (0, 1, 2, 3) as in reference
    ``Aw_2D_b1.cpp:47-98``; bc=1 zeroes the boundary faces of the current cell in
    G and dG (on a copy here) before evaluating, bc=3 drops out-of-grid entries
    (``Aw_2D_b3.cpp:37-81``).  ``safe_sign=True`` uses sign(G) (0 at G = 0) in
    the derivative modes instead of the reference's G/|G| (NaN at 0).
    """
    i, j = _ij(M, N)
    n = M * N
    G = np.array(G, dtype=np.float64, copy=True)
    dG = np.zeros((n, 4)) if dG is None else np.array(dG, dtype=np.float64, copy=True)
    k = j * M + i
    row = np.repeat(k[:, None], 5, axis=1)
    left = i == 0
    right = (i == M - 1) & ~left
    bot = j == 0
    top = (j == N - 1) & ~bot
    if bc == 1:
        i_n = np.where(left, i, i - 1)
        i_p = np.where(right, i, i + 1)
        j_n = np.where(bot, j, j - 1)
        j_p = np.where(top, j, j + 1)
        # folding happens when the clamped neighbour equals the cell itself
        fe = (j * M + i_p) == k
        fw = (j * M + i_n) == k
        fn = (j_p * M + i) == k
        fs = (j_n * M + i) == k
        G[fe, 0] = 0.0; dG[fe, 0] = 0.0; row[fe, 1] = n
        G[fw, 2] = 0.0; dG[fw, 2] = 0.0; row[fw, 2] = n
        G[fn, 1] = 0.0; dG[fn, 1] = 0.0; row[fn, 3] = n
        G[fs, 3] = 0.0; dG[fs, 3] = 0.0; row[fs, 4] = n
    elif bc == 3:
        i_n, i_p, j_n, j_p = i - 1, i + 1, j - 1, j + 1
        row[i == M - 1, 1] = n
        row[i == 0, 2] = n
        row[j == N - 1, 3] = n
        row[j == 0, 4] = n
    else:
        raise ValueError("bc must be 1 or 3")
    aG = np.abs(G)
    with np.errstate(invalid="ignore", divide="ignore"):
        sG = np.sign(G) if safe_sign else G / aG
    if diff == 1:
        val = np.stack([(sG[:, 0] * dG[:, 0] + dG[:, 0] + sG[:, 2] * dG[:, 2] - dG[:, 2]) * hy / 2,
                        -(sG[:, 0] * dG[:, 0] - dG[:, 0]) * hy / 2,
                        -(sG[:, 2] * dG[:, 2] + dG[:, 2]) * hy / 2,
                        np.zeros(n), np.zeros(n)], axis=1)
    elif diff == 2:
        val = np.stack([(sG[:, 1] * dG[:, 1] + dG[:, 1] + sG[:, 3] * dG[:, 3] - dG[:, 3]) * hx / 2,
                        np.zeros(n), np.zeros(n),
                        -(sG[:, 1] * dG[:, 1] - dG[:, 1]) * hx / 2,
                        -(sG[:, 3] * dG[:, 3] + dG[:, 3]) * hx / 2], axis=1)
    else:
        val = np.stack([(aG[:, 0] + G[:, 0] + aG[:, 2] - G[:, 2]) * hy / 2
                        + (aG[:, 1] + G[:, 1] + aG[:, 3] - G[:, 3]) * hx / 2,
                        -(aG[:, 0] - G[:, 0]) * hy / 2,
                        -(aG[:, 2] + G[:, 2]) * hy / 2,
                        -(aG[:, 1] - G[:, 1]) * hx / 2,
                        -(aG[:, 3] + G[:, 3]) * hx / 2], axis=1)
    col = np.stack([k, j * M + i_p, j * M + i_n, j_p * M + i, j_n * M + i], axis=1)
    return row.astype(np.int32).ravel(), col.astype(np.int32).ravel(), val.ravel()


def to_csc(M, N, row, col, val, nan_to_zero=False):
    """Reference post-processing: drop sentinel rows, sum duplicates (e.g.
    ``spdes/advection_diffusion2D.py:226-260``)."""
    n = M * N
    keep = row != n
    r, c, v = row[keep], col[keep], val[keep].copy()
    if nan_to_zero:
        v[np.isnan(v)] = 0.0
    return sparse.csc_matrix((v, (r, c)), shape=(n, n))
