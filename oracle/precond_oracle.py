"""Oracle (test infrastructure only): FP64 numpy restatement of the learned
space-time preconditioner M^-1 = G^T G and of its training loss and gradient.

The reference has no counterpart (it factors every system with CHOLMOD), so
this restatement is pinned by central finite differences of its own loss
(``tests/test_precond_oracle.py``).  The GPU kernels (``csrc/pcg.cu``) are
checked against it.

Conventions (shared with the kernels):
  * A (= Q or Q + tau S^T S) in the 43-slot stencil layout: dt = -1: 3 x 3,
    dt = 0: 5 x 5, dt = +1: 3 x 3, slot 21 the centre (spatial grids use the
    dt = 0 slots only);
  * features f_p = A_p,. / A_pp without the centre (42 values), s_p = A_pp^-1/2;
  * network 42-32-32-27, tanh, parameters W1[32][42], b1, W2[32][32], b2,
    W3[27][32], b3 flattened in that order;
  * G offsets o = (dt + 1) 9 + (dy + 1) 3 + (dx + 1), weights
    w_o(p) = (delta_o,13 + out_o(p)) s_p, zero where p + o leaves the grid;
  * loss ||z - G A G^T z||^2 / (n k).
"""
from __future__ import annotations

import numpy as np

FEAT, HID, OFF = 42, 32, 27
SIZES = [("W1", (HID, FEAT)), ("b1", (HID,)), ("W2", (HID, HID)), ("b2", (HID,)), ("W3", (OFF, HID)), ("b3", (OFF,))]
NPARAMS = sum(int(np.prod(s)) for _, s in SIZES)


def unpack(prm):
    out, o = {}, 0
    for name, shape in SIZES:
        k = int(np.prod(shape))
        out[name] = np.asarray(prm[o:o + k], dtype=np.float64).reshape(shape)
        o += k
    return out


def pack(d):
    return np.concatenate([d[name].ravel() for name, _ in SIZES])


def _slot43():
    tab = {}
    for s in range(43):
        if s < 9:
            dt, dy, dx = -1, s // 3 - 1, s % 3 - 1
        elif s < 34:
            dt, dy, dx = 0, (s - 9) // 5 - 2, (s - 9) % 5 - 2
        else:
            dt, dy, dx = 1, (s - 34) // 3 - 1, (s - 34) % 3 - 1
        tab[(dx, dy, dt)] = s
    return tab


SLOT43 = _slot43()


def stencil43(A, Mx, Ny, T):
    """Rows of the sparse matrix A (natural node order) in the 43-slot layout."""
    A = A.tocoo()
    n = Mx * Ny * T
    out = np.zeros((n, 43))
    rt, rr = np.divmod(A.row, Mx * Ny)
    ry, rx = np.divmod(rr, Mx)
    ct, cr = np.divmod(A.col, Mx * Ny)
    cy, cx = np.divmod(cr, Mx)
    for r, dx, dy, dt, v in zip(A.row, cx - rx, cy - ry, ct - rt, A.data):
        s = SLOT43.get((int(dx), int(dy), int(dt)))
        if s is None:
            raise ValueError("entry outside the 43-point stencil")
        out[r, s] += v
    return out


def features(S43):
    diag = S43[:, 21].copy()
    f = np.delete(S43, 21, axis=1) / diag[:, None]
    return f, 1.0 / np.sqrt(diag)


def forward(prm, f):
    P = unpack(prm)
    h1 = np.tanh(f @ P["W1"].T + P["b1"])
    h2 = np.tanh(h1 @ P["W2"].T + P["b2"])
    return h1, h2, h2 @ P["W3"].T + P["b3"]


def offsets27():
    return [(o % 3 - 1, (o // 3) % 3 - 1, o // 9 - 1) for o in range(OFF)]


def _coords(Mx, Ny, T):
    k = np.arange(Mx * Ny * T)
    t, r = np.divmod(k, Mx * Ny)
    y, x = np.divmod(r, Mx)
    return x, y, t


def weights(out, s, Mx, Ny, T):
    x, y, t = _coords(Mx, Ny, T)
    w = out.copy()
    w[:, 13] += 1.0
    w *= s[:, None]
    for o, (dx, dy, dt) in enumerate(offsets27()):
        ok = (x + dx >= 0) & (x + dx < Mx) & (y + dy >= 0) & (y + dy < Ny) & (t + dt >= 0) & (t + dt < T)
        w[~ok, o] = 0.0
    return w


def apply_G(w, v, Mx, Ny, T, transpose=False):
    """G v (or G^T v) for v of shape (n,) or (n, k)."""
    v2 = v.reshape(v.shape[0], -1)
    out = np.zeros_like(v2)
    x, y, t = _coords(Mx, Ny, T)
    for o, (dx, dy, dt) in enumerate(offsets27()):
        ok = (x + dx >= 0) & (x + dx < Mx) & (y + dy >= 0) & (y + dy < Ny) & (t + dt >= 0) & (t + dt < T)
        p = np.nonzero(ok)[0]
        nb = p + (dt * Ny + dy) * Mx + dx
        if not transpose:
            out[p] += w[p, o][:, None] * v2[nb]
        else:
            np.add.at(out, nb, w[p, o][:, None] * v2[p])
    return out.reshape(v.shape)


def loss_grad(prm, A, Mx, Ny, T, z):
    """Loss ||z - G A G^T z||^2 / (n k) and its gradient in the parameters."""
    n = Mx * Ny * T
    z = z.reshape(n, -1)
    k = z.shape[1]
    S43 = stencil43(A, Mx, Ny, T)
    f, s = features(S43)
    h1, h2, out = forward(prm, f)
    w = weights(out, s, Mx, Ny, T)
    y = apply_G(w, z, Mx, Ny, T, transpose=True)
    u = A @ y
    e = z - apply_G(w, u, Mx, Ny, T)
    g2 = A @ apply_G(w, e, Mx, Ny, T, transpose=True)
    loss = float((e * e).sum() / (n * k))
    # dL/dw_o(p) = -2/(n k) sum_r (e_pr u_(p+o)r + z_pr g2_(p+o)r)
    x, yy, t = _coords(Mx, Ny, T)
    dw = np.zeros((n, OFF))
    for o, (dx, dy, dt) in enumerate(offsets27()):
        ok = (x + dx >= 0) & (x + dx < Mx) & (yy + dy >= 0) & (yy + dy < Ny) & (t + dt >= 0) & (t + dt < T)
        p = np.nonzero(ok)[0]
        nb = p + (dt * Ny + dy) * Mx + dx
        dw[p, o] = (e[p] * u[nb]).sum(1) + (z[p] * g2[nb]).sum(1)
    dw *= -2.0 / (n * k)
    dout = dw * s[:, None]
    P = unpack(prm)
    d2 = (dout @ P["W3"]) * (1 - h2 ** 2)
    d1 = (d2 @ P["W2"]) * (1 - h1 ** 2)
    grad = {"W3": dout.T @ h2, "b3": dout.sum(0), "W2": d2.T @ h1, "b2": d2.sum(0), "W1": d1.T @ f,
            "b1": d1.sum(0)}
    return loss, pack(grad), w


def pcg(A, b, apply_minv, tol=1e-8, maxit=10000):
    """Textbook preconditioned CG; returns (x, iterations, relative residual)."""
    x = np.zeros_like(b)
    r = b.copy()
    z = apply_minv(r)
    p = z.copy()
    rz = r @ z
    nb = np.linalg.norm(b)
    it = 0
    while it < maxit and np.linalg.norm(r) > tol * nb:
        ap = A @ p
        alpha = rz / (p @ ap)
        x += alpha * p
        r -= alpha * ap
        z = apply_minv(r)
        rzn = r @ z
        p = z + (rzn / rz) * p
        rz = rzn
        it += 1
    return x, it, np.linalg.norm(b - A @ x) / nb
