"""Fixed effects (an intercept and a covariate coefficient) on top of the sparse
GPU factor, by block elimination (reference ``model.py:120-150``, ``useCov``).

The reference augments the latent field x (n lattice nodes) with p <= 2
coefficients b: Q_aug = blockdiag(Q, diag(exp(sigmas))) and S_aug = [S_n, X]
(``Grid.getS`` after ``addCov`` / ``addInt``), and every ``update`` adds
tau S_aug^T S_aug to Q_aug before it solves.  With

    A = Q + tau S_n^T S_n   (sparse; factored on the GPU)
    B = tau S_n^T X         (n x p, dense)
    C = diag(exp(sigmas)) + tau X^T X   (p x p)

a solve with Q_aug = [[A, B], [B^T, C]] goes through the Schur complement
Sc = C - B^T A^-1 B:

    d_b = Sc^-1 (r_b - (A^-1 B)^T r_n),   d_n = A^-1 r_n - (A^-1 B) d_b,

i.e. one solve with A for the p + 1 columns [B, r_n] plus p x p host algebra.
A draw from N(0, Q_aug^-1) is x_b = L_Sc^-T z_b, x_n = P L_A^-T z_n - (A^-1 B) x_b
(L_Sc L_Sc^T = Sc, A = P L_A L_A^T P^T), whose covariance is exactly Q_aug^-1.

The solvers are passed in, so the same code runs against the GPU plan and,
in the tests, against dense CPU algebra.
"""
from __future__ import annotations

import numpy as np
import scipy.linalg as sla


class Border:
    """The border B and corner C of the augmented precision, accumulated over updates."""

    def __init__(self, n, prior_precision):
        self.n = int(n)
        self.prior = np.atleast_1d(np.asarray(prior_precision, dtype=np.float64))
        self.p = self.prior.size
        self.B = np.zeros((self.n, self.p))
        self.C = np.diag(self.prior).astype(np.float64)

    def add(self, nodes, X, tau):
        """Observations at lattice `nodes` with fixed-effect rows X (m x p) and precision tau."""
        X = np.asarray(X, dtype=np.float64).reshape(len(nodes), self.p)
        np.add.at(self.B, np.asarray(nodes, dtype=np.int64), tau * X)
        self.C += tau * X.T @ X

    def solve(self, solve_A, r_n, r_b):
        """(d_n, d_b) with Q_aug [d_n; d_b] = [r_n; r_b]; solve_A(R) returns A^-1 R (n x k)."""
        sol = np.asarray(solve_A(np.column_stack([self.B, r_n]))).reshape(self.n, self.p + 1)
        AiB, Air = sol[:, : self.p], sol[:, self.p]
        Sc = self.C - self.B.T @ AiB
        d_b = np.linalg.solve(Sc, np.asarray(r_b, dtype=np.float64) - AiB.T @ r_n)
        return Air - AiB @ d_b, d_b

    def sample(self, sample_A, solve_A, z_n, z_b):
        """Columns of (x_n, x_b) ~ N(0, Q_aug^-1) from standard normal z_n (n x k), z_b (p x k);
        sample_A(Z) returns P L_A^-T Z."""
        z_n = np.asarray(z_n, dtype=np.float64).reshape(self.n, -1)
        z_b = np.asarray(z_b, dtype=np.float64).reshape(self.p, -1)
        AiB = np.asarray(solve_A(self.B)).reshape(self.n, self.p)
        Sc = self.C - self.B.T @ AiB
        L = np.linalg.cholesky(Sc)
        x_b = sla.solve_triangular(L.T, z_b, lower=False)
        x_n = np.asarray(sample_A(z_n)).reshape(self.n, -1) - AiB @ x_b
        return x_n, x_b


def update_step(border, solve_A, mu, nodes, X, y, tau):
    """One ``Model.update`` with fixed effects (reference model.py:120-127): the
    new rows are added to the border (the caller adds them to A and refactors
    before calling), then mu += Q_aug^-1 tau S_aug^T (y - S_aug mu)."""
    n, p = border.n, border.p
    X = np.asarray(X, dtype=np.float64).reshape(len(nodes), p)
    nodes = np.asarray(nodes, dtype=np.int64)
    border.add(nodes, X, tau)
    resid = np.asarray(y, dtype=np.float64) - (mu[nodes] + X @ mu[n:])
    r_n = np.zeros(n)
    np.add.at(r_n, nodes, tau * resid)
    r_b = tau * X.T @ resid
    d_n, d_b = border.solve(solve_A, r_n, r_b)
    return mu + np.concatenate([d_n, d_b])
