"""Oracles for the adjoint of the fractional FE operator (test infrastructure).

Test infrastructure only: the GPU gradient is checked against these; nothing
in the product imports them.

The loss is L(kappa, b) = 1/2 ||f(A(kappa)) b - d||^2, where:
- A(kappa) = M^{-1/2} K(kappa) M^{-1/2} on the interior nodes of a P1 mesh;
- K(kappa) = sum_e kappa_e K_e;
- M is the lumped mass (area/3 per vertex).

The reference builds this operator in problem_startup_nonuniform.m and
process_nonuniform.m:90-91. It has no gradient: the adjoint is an extension
of the method.

* ``dense_grad``: exact FP64 gradient from a dense eigendecomposition
  A = Q diag(lam) Q^T. This is the Daleckii-Krein form of the Frechet
  derivative:

      g^T L_f(A, E) b = sum_kl ghat_k F_kl bhat_l (Q^T E Q)_kl,

  where F_kl = f[lam_k, lam_l] (the divided difference, f' on the diagonal).
  So dL/dA_ac = H_ac with H = Q (ghat F bhat^T) Q^T, and
  dL/dkappa_e = sum_ac msi_a K_e[a][c] msi_c H[a][c]. Also, dL/db = f(A) g.
* ``contour_grad``: the same derivative through the quadrature the engine
  uses, with exact sparse solves:

      dL/dkappa_e = Im sum_j w_j s_j^T dA_e r_j,
      r_j = (xi_j - A)^{-1} b,  s_j = (xi_j - A)^{-1} g.

  It separates the quadrature error from the Krylov error.
"""
from __future__ import annotations

import numpy as np
import scipy.linalg as sla
import scipy.sparse as sp
import scipy.sparse.linalg as spla

from gpumatfun_gb300 import problems


def fe_parts(mesh, kappa):
    """A(kappa), interior node index (-1 on the boundary), M^{-1/2} per node,
    and the unit-coefficient element stiffness K_e (nt, 3, 3)."""
    A, ms, inner = problems.fe_operator(mesh, kappa)
    nn = mesh.nodes.shape[0]
    idx = np.full(nn, -1, dtype=np.int64)
    idx[inner] = np.arange(inner.size)
    msi = np.zeros(nn)
    msi[inner] = 1.0 / ms
    area, G = problems.p1_element_grads(mesh.nodes, mesh.tris)
    K1 = np.einsum("tid,tjd->tij", G, G) * area[:, None, None]
    return A, idx, msi, K1


def _grad_from_pairs(mesh, idx, msi, K1, pair):
    """dkappa_e = sum_{a,c interior} msi_a K1_e[a][c] msi_c pair(row_a, row_c)."""
    tri = mesh.tris
    rows = idx[tri]
    dk = np.zeros(tri.shape[0])
    for a in range(3):
        for c in range(3):
            ok = (rows[:, a] >= 0) & (rows[:, c] >= 0)
            coef = msi[tri[:, a]] * K1[:, a, c] * msi[tri[:, c]]
            dk[ok] += coef[ok] * pair(rows[ok, a], rows[ok, c])
    return dk


def divided_differences(lam, f, fprime):
    """F_kl = (f(lam_k) - f(lam_l)) / (lam_k - lam_l), f' where they (nearly) coincide."""
    fl = f(lam)
    dl = lam[:, None] - lam[None, :]
    near = np.abs(dl) <= 1e-10 * np.maximum(np.abs(lam[:, None]), np.abs(lam[None, :]))
    with np.errstate(divide="ignore", invalid="ignore"):
        F = (fl[:, None] - fl[None, :]) / dl
    mid = 0.5 * (lam[:, None] + lam[None, :])
    F[near] = fprime(mid[near])
    return F


def dense_grad(mesh, kappa, b, d, f, fprime):
    """(L, x, dL/dkappa, dL/db) by dense FP64 eigendecomposition."""
    A, idx, msi, K1 = fe_parts(mesh, kappa)
    lam, Q = sla.eigh(A.toarray())
    b = np.asarray(b, dtype=np.float64)
    bh = Q.T @ b
    x = Q @ (f(lam) * bh)
    g = x - d
    gh = Q.T @ g
    F = divided_differences(lam, f, fprime)
    H = Q @ ((gh[:, None] * F * bh[None, :]) @ Q.T)
    dk = _grad_from_pairs(mesh, idx, msi, K1, lambda ra, rc: H[ra, rc])
    db = Q @ (f(lam) * gh)
    return 0.5 * float(g @ g), x, dk, db


def contour_grad(mesh, kappa, b, d, xi, w):
    """(L, x, dL/dkappa) from the quadrature f(A) = Im sum_j w_j (xi_j - A)^{-1}
    with sparse LU solves at every node."""
    A, idx, msi, K1 = fe_parts(mesh, kappa)
    n = A.shape[0]
    b = np.asarray(b, dtype=np.float64)
    I = sp.identity(n, format="csc", dtype=np.complex128)
    Ac = sp.csc_matrix(A, dtype=np.complex128)
    lus = [spla.splu((xj * I - Ac).tocsc()) for xj in xi]
    r = [lu.solve(b.astype(np.complex128)) for lu in lus]
    x = np.imag(sum(wj * rj for wj, rj in zip(w, r)))
    g = x - d
    s = [lu.solve(g.astype(np.complex128)) for lu in lus]

    def pair(ra, rc):
        return np.imag(sum(wj * sj[ra] * rj[rc] for wj, sj, rj in zip(w, s, r)))

    dk = _grad_from_pairs(mesh, idx, msi, K1, pair)
    return 0.5 * float(g @ g), x, dk


def krylov_grad(mesh, kappa, V, Yr, Yi, gs, w):
    """dL/dkappa from a given Krylov state: the GPU gradient restated in FP64.

    The inputs are:
    - V (2, m, n): the Lanczos bases of U = [b, g];
    - Yr, Yi (m, 2C): the shifted solutions, column r*C + j;
    - gs (d+1, C): the shifted-polynomial coefficients;
    - w (C,): the quadrature weights.

    The gradient is Im sum_j S_j^T dA_e R_j, with:
    - R_j = q_j(A) V_b y_b,j / w_j and S_j = q_j(A) V_g y_g,j;
    - q_j(A) = sum_i gs(i, j) A^(d-i), applied by Horner.
    """
    A, idx, msi, K1 = fe_parts(mesh, kappa)
    C = w.size
    yb = (Yr[:, :C] + 1j * Yi[:, :C]) / w[None, :]
    yg = Yr[:, C:2 * C] + 1j * Yi[:, C:2 * C]
    Zb = V[0].T @ yb
    Zg = V[1].T @ yg
    Xb = gs[0][None, :] * Zb
    Xg = gs[0][None, :] * Zg
    for i in range(1, gs.shape[0]):
        Xb = A @ Xb + gs[i][None, :] * Zb
        Xg = A @ Xg + gs[i][None, :] * Zg
    return _grad_from_pairs(mesh, idx, msi, K1, lambda ra, rc: np.imag(np.sum(Xg[ra] * Xb[rc], axis=1)))
