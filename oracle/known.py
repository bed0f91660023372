"""Known answers for f(A)b (test infrastructure).

* ``dst_fab_2d`` -- exact f(A)b for the 2D Dirichlet 5-point Laplacian by
  DST-I diagonalisation, the reference's own validation mechanism
  (startup_nicksmethod_GPU.m:91-109: dst, scale by f(lambda_i + lambda_j), idst).
* ``dense_fab`` -- f(A)b = Q f(Lambda) Q^T b from a dense symmetric
  eigendecomposition (n up to a few thousand).
"""
from __future__ import annotations

import numpy as np
import scipy.fft as sfft
import scipy.linalg as sla


def dst_fab_2d(b: np.ndarray, N: int, f, scale: float = 1.0) -> np.ndarray:
    """Exact f(A) b for A = scale * (I kron T + T kron I) on an N x N Dirichlet grid.

    b is indexed i + N j (x fastest).  The orthonormal DST-I is its own inverse.
    """
    lam = 4 * np.sin(np.arange(1, N + 1) * np.pi / (2 * (N + 1))) ** 2
    mu = f((lam[:, None] + lam[None, :]) * scale)  # [j (y), i (x)] symmetric form
    B = np.asarray(b, dtype=np.float64).reshape(N, N)  # rows = y index j, cols = x index i
    Bh = sfft.dstn(B, type=1, norm="ortho")
    return sfft.idstn(Bh * mu, type=1, norm="ortho").reshape(-1)


def dense_fab(A, b: np.ndarray, f) -> np.ndarray:
    """f(A) b via dense eigh (A symmetric)."""
    Ad = A.toarray() if hasattr(A, "toarray") else np.asarray(A)
    lam, Q = sla.eigh(Ad)
    return Q @ (f(lam)[:, None] * (Q.T @ np.asarray(b, dtype=np.float64).reshape(Ad.shape[0], -1))).squeeze()
