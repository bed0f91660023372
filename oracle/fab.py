"""FP64 numpy restatement of GPUMatfun's f(A)b engine (test infrastructure).

This module is the oracle the engine is checked against: only tests,
``__graft_entry__.smoke()`` and the CPU-baseline leg of ``bench.py`` use it.  Every function follows the
reference statement by statement and cites it.

Notation (the reference's, lanczos.h:24-86): n rows, m = Krylov dimension
(``N``), C = contour nodes (``contour_size``), d = polynomial degree
(``gamma_size`` = d+1), k = deflation vectors (``num_eigs``), R = number of
right-hand sides (the reference fixes R = 2: column 0 is the exp part,
column 1 the phi part).  Matrices are column-major as in MATLAB; numpy arrays
here are (rows, cols) with the same meaning.
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np
import scipy.linalg as sla
import scipy.sparse as sp

__all__ = [
    "deflate", "lanczos", "tridiag_solves", "apply_V_per_node",
    "apply_V_collapsed", "collapse_coeffs", "update_U", "update_U_monodomain",
    "OracleEngine", "nicksmethodcpu", "pack_aabb",
]


def deflate(Q: np.ndarray, U: np.ndarray, flam: np.ndarray):
    """Deflation step of the engine constructor (lanczos_impl.cu:84-89).

    Z = Q^T U; U <- U - Q Z; Z(:, r) *= flam(:, r); update = Q Z.
    ``flam`` is (k, R): the reference passes exp_lambda and phi_lambda as the
    two columns.  Returns (U_deflated, update).
    """
    U = np.array(U, dtype=np.float64, copy=True)
    if Q is None or Q.shape[1] == 0:
        return U, np.zeros_like(U)
    Z = Q.T @ U
    U = U - Q @ Z
    Z = Z * flam
    return U, Q @ Z


def lanczos(A: sp.spmatrix, U: np.ndarray, m: int, gamma: np.ndarray, reorth: int = 0):
    """Polynomial-preconditioned Lanczos, one recurrence per column of U.

    Follows build_subspace.cu:5-89 (and its CPU twin lanczos.m:21-53):
    beta_0 = ||u||; v_0 = u * (1/beta_0); for j = 0..m-1:
    Horner u = p(A) v_j with p(x) = sum_i gamma_i x^(d-i) (:30-47),
    w = A u (:50); w -= beta_j v_{j-1} (j > 0, :53-60); alpha_j = w.v_j (:63-64);
    w -= alpha_j v_j (:67-72); beta_{j+1} = ||w|| (:75-76);
    v_{j+1} = w * (1/beta_{j+1}) (j < m-1, :79-88).  The reference does no
    reorthogonalisation (reorth = 0).  The engine's optional classical
    Gram-Schmidt (reorth = 1, or 2 for CGS2) runs after w -= alpha_j v_j and
    before beta_{j+1} = ||w||: w -= V_{0..j} (V_{0..j}^T w), reorth times;
    alpha and beta keep their three-term values.

    Returns V (R, m, n), alpha (R, m), beta (R, m+1).
    """
    A = sp.csr_matrix(A)
    gamma = np.asarray(gamma, dtype=np.float64)
    n, R = U.shape
    V = np.zeros((R, m, n))
    alpha = np.zeros((R, m))
    beta = np.zeros((R, m + 1))
    for r in range(R):
        beta[r, 0] = np.linalg.norm(U[:, r])
        V[r, 0] = U[:, r] * (1.0 / beta[r, 0])
    for j in range(m):
        vj = V[:, j, :].T  # (n, R)
        u = gamma[0] * vj
        for i in range(1, gamma.size):
            W = A @ u
            u = gamma[i] * vj + W
        W = A @ u
        if j != 0:
            W = W - beta[:, j][None, :] * V[:, j - 1, :].T
        a = np.einsum("nr,nr->r", W, vj)
        alpha[:, j] = a
        W = W - a[None, :] * vj
        for _ in range(reorth):
            for r in range(R):
                Vr = V[r, : j + 1]                 # (j+1, n)
                W[:, r] = W[:, r] - Vr.T @ (Vr @ W[:, r])
        beta[:, j + 1] = np.linalg.norm(W, axis=0)
        if j != m - 1:
            V[:, j + 1, :] = (W * (1.0 / beta[:, j + 1])[None, :]).T
    return V, alpha, beta


def pack_aabb(alpha: np.ndarray, beta: np.ndarray) -> np.ndarray:
    """The engine's ``aabb`` matrix ((m+1) x 2R, lanczos.h:51, build_subspace.cu:63-76).

    Columns 0..R-1 hold alpha (rows 0..m-1), columns R..2R-1 hold beta (rows 0..m).
    """
    R, m = alpha.shape
    out = np.zeros((m + 1, 2 * R))
    out[:m, :R] = alpha.T
    out[:, R:] = beta.T
    return out


def tridiag_solves(alpha, beta, wts, shifts, m=None):
    """Batched shifted tridiagonal solves (lin_sys_solves.cu:5-19,
    lanczos_impl.cu:292-406).

    For RHS r and node j: D = alpha_r - shift (per diagonal entry, from the
    4mC shifts layout), off-diagonals beta_r[1..m-1], x = -beta_r[0] w_{r,j} e1;
    solve (T - sigma) y = x, i.e. y = w beta_0 (sigma I - T)^{-1} e1.
    ``wts`` is a list of R (C, 2) [real, imag] arrays (wts1, wts2, ...);
    ``shifts`` has 2*m*C*R entries.  Returns Yreal, Yimag of shape (m, R*C).
    The reference's CPU twin solves the same systems with sparse backslash
    (nicksmethodcpu.m:18-21); here LAPACK's banded LU with partial pivoting.
    """
    R, mm = alpha.shape
    m = mm if m is None else m
    C = wts[0].shape[0]
    sh = np.asarray(shifts, dtype=np.float64).reshape(R * C, m, 2)
    Yr = np.zeros((m, R * C))
    Yi = np.zeros((m, R * C))
    for r in range(R):
        w = wts[r][:, 0] + 1j * wts[r][:, 1]
        for j in range(C):
            b = r * C + j
            diag = alpha[r, :m] - (sh[b, :, 0] + 1j * sh[b, :, 1])
            off = beta[r, 1:m].astype(np.complex128)
            ab = np.zeros((3, m), dtype=np.complex128)
            ab[0, 1:] = off
            ab[1, :] = diag
            ab[2, :-1] = off
            rhs = np.zeros(m, dtype=np.complex128)
            rhs[0] = -(beta[r, 0] * w[j].real + 1j * beta[r, 0] * w[j].imag)
            y = sla.solve_banded((1, 1), ab, rhs)
            Yr[:, b] = y.real
            Yi[:, b] = y.imag
    return Yr, Yi


def apply_V_per_node(A, V, Yr, Yi, gs_re, gs_im):
    """Per-node lift + shifted polynomial + imaginary-part sum, as written in
    apply_V.cu:8-92 (CPU twin nicksmethodcpu.m:33-43, jacobi_poly_eval.m:12-18).

    For each RHS r and node j: B = V_r (Yr + i Yi)[:, rC+j]; U = gs_0 B;
    for i = 1..d: U = A U + gs_i B; X_r += Im U.  Returns the increment (n, R).
    """
    A = sp.csr_matrix(A)
    R, m, n = V.shape
    C = gs_re.shape[1]
    X = np.zeros((n, R))
    for r in range(R):
        for j in range(C):
            b = r * C + j
            Br = V[r].T @ Yr[:, b]
            Bi = V[r].T @ Yi[:, b]
            ur = gs_re[0, j] * Br - gs_im[0, j] * Bi
            ui = gs_re[0, j] * Bi + gs_im[0, j] * Br
            for i in range(1, gs_re.shape[0]):
                Wr = A @ ur
                Wi = A @ ui
                ur = gs_re[i, j] * Br - gs_im[i, j] * Bi + Wr
                ui = gs_re[i, j] * Bi + gs_im[i, j] * Br + Wi
            X[:, r] += ui
    return X


def collapse_coeffs(Yr, Yi, gs_re, gs_im, R):
    """c[r, i, :] = sum_j Im(gs(i, j) y_{r, j}) -- the m-vectors that collapse
    apply_V's 2C per-node passes into one V.c pass per polynomial term."""
    m = Yr.shape[0]
    C = gs_re.shape[1]
    d1 = gs_re.shape[0]
    c = np.zeros((R, d1, m))
    for r in range(R):
        yr = Yr[:, r * C:(r + 1) * C]
        yi = Yi[:, r * C:(r + 1) * C]
        # Im(gs * y) = gs_re * y_im + gs_im * y_re, summed over nodes j
        c[r] = gs_re @ yi.T + gs_im @ yr.T
    return c


def apply_V_collapsed(A, V, Yr, Yi, gs_re, gs_im):
    """Same sum as ``apply_V_per_node`` reordered: since A is real,
    sum_j Im(q_j(A) V y_j) = sum_i A^(d-i) V c_i with c_i = sum_j Im(gs(i,j) y_j);
    evaluated as X = V c_0; X = A X + V c_i (i = 1..d).  Returns (n, R)."""
    A = sp.csr_matrix(A)
    R, m, n = V.shape
    c = collapse_coeffs(Yr, Yi, gs_re, gs_im, R)
    X = np.zeros((n, R))
    for r in range(R):
        P = V[r].T @ c[r].T  # (n, d+1)
        x = P[:, 0].copy()
        for i in range(1, P.shape[1]):
            x = A @ x + P[:, i]
        X[:, r] = x
    return X


def update_U(X, update, mass, dt):
    """Fisher-KPP exponential-Euler step of update_U.cu:8-16 (before the
    re-deflation): u = X0+X1+update0+update1; u *= (u >= 0);
    g = mass * (u/mass) * (1 - u/mass); U = [u, dt*g]."""
    u = X[:, 0] + X[:, 1] + update[:, 0] + update[:, 1]
    u = u * (u >= 0.0)
    uo = u / mass
    g = mass * uo * (1.0 - uo)
    g = g * dt
    return np.stack([u, g], axis=1)


def update_U_monodomain(X, update, ode, dt, aode, bode, code, vrest, vamp, vpeak, c1ion):
    """FitzHugh-Nagumo step of update_U_monodomain.cu:8-22 (before the
    re-deflation).  Returns (U, ode_new)."""
    u = X[:, 0] + X[:, 1] + update[:, 0] + update[:, 1]
    p1 = u * (dt * aode)
    p2 = ode * (dt * bode)
    ode = ode + (p1 + p2 + code)
    src = (u - vrest) * u * (u - vpeak)
    src = src * (c1ion / vamp / vamp)
    g = (src - ode) * dt
    return np.stack([u, g], axis=1), ode


@dataclass
class OracleEngine:
    """Host mirror of the engine handle (lanczos.h:16-174) in FP64 numpy.

    Holds the same state and offers the same methods as the MEX handle:
    build_subspace, lin_sys_solves, apply_V, update_U, update_U_monodomain,
    get_U, get_xsol.  ``apply_mode`` selects the per-node apply as written
    ("ref") or the algebraically identical collapsed apply ("collapsed").
    """
    A: sp.spmatrix
    U0: np.ndarray
    Q: np.ndarray | None
    m: int
    gamma: np.ndarray
    gs_re: np.ndarray
    gs_im: np.ndarray
    flam: np.ndarray            # (k, R)
    wts: list                   # R arrays (C, 2)
    shifts: np.ndarray          # 2 m C R
    dt: float = 1.0
    col_scale: np.ndarray | None = None
    mass: np.ndarray | None = None
    ode: np.ndarray | None = None
    fhn: tuple = (0.0, 0.0, 0.0, 0.0, 1.0, 0.0, 0.0, 0.0)  # aode,bode,code,vrest,vamp,vth,vpeak,c1ion
    apply_mode: str = "collapsed"
    reorth: int = 0
    V: np.ndarray = field(default=None, init=False)
    alpha: np.ndarray = field(default=None, init=False)
    beta: np.ndarray = field(default=None, init=False)

    def __post_init__(self):
        self.A = sp.csr_matrix(self.A)
        U = np.array(self.U0, dtype=np.float64, copy=True)
        n, R = U.shape
        # lanczos_impl.cu:79 scales the second column by dt (exponential integrator)
        if self.col_scale is None:
            self.col_scale = np.ones(R)
            if R == 2:
                self.col_scale[1] = self.dt
        U = U * self.col_scale[None, :]
        self.Usol = U.copy()                               # :81-82
        self.U, self.update = deflate(self.Q, U, self.flam)  # :84-89
        self.X = np.zeros((n, R))
        if self.mass is None:
            self.mass = np.ones(n)
        if self.ode is None:
            self.ode = np.zeros(n)

    @property
    def R(self):
        return self.U.shape[1]

    def build_subspace(self):
        self.V, self.alpha, self.beta = lanczos(self.A, self.U, self.m, self.gamma, self.reorth)

    def lin_sys_solves(self):
        self.Yr, self.Yi = tridiag_solves(self.alpha, self.beta, self.wts, self.shifts, self.m)

    def apply_V(self):
        fn = apply_V_per_node if self.apply_mode == "ref" else apply_V_collapsed
        self.X = self.X + fn(self.A, self.V, self.Yr, self.Yi, self.gs_re, self.gs_im)

    def _redeflate(self, U):
        self.Usol = U.copy()
        self.U, self.update = deflate(self.Q, U, self.flam)
        self.X = np.zeros_like(self.X)

    def update_U(self):
        """update_U.cu:5-32."""
        self._redeflate(update_U(self.X, self.update, self.mass, self.dt))

    def update_U_monodomain(self):
        """update_U_monodomain.cu:5-43."""
        a, b, c, vrest, vamp, _vth, vpeak, c1 = self.fhn
        U, self.ode = update_U_monodomain(self.X, self.update, self.ode, self.dt,
                                          a, b, c, vrest, vamp, vpeak, c1)
        self._redeflate(U)

    def get_U(self):
        return self.Usol.copy()

    def get_xsol(self):
        return self.X.copy()

    def aabb(self):
        return pack_aabb(self.alpha, self.beta)

    def solve(self):
        """One f(A)b evaluation per column: X + update after build/solve/apply."""
        self.build_subspace()
        self.lin_sys_solves()
        self.apply_V()
        return self.X + self.update


def nicksmethodcpu(wts_list, A, vecs, C, m, gamma, gs_re, gs_im, etaxi, scaling=1.0):
    """The reference's CPU path, nicksmethodcpu.m:7-43, for any number of
    right-hand sides: Lanczos (lanczos.m), C shifted solves per RHS with the
    node weight (and ``scaling``) applied to the solution (:18-21), then per
    node V y followed by the complex Horner of jacobi_poly_eval.m, summing
    imaginary parts (:33-43).  ``vecs`` is (n, R) (already deflated)."""
    V, alpha, beta = lanczos(A, vecs, m, gamma)
    R = vecs.shape[1]
    out = np.zeros_like(vecs)
    for r in range(R):
        H = sp.diags([beta[r, 1:m], alpha[r, :m], beta[r, 1:m]], [-1, 0, 1]).toarray()
        w = wts_list[r][:, 0] + 1j * wts_list[r][:, 1] if np.ndim(wts_list[r]) == 2 else wts_list[r]
        e = np.zeros(m)
        e[0] = beta[r, 0]
        Y = np.zeros((m, C), dtype=np.complex128)
        for j in range(C):
            Y[:, j] = scaling * w[j] * np.linalg.solve(etaxi[j] * np.eye(m) - H, e)
        acc = np.zeros(A.shape[0])
        for j in range(C):
            Br = V[r].T @ Y[:, j].real
            Bi = V[r].T @ Y[:, j].imag
            ur = Br * gs_re[0, j] - Bi * gs_im[0, j]
            ui = Br * gs_im[0, j] + Bi * gs_re[0, j]
            for i in range(1, gs_re.shape[0]):
                Ar = A @ ur
                Ai = A @ ui
                ur, ui = (Ar + Br * gs_re[i, j] - Bi * gs_im[i, j],
                          Ai + Br * gs_im[i, j] + Bi * gs_re[i, j])
            acc += ui
        out[:, r] = acc
    return out
