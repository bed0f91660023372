"""Workload builders: everything ``lanczos_create`` needs for one problem.

A ``FabProblem`` bundles the operator and the method parameters that the
reference computes in its MATLAB start-up scripts (startup_nicksmethod_GPU.m:
27-218, problem_startup_nonuniform.m:25-119): the deflation pairs (Q, lambda)
and f(lambda) per right-hand side, the HHT nodes/weights, the polynomial
preconditioner gamma and its shifted coefficients, and the per-diagonal
shift array.  Right-hand sides are generalised from the reference's fixed
pair (exp part, phi part) to R columns, each with its own function.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field
from typing import Callable, Sequence

import numpy as np
import scipy.sparse as sp

from . import params, problems

__all__ = ["FabProblem", "make_problem", "fd2d_problem", "config1", "config1_small",
           "fe_disk_problem", "config2", "fd3d_problem", "config3"]


@dataclass
class FabProblem:
    name: str
    A: sp.csr_matrix
    U: np.ndarray                 # (n, R) right-hand sides (before deflation)
    Q: np.ndarray                 # (n, k)
    lam: np.ndarray               # (k,)
    flam: np.ndarray              # (k, R)  f_r(lambda)
    m: int
    gamma: np.ndarray             # (d+1,)
    gs_re: np.ndarray             # (d+1, C)
    gs_im: np.ndarray
    wts: list                     # R arrays (C, 2)
    shifts: np.ndarray            # 2 m C R
    sigma: np.ndarray             # (C,) complex
    contour: params.Contour
    funcs: list                   # R callables
    l1: float
    lN: float
    col_scale: np.ndarray | None = None
    meta: dict = field(default_factory=dict)
    row_weight: np.ndarray | None = None   # near-null vector of A (mixed engine's diagonal compensation)

    @property
    def n(self):
        return self.A.shape[0]

    @property
    def R(self):
        return self.U.shape[1]

    @property
    def C(self):
        return self.sigma.size

    @property
    def d(self):
        return self.gamma.size - 1

    @property
    def k(self):
        return self.Q.shape[1]


def make_problem(name, A, U, Q, lam, funcs: Sequence[Callable], m, C, l1, lN,
                 degree=0, prob_dim=2.0, col_scale=None, meta=None, row_weight=None) -> FabProblem:
    """Assemble the method parameters for operator A (startup_nicksmethod_GPU.m:159-218)."""
    A = sp.csr_matrix(A)
    A.sort_indices()
    U = np.ascontiguousarray(np.asarray(U, dtype=np.float64).reshape(A.shape[0], -1))
    R = U.shape[1]
    if len(funcs) != R:
        raise ValueError("one function per right-hand side")
    con = params.hht_contour(l1, lN, C)
    gamma = params.polynomial_coeffs(degree, prob_dim)
    gs, sigma = params.shifted_poly_coeffs(gamma, con.xi)
    wts = [con.weights_mat(f) for f in funcs]
    flam = np.stack([np.real(f(lam.astype(np.float64))) for f in funcs], axis=1) if Q.shape[1] else np.zeros((0, R))
    shifts = params.shifts_vector(sigma, m, R)
    return FabProblem(name=name, A=A, U=U, Q=np.ascontiguousarray(Q), lam=np.asarray(lam, dtype=np.float64),
                      flam=flam, m=int(m), gamma=gamma, gs_re=np.ascontiguousarray(gs.real),
                      gs_im=np.ascontiguousarray(gs.imag), wts=wts, shifts=shifts, sigma=sigma,
                      contour=con, funcs=list(funcs), l1=float(l1), lN=float(lN),
                      col_scale=col_scale, meta=dict(meta or {}), row_weight=row_weight)


def fd2d_problem(N: int, k: int, m: int, C: int, funcs, R: int = 1, scale: float = 1.0,
                 seed: int = 0, degree: int = 0, normalise: bool = True, name: str = "fd2d"):
    """2D Dirichlet 5-point Laplacian (N x N interior, times ``scale``) with the k
    smallest analytic sine modes deflated; l1 = k-th eigenvalue, lN = lambda_max
    (startup_nicksmethod_GPU.m:33-37).  b ~ U[0,1) from ``seed``."""
    A = problems.laplacian_2d(N, "D", scale)
    if k > 0:
        lam, Q = problems.laplacian_2d_eigpairs(N, k, "D", scale)
        l1 = float(lam.max())
    else:
        lam, Q = np.zeros(0), np.zeros((N * N, 0))
        l1 = float(2 * 4 * math.sin(math.pi / (2 * (N + 1))) ** 2 * scale)
    lN = float(8 * math.sin(N * math.pi / (2 * (N + 1))) ** 2 * scale)
    rng = np.random.default_rng(seed)
    U = rng.random((N * N, R))
    if normalise:
        U /= np.linalg.norm(U, axis=0, keepdims=True)
    return make_problem(name, A, U, Q, lam, funcs, m, C, l1, lN, degree=degree,
                        prob_dim=2.0 * scale, meta=dict(N=N, scale=scale, seed=seed, bc="D"))


def config1(R: int = 1, seed: int = 0) -> FabProblem:
    """Plain FP64 workload: 2D 5-point Dirichlet Laplacian on a 256 x 256 interior
    grid scaled by 1/h^2 (h = 1/257), f = exp(-1e-3 lambda^0.75), m = 60,
    32 contour nodes, 10 deflated sine modes, no polynomial preconditioning."""
    N = 256
    f = params.frac_exp(1e-3, 1.5)
    return fd2d_problem(N, 10, 60, 32, [f] * R, R=R, scale=257.0 ** 2, seed=seed, name="fd2d-256-fp64")


def config1_small(N=24, k=4, m=40, C=24, R=2, seed=1, degree=0) -> FabProblem:
    """Small version of the plain workload used by parity tests."""
    f1 = params.frac_exp(1e-3, 1.5)
    f2 = params.frac_phi(1e-3, 1.5)
    funcs = [f1, f2] if R == 2 else [f1] * R
    return fd2d_problem(N, k, m, C, funcs, R=R, scale=float((N + 1) ** 2), seed=seed, degree=degree,
                        name=f"fd2d-{N}")


def fd3d_problem(N: int, m: int, C: int, funcs, R: int = 1, seed: int = 0, degree: int = 0,
                 name: str = "fd3d", lam_bounds=None):
    """3D 7-point variable-coefficient Laplacian (no deflation).  Spectrum bounds:
    l1 from the constant-coefficient Dirichlet minimum times min kappa (0.5),
    lN from Gershgorin."""
    A = problems.laplacian_3d_var(N)
    h = 1.0 / (N + 1)
    if lam_bounds is None:
        l1 = 0.5 * 3 * 4 * math.sin(math.pi * h / 2) ** 2 / (h * h)
        lN = float(2 * np.abs(A.diagonal()).max())
    else:
        l1, lN = lam_bounds
    rng = np.random.default_rng(seed)
    U = rng.random((A.shape[0], R))
    U /= np.linalg.norm(U, axis=0, keepdims=True)
    return make_problem(name, A, U, np.zeros((A.shape[0], 0)), np.zeros(0), funcs, m, C, l1, lN,
                        degree=degree, prob_dim=lN / 4, meta=dict(N=N))


def config3(N: int = 256, R: int = 1, seed: int = 0) -> FabProblem:
    """Mixed-precision large workload: 3D 7-point Laplacian on N^3 with
    kappa = 1 + 0.5 sin sin sin, f = exp(-5e-4 lambda^0.6), m = 100."""
    f = params.frac_exp(5e-4, 1.2)
    return fd3d_problem(N, 100, 32, [f] * R, R=R, seed=seed, name=f"fd3d-{N}-mixed")


def fe_disk_problem(n_target: int, k: int, m: int, C: int, degree: int, alpha: float = 1.6,
                    R: int = 1, seed: int = 0, ell: float = 0.1, sigma_g: float = 1.0,
                    deflation: str = "eigsh", name: str = "fe-disk"):
    """Nonuniform FE fractional-diffusion workload: P1 on a seeded Delaunay disk
    mesh, kappa = exp(g) per triangle (g a Gaussian field, sigma_g, correlation
    length ell), Dirichlet boundary, A = M^{-1/2} K M^{-1/2}, f = lambda^(-alpha/2),
    Jacobi polynomial with prob_dim = lN/4 (problem_startup_nonuniform.m:87)."""
    mesh = problems.disk_mesh(n_target, seed=seed)
    cent = mesh.nodes[mesh.tris].mean(axis=1)
    g = problems.gaussian_random_field(cent, sigma=sigma_g, ell=ell, seed=seed + 1)
    kappa = np.exp(g)
    A, ms, inner = problems.fe_operator(mesh, kappa)
    n = A.shape[0]
    import time
    import scipy.sparse.linalg as sla
    lmax = float(sla.eigsh(A, k=1, which="LA", return_eigenvectors=False, tol=1e-6)[0]) * 1.01
    timing = {}
    if k > 0:
        t0 = time.perf_counter()
        if deflation == "eigsh":
            # shift-invert at 0 with a symmetric minimum-degree ordering of the LU
            # (about 2x cheaper than scipy's default COLAMD on 2D meshes)
            lu = sla.splu(sp.csc_matrix(A), permc_spec="MMD_AT_PLUS_A", options=dict(SymmetricMode=True))
            op = sla.LinearOperator(A.shape, matvec=lu.solve, dtype=np.float64)
            lam, Q = sla.eigsh(A, k=k + 1, sigma=0.0, which="LM", OPinv=op, tol=1e-10)
            del lu
        elif deflation == "gpu":
            # Chebyshev-filtered subspace iteration on the GPU (gm_deflation_pairs)
            from . import eigs
            lam, Q, _ = eigs.deflation_pairs(A, k + 1)
        else:
            raise ValueError(deflation)
        timing[f"{deflation}_s"] = time.perf_counter() - t0
        o = np.argsort(lam)
        lam, Q = lam[o], Q[:, o]
        l1 = float(lam[k])  # first eigenvalue left after deflating k
        lam, Q = lam[:k], np.ascontiguousarray(Q[:, :k])
    else:
        lam0 = sla.eigsh(A, k=1, sigma=0.0, which="LM", return_eigenvectors=False)
        l1 = float(lam0[0])
        lam, Q = np.zeros(0), np.zeros((n, 0))
    rng = np.random.default_rng(seed + 2)
    U = rng.random((n, R))
    U /= np.linalg.norm(U, axis=0, keepdims=True)
    f = params.frac_power(-alpha / 2)
    return make_problem(name, A, U, Q, lam, [f] * R, m, C, l1, lmax, degree=degree,
                        prob_dim=lmax / 4, meta=dict(n_target=n_target, nt=mesh.tris.shape[0], seed=seed,
                                                     deflation=deflation, **timing),
                        row_weight=ms)


def config2(n_target: int = 1_000_000, R: int = 1, seed: int = 0) -> FabProblem:
    """FE disk with ~1M nodes, f = lambda^-0.8, degree-8 Jacobi polynomial,
    m = 80, 20 deflated vectors, 48 contour shifts."""
    return fe_disk_problem(n_target, 20, 80, 48, 8, alpha=1.6, R=R, seed=seed, name="fe-disk-1M-fp64")


def cached_problem(name: str, R: int = 1, cache_dir: str | None = None, seed: int = 0) -> FabProblem:
    """Build a named workload, caching the expensive operator/deflation setup
    (mesh, assembly, shift-invert eigenpairs) in ``cache_dir`` as .npz.

    Names: ``fe-disk-1M`` (1M-node FE disk), ``fe-disk-<n>`` (any node count),
    ``fd2d-256`` (256^2 Dirichlet Laplacian), ``fd3d-<N>`` (N^3 7-point).
    """
    import hashlib
    import os
    if name == "fd2d-256":
        return config1(R=R, seed=seed)
    if name.startswith("fd3d-"):
        return config3(N=int(name.split("-")[1]), R=R, seed=seed)
    if not name.startswith("fe-disk-"):
        raise ValueError(f"unknown workload {name}")
    tag = name.split("-")[2]
    n_target = 1_000_000 if tag == "1M" else int(tag)
    cache_dir = cache_dir or os.environ.get("GPUMATFUN_CACHE", os.path.join(os.environ.get("TMPDIR", "/tmp"), "gpumatfun_cache"))
    os.makedirs(cache_dir, exist_ok=True)
    key = hashlib.sha1(f"fe-disk|{n_target}|k20|seed{seed}|v2".encode()).hexdigest()[:12]
    path = os.path.join(cache_dir, f"fe-disk-{n_target}-{key}.npz")
    alpha = 1.6
    f = params.frac_power(-alpha / 2)
    if os.path.exists(path):
        z = np.load(path)
        A = sp.csr_matrix((z["data"], z["indices"], z["indptr"]), shape=tuple(z["shape"]))
        U = z["U"]
        if U.shape[1] < R:
            rng = np.random.default_rng(seed + 2)
            U = rng.random((A.shape[0], R))
            U /= np.linalg.norm(U, axis=0, keepdims=True)
        meta = dict(n_target=n_target, seed=seed, cached=True)
        if "eigsh_s" in z:
            meta["eigsh_s"] = float(z["eigsh_s"])
        return make_problem(f"fe-disk-{tag}-fp64", A, U[:, :R], z["Q"], z["lam"], [f] * R, 80, 48,
                            float(z["l1"]), float(z["lN"]), degree=8, prob_dim=float(z["lN"]) / 4,
                            meta=meta, row_weight=z["ms"])
    P = fe_disk_problem(n_target, 20, 80, 48, 8, alpha=alpha, R=max(R, 4), seed=seed, name=f"fe-disk-{tag}-fp64")
    tmp = path + f".tmp{os.getpid()}.npz"
    np.savez(tmp, data=P.A.data, indices=P.A.indices, indptr=P.A.indptr, shape=np.array(P.A.shape),
             U=P.U, Q=P.Q, lam=P.lam, l1=P.l1, lN=P.lN, ms=P.row_weight, eigsh_s=P.meta.get("eigsh_s", np.nan))
    os.replace(tmp, path)
    return make_problem(P.name, P.A, P.U[:, :R], P.Q, P.lam, [f] * R, 80, 48, P.l1, P.lN, degree=8,
                        prob_dim=P.lN / 4, meta=P.meta, row_weight=P.row_weight)


def batch_sizes(nprob: int, lo: int = 64, hi: int = 1024, seed: int = 0) -> np.ndarray:
    """Grid sides drawn log-uniformly in [lo, hi] from the seed."""
    rng = np.random.default_rng(seed)
    return np.round(np.exp(rng.uniform(math.log(lo), math.log(hi), nprob))).astype(int)


def config5_batch(nprob: int = 64, R: int = 4, seed: int = 0, lo: int = 64, hi: int = 1024,
                  m: int = 32, C: int = 32, alpha: float = 1.5, degree: int = 0, side: float = 2.5,
                  Kalpha: float = 1e-4, dt: float = 0.05) -> list:
    """Batched serving-style workload: ``nprob`` independent fractional
    diffusion problems, each one time step u <- exp(-dt K_alpha A^(alpha/2)) u
    (the monodomain's physical parameters: square of side 2.5, K_alpha = 1e-4,
    dt = 0.05, alpha = 1.5) on a 2D 5-point Dirichlet Laplacian with N^2
    interior nodes (N log-uniform in [lo, hi], A scaled by 1/h^2,
    h = side/(N+1)), R right-hand sides each, all solved by one launch."""
    f = params.frac_exp(Kalpha * dt, alpha)
    out = []
    for i, N in enumerate(batch_sizes(nprob, lo, hi, seed)):
        P = fd2d_problem(int(N), 0, m, C, [f] * R, R=R, scale=((N + 1.0) / side) ** 2, seed=seed + 1 + i,
                         degree=degree, name=f"batch{i}-{N}")
        out.append(P)
    return out


FHN = dict(aode=0.5 * 0.01, bode=-1 * 0.01, code=0.0, vrest=0.1, vamp=1.0, vth=0.0, vpeak=1.0, c1ion=-1.0,
           c2ion=0.0)


def monodomain_problem(N: int = 512, alpha: float = 1.5, Kalpha: float = 1e-4, dt: float = 0.05, k: int = 10,
                       m: int | None = None, C: int | None = None, tol: float | None = None):
    """Fractional monodomain (FitzHugh-Nagumo) time loop of
    problem_startup_monodomain.m:10-142 on an N x N Neumann grid over
    [0, 2.5]^2: eta = Kalpha dt / dx^alpha, f1 = exp(-eta x^(alpha/2)) for the
    solution column and f2 = phi(-eta x^(alpha/2)) for the reaction column,
    the k smallest cosine modes deflated (phi = 1 on the zero mode), m from the
    Krylov rule and C from the contour bound at tol = 1/N^2 unless given.
    Returns (FabProblem with R = 2, dt, ode, FHN parameters)."""
    tol = 1.0 / N ** 2 if tol is None else tol
    A = problems.laplacian_2d(N, "N", 1.0)
    lam, Q = problems.laplacian_2d_eigpairs(N, k, "N", 1.0)
    l1 = float(lam.max())
    lN = float(8 * math.sin((N - 1) * math.pi / (2 * N)) ** 2)
    dx = 2.5 / (N - 1)
    eta = Kalpha * dt / dx ** alpha
    f1 = params.frac_exp(eta, alpha)

    def f2(x):
        x = np.asarray(x)
        z = -eta * np.power(x, alpha / 2.0)
        with np.errstate(invalid="ignore", divide="ignore"):
            v = np.expm1(z) / z
        return np.where(z == 0, 1.0, v)

    if m is None:
        m = params.krylov_dim([1.0], l1, lN, tol)
    if C is None:
        C = params.contour_size_from_bound(l1, lN, [f1, f2], tol)
    g = np.linspace(0, 2.5, N)
    X, Y = np.meshgrid(g, g)
    ode = np.zeros_like(X)
    xh = np.zeros_like(X)
    ode[Y >= 1.25] = 0.1
    xh[(X <= 1.25) & (Y < 1.25)] = 1.0
    ode = ode.reshape(-1, order="F")
    xh = xh.reshape(-1, order="F")
    p = FHN
    yh = p["c1ion"] / p["vamp"] ** 2 * xh * (xh - p["vrest"]) * (xh - p["vpeak"]) - ode
    U = np.stack([xh, yh], axis=1)
    P = make_problem(f"monodomain-{N}", A, U, Q, lam, [f1, f2], m, C, l1, lN, degree=0, prob_dim=2.0,
                     meta=dict(N=N, alpha=alpha, Kalpha=Kalpha, dt=dt, eta=eta, k=k))
    return P, dt, ode, dict(p)


def adjoint_case(n_target: int = 250_000, seed: int = 0, sigma_g: float = 1.0, ell: float = 0.1):
    """Inverse-problem workload on the FE disk: the mesh, the current per-triangle
    coefficient kappa, the ground truth kappa* (two independent Gaussian fields,
    kappa = exp(g)) and a normalised b ~ U[0,1).  The data d = f(A(kappa*)) b
    plus 1% noise is synthesised by the caller with the engine it measures."""
    mesh = problems.disk_mesh(n_target, seed=seed)
    cent = mesh.nodes[mesh.tris].mean(axis=1)
    kstar = np.exp(problems.gaussian_random_field(cent, sigma=sigma_g, ell=ell, seed=seed + 1))
    kappa = np.exp(problems.gaussian_random_field(cent, sigma=sigma_g, ell=ell, seed=seed + 7))
    n = int((~mesh.boundary).sum())
    rng = np.random.default_rng(seed + 2)
    b = rng.random(n)
    b /= np.linalg.norm(b)
    return mesh, kappa, kstar, b


# Method parameters of the adjoint workload: degree-16 Jacobi polynomial and
# m = 900 converge f(A)b on the 250k-node disk (condition number ~4e6 for this
# coefficient field) to ~7e-10 vs m = 1600 (m = 500: 6e-6, m = 700: 8e-8);
# degree 24 is not usable (its monomial coefficients lose the approximation).
ADJOINT_PARAMS = dict(alpha=1.6, m=900, C=32, degree=16, margin=1.25)
