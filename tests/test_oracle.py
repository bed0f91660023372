"""The oracle pinned against known answers (no GPU).

The reference cannot run here, so the FP64 restatement is pinned to the
reference's own validation mechanism (the DST exact solution of the Dirichlet
Laplacian, startup_nicksmethod_GPU.m:91-109), to dense eigendecompositions,
and to the FE meshes shipped with the reference (tests/golden/circle_fab.npz).
"""
import os

import numpy as np
import pytest
import scipy.sparse as sp

from gpumatfun_gb300 import params, workloads
from oracle import fab, known

GOLD = os.path.join(os.path.dirname(__file__), "golden")


def rel(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def oracle_for(P, **kw):
    return fab.OracleEngine(A=P.A, U0=P.U, Q=P.Q, m=P.m, gamma=P.gamma, gs_re=P.gs_re, gs_im=P.gs_im,
                            flam=P.flam, wts=P.wts, shifts=P.shifts, col_scale=np.ones(P.R), **kw)


@pytest.mark.parametrize("degree", [0, 3])
def test_oracle_vs_dst_exact(degree):
    N = 24
    P = workloads.config1_small(N=N, k=4, m=60, C=32, R=2, degree=degree)
    x = oracle_for(P).solve()
    for r in range(2):
        ex = known.dst_fab_2d(P.U[:, r], N, P.funcs[r], scale=(N + 1.0) ** 2)
        assert rel(x[:, r], ex) < 1e-12


def test_dst_vs_dense():
    N = 12
    A = workloads.problems.laplacian_2d(N, "D", 3.0)
    b = np.random.default_rng(0).random(N * N)
    f = params.frac_exp(0.05, 1.5)
    assert rel(known.dst_fab_2d(b, N, f, 3.0), known.dense_fab(A, b, f)) < 1e-13


def test_per_node_equals_collapsed_apply():
    P = workloads.config1_small(N=16, k=3, m=30, C=20, R=2, degree=4)
    a = oracle_for(P, apply_mode="ref").solve()
    b = oracle_for(P, apply_mode="collapsed").solve()
    assert rel(a, b) < 1e-13


def test_cpu_path_restatement_matches_engine_oracle():
    """nicksmethodcpu.m (weights applied to the solution, backslash solves)
    gives the same f(A)b as the engine's step order."""
    P = workloads.config1_small(N=16, k=3, m=30, C=20, R=2, degree=2)
    ora = oracle_for(P)
    want = ora.solve() - ora.update
    got = fab.nicksmethodcpu(P.wts, P.A, ora.U, P.C, P.m, P.gamma, P.gs_re, P.gs_im, P.sigma)
    assert rel(got, want) < 1e-12


def test_analytic_eigpairs():
    N = 10
    A = workloads.problems.laplacian_2d(N, "D", 2.0).toarray()
    lam, Q = workloads.problems.laplacian_2d_eigpairs(N, 7, "D", 2.0)
    np.testing.assert_allclose(A @ Q, Q * lam, atol=1e-12)
    np.testing.assert_allclose(Q.T @ Q, np.eye(7), atol=1e-12)
    assert np.all(np.diff(lam) >= 0)
    ev = np.linalg.eigvalsh(A)
    np.testing.assert_allclose(lam, ev[:7], rtol=1e-12)
    lamN, QN = workloads.problems.laplacian_2d_eigpairs(N, 5, "N", 1.0)
    AN = workloads.problems.laplacian_2d(N, "N", 1.0).toarray()
    np.testing.assert_allclose(AN @ QN, QN * lamN, atol=1e-12)


@pytest.mark.parametrize("case", ["circle1", "circle2"])
def test_oracle_vs_circle_golden(case):
    g = np.load(os.path.join(GOLD, "circle_fab.npz"))
    ptr, ind, dat = g[f"{case}_indptr"], g[f"{case}_indices"], g[f"{case}_data"]
    n = ptr.size - 1
    A = sp.csr_matrix((dat, ind, ptr), shape=(n, n))
    lam5, Q, b = g[f"{case}_lam"], g[f"{case}_Q"], g[f"{case}_b"]
    for fname, f, tol in (("pow", params.frac_power(-0.8), 1e-9), ("exp", params.frac_exp(0.01, 1.5), 1e-9)):
        P = workloads.make_problem(case, A, b[:, None], Q, lam5[:4], [f], m=min(n - 5, 120), C=48,
                                   l1=float(lam5[4]), lN=float(g[f"{case}_lmax"]) * 1.001)
        x = oracle_for(P).solve()[:, 0]
        assert rel(x, g[f"{case}_x_{fname}"]) < tol


def test_oracle_golden_fd16_stable():
    g = np.load(os.path.join(GOLD, "fd16_oracle.npz"))
    P = workloads.config1_small(N=16, k=3, m=24, C=16, R=2, degree=2)
    ora = oracle_for(P)
    ora.solve()
    assert rel(ora.X, g["X"]) < 1e-13
    assert rel(ora.update, g["update"]) < 1e-14


def test_update_U_semantics():
    rng = np.random.default_rng(0)
    X = rng.standard_normal((50, 2))
    upd = rng.standard_normal((50, 2))
    mass = 1 + rng.random(50)
    U = fab.update_U(X, upd, mass, 0.1)
    u = X.sum(1) + upd.sum(1)
    u = np.where(u >= 0, u, 0.0)
    np.testing.assert_allclose(U[:, 0], u)
    np.testing.assert_allclose(U[:, 1], 0.1 * mass * (u / mass) * (1 - u / mass))


@pytest.mark.parametrize("reorth", [1, 2])
def test_oracle_reorth_keeps_basis_orthonormal(reorth):
    """Degree 3, m = 40: the plain recurrence's basis loses orthogonality;
    Gram-Schmidt keeps it at rounding level, and f(A)b is unchanged to the
    method's accuracy (both agree with the exact DST solution)."""
    N = 20
    P = workloads.config1_small(N=N, k=3, m=40, C=20, R=1, degree=3, seed=3)
    ex = known.dst_fab_2d(P.U[:, 0], N, P.funcs[0], scale=(N + 1.0) ** 2)
    out = {}
    for ro in (0, reorth):
        o = fab.OracleEngine(A=P.A, U0=P.U, Q=P.Q, m=P.m, gamma=P.gamma, gs_re=P.gs_re, gs_im=P.gs_im,
                             flam=P.flam, wts=P.wts, shifts=P.shifts, col_scale=np.ones(1), reorth=ro)
        x = o.solve()[:, 0]
        V = o.V[0]
        out[ro] = (np.abs(V @ V.T - np.eye(P.m)).max(), np.linalg.norm(x - ex) / np.linalg.norm(ex))
    assert out[0][0] > 1e-2
    assert out[reorth][0] < 1e-14
    assert out[0][1] < 1e-11 and out[reorth][1] < 1e-11
