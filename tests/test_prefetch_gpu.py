"""L2 bulk prefetch of the SELL values with each slice's column copy
(val_prefetch = 1 forces it; by default it is on only for matrices that do not
stay in the L2 persisting window, which these test sizes do).

The prefetch changes where a value comes from, not the arithmetic: results
must be bit-identical to the engine without it and within the FP64 parity
tolerance of the oracle.
"""
import os

import numpy as np
import pytest
import scipy.sparse as sp

from gpumatfun_gb300 import BatchEngine, Engine, params, workloads
from oracle import fab

pytestmark = pytest.mark.gpu

FP64_TOL = 1e-10


def rel(a, b):
    return float(np.linalg.norm(np.asarray(a) - np.asarray(b)) / max(np.linalg.norm(b), 1e-300))


def oracle_for(P, **kw):
    return fab.OracleEngine(A=P.A, U0=P.U, Q=P.Q, m=P.m, gamma=P.gamma, gs_re=P.gs_re, gs_im=P.gs_im,
                            flam=P.flam, wts=P.wts, shifts=P.shifts, col_scale=np.ones(P.R), **kw)


def solve(P, **kw):
    eng = Engine.from_problem(P, **kw)
    eng.solve()
    x = eng.get_solution()
    info = eng.info()
    eng.delete()
    return x, info


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
@pytest.mark.parametrize("R", [1, 2, 4])
@pytest.mark.parametrize("degree", [0, 3])
def test_prefetched_values_bit_identical(engine_lib, precision, R, degree):
    P = workloads.config1_small(N=40, k=3, m=30, C=20, R=R, degree=degree, seed=6)
    x0, i0 = solve(P, precision=precision, val_prefetch=2)
    x1, i1 = solve(P, precision=precision, val_prefetch=1)
    assert i0["value_prefetch_bytes"] == 0
    assert i1["value_prefetch_bytes"] == (8 if precision == "fp64" else 4)
    np.testing.assert_array_equal(x1, x0)
    if precision == "fp64":
        assert rel(x1, oracle_for(P).solve()) < FP64_TOL


def test_prefetched_values_fe_mesh(engine_lib):
    """Irregular FE rows (a reference mesh) with slices of several lengths."""
    g = np.load(os.path.join(os.path.dirname(__file__), "golden", "circle_fab.npz"))
    ptr, ind, dat = g["circle2_indptr"], g["circle2_indices"], g["circle2_data"]
    n = ptr.size - 1
    A = sp.csr_matrix((dat, ind, ptr), shape=(n, n))
    lam5, Q = g["circle2_lam"], g["circle2_Q"]
    P = workloads.make_problem("circle2", A, g["circle2_b"][:, None], Q, lam5[:4], [params.frac_power(-0.8)],
                               m=60, C=32, l1=float(lam5[4]), lN=float(g["circle2_lmax"]) * 1.001, degree=4,
                               prob_dim=float(g["circle2_lmax"]) / 4)
    x0, _ = solve(P, val_prefetch=2)
    x1, i1 = solve(P, val_prefetch=1)
    assert i1["value_prefetch_bytes"] == 8
    np.testing.assert_array_equal(x1, x0)
    assert rel(x1, oracle_for(P).solve()) < FP64_TOL


def test_prefetched_values_many_blocks_and_policies(engine_lib):
    N = 180
    P = workloads.fd2d_problem(N, 3, 24, 24, [params.frac_exp(1e-3, 1.5)] * 2, R=2, scale=(N + 1.0) ** 2,
                               seed=2, degree=3)
    want = oracle_for(P).solve()
    out = []
    for pol in (0, 1):
        eng = Engine.from_problem(P, sync_policy=pol, threads=128, sync=False, val_prefetch=1)
        assert eng.info()["grid_blocks"] > 200
        for _ in range(2):
            eng.solve()
            out.append(eng.get_solution())
        eng.delete()
    for x in out[1:]:
        np.testing.assert_array_equal(x, out[0])
    assert rel(out[0], want) < FP64_TOL


def test_prefetched_values_with_matrix_powers_and_sigma(engine_lib):
    P = workloads.config1_small(N=48, k=3, m=20, C=20, R=1, degree=5, seed=9)
    x0, _ = solve(P, val_prefetch=2)
    x1, i1 = solve(P, val_prefetch=1, matrix_powers=1)
    assert i1["matrix_powers"] == 1
    np.testing.assert_array_equal(x1, x0)
    x2, _ = solve(P, val_prefetch=1, sell_sigma=64)
    assert rel(x2, x0) < 1e-13


def test_prefetched_values_batch(engine_lib):
    probs = workloads.config5_batch(nprob=5, R=2, seed=4, lo=12, hi=60, m=24, C=20, degree=2)
    xs = []
    for vs in (2, 1):
        eng = BatchEngine(probs, precision="fp64", sync=False, threads=128, val_prefetch=vs)
        eng.solve()
        xs.append(eng.get_solution())
        eng.delete()
    np.testing.assert_array_equal(xs[1], xs[0])
