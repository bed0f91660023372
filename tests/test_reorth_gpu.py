"""Gram-Schmidt reorthogonalisation (reorth = 1: classical Gram-Schmidt,
2: twice) on the GPU against the FP64 oracle's, through the C ABI.

The reference's recurrence has no reorthogonalisation (build_subspace.cu:53-88);
the oracle's optional CGS runs after w -= alpha_j v_j and before
beta_{j+1} = ||w||, as the engine's does.  Tolerances: FP64 engine vs FP64
oracle 1e-10 relative; mixed engine vs FP64 oracle 1e-6 relative.
"""
import numpy as np
import pytest

from gpumatfun_gb300 import BatchEngine, Engine, GmError, params, workloads
from oracle import fab

pytestmark = pytest.mark.gpu

FP64_TOL = 1e-10
MIXED_TOL = 1e-6


def rel(a, b):
    return float(np.linalg.norm(np.asarray(a) - np.asarray(b)) / max(np.linalg.norm(b), 1e-300))


def oracle_for(P, **kw):
    return fab.OracleEngine(A=P.A, U0=P.U, Q=P.Q, m=P.m, gamma=P.gamma, gs_re=P.gs_re, gs_im=P.gs_im,
                            flam=P.flam, wts=P.wts, shifts=P.shifts, col_scale=np.ones(P.R), **kw)


def orth_loss(V):
    """max |V^T V - I| of one right-hand side's basis (m, n)."""
    return float(np.abs(V @ V.T - np.eye(V.shape[0])).max())


# Degree 3 and m = 40 on the 20 x 20 grid: the plain recurrence loses
# orthogonality (max |V^T V - I| about 0.6 in the oracle) while f(A)b has
# converged; past that point alpha/beta depend on rounding, so longer runs are
# compared on the solution and on the basis's orthogonality.
def long_case(R):
    return workloads.config1_small(N=20, k=3, m=40, C=20, R=R, degree=3, seed=3)


@pytest.mark.parametrize("R", [1, 2, 4])
@pytest.mark.parametrize("reorth", [1, 2])
def test_reorth_parity_fp64(engine_lib, R, reorth):
    P = long_case(R)
    eng = Engine.from_problem(P, reorth=reorth)
    eng.solve()
    want = oracle_for(P, reorth=reorth).solve()
    assert rel(eng.get_solution(), want) < FP64_TOL
    V = eng.get_basis()
    assert V.shape == (R, P.m, P.n)
    for r in range(R):
        assert orth_loss(V[r]) < 1e-13
    eng.delete()


def test_plain_recurrence_loses_orthogonality(engine_lib):
    P = long_case(1)
    eng = Engine.from_problem(P, reorth=0)
    eng.solve()
    assert orth_loss(eng.get_basis()[0]) > 1e-3
    eng.delete()


@pytest.mark.parametrize("reorth", [0, 1, 2])
def test_basis_and_recurrence_stepwise(engine_lib, reorth):
    # m = 12: alpha, beta and V are well conditioned and compared directly
    P = workloads.config1_small(N=20, k=3, m=12, C=20, R=2, degree=3, seed=3)
    eng = Engine.from_problem(P, reorth=reorth)
    ora = oracle_for(P, reorth=reorth)
    eng.build_subspace()
    ora.build_subspace()
    assert rel(eng.get_basis(), ora.V) < FP64_TOL
    assert rel(eng.get_aabb(), ora.aabb()) < FP64_TOL
    eng.lin_sys_solves(); eng.apply_V()
    ora.lin_sys_solves(); ora.apply_V()
    assert rel(eng.get_solution(), ora.X + ora.update) < FP64_TOL
    eng.delete()


@pytest.mark.parametrize("reorth", [1, 2])
def test_reorth_mixed(engine_lib, reorth):
    P = long_case(2)
    eng = Engine.from_problem(P, precision="mixed", reorth=reorth)
    eng.solve()
    assert rel(eng.get_solution(), oracle_for(P, reorth=reorth).solve()) < MIXED_TOL
    V = eng.get_basis()
    for r in range(2):
        assert orth_loss(V[r]) < 1e-5   # FP32-stored vectors
    eng.delete()


def test_reorth_batch(engine_lib):
    probs = workloads.config5_batch(nprob=5, R=2, seed=4, lo=12, hi=60, m=30, C=20, degree=3)
    eng = BatchEngine(probs, precision="fp64", sync=False, threads=128, reorth=1)
    eng.solve()
    for P, x in zip(probs, eng.split(eng.get_solution())):
        assert rel(x, oracle_for(P, reorth=1).solve()) < FP64_TOL
    V = eng.get_basis()
    row0 = eng.row0
    for p in range(len(probs)):
        for r in range(2):
            Vp = V[r][:, row0[p]:row0[p + 1]]
            # each problem's own basis is orthonormal (its meff columns)
            assert orth_loss(Vp[: eng.meff()[p * 2 + r]]) < 1e-12
    eng.delete()


def test_reorth_deterministic_on_many_blocks(engine_lib):
    """Hundreds of blocks: per-block partial dots and their fixed-order totals
    give the same bits on every run and with either pass ordering."""
    N = 180
    P = workloads.fd2d_problem(N, 3, 24, 24, [params.frac_exp(1e-3, 1.5)] * 2, R=2, scale=(N + 1.0) ** 2,
                               seed=2, degree=3)
    want = oracle_for(P, reorth=2).solve()
    out = []
    for pol in (0, 1):
        eng = Engine.from_problem(P, sync_policy=pol, threads=128, sync=False, reorth=2)
        assert eng.info()["grid_blocks"] > 200
        for _ in range(3):
            eng.solve()
            out.append(eng.get_solution())
        eng.delete()
    for x in out[1:]:
        np.testing.assert_array_equal(x, out[0])
    assert rel(out[0], want) < FP64_TOL


def test_reorth_takes_precedence_over_matrix_powers(engine_lib):
    P = workloads.config1_small(N=20, k=3, m=12, C=20, R=1, degree=4, seed=3)
    eng = Engine.from_problem(P, reorth=1, matrix_powers=1)
    assert eng.info()["matrix_powers"] == 0
    eng.solve()
    assert rel(eng.get_solution(), oracle_for(P, reorth=1).solve()) < FP64_TOL
    eng.delete()


def test_reorth_argument_checked(engine_lib):
    P = workloads.config1_small(N=8, k=2, m=6, C=8, R=1, degree=0, seed=1)
    with pytest.raises(GmError, match="reorth"):
        Engine.from_problem(P, reorth=3)


@pytest.mark.parametrize("reorth", [1, 2])
def test_reorth_breakdown_invariant_subspace(engine_lib, reorth):
    """b on 3 coordinates of a diagonal A: the Krylov space is 3-dimensional;
    Gram-Schmidt leaves beta_3 at rounding level, the default tolerance stops
    the recurrence at m_eff = 3 and f(A)b is exact."""
    import scipy.sparse as sp
    n = 64
    d = np.linspace(1.0, 10.0, n)
    A = sp.diags(d).tocsr()
    b = np.zeros(n)
    b[[3, 20, 50]] = [1.0, -2.0, 0.5]
    f = params.frac_power(-0.8)
    P = workloads.make_problem("diag", A, b[:, None], np.zeros((n, 0)), np.zeros(0), [f], m=12, C=40,
                               l1=0.9, lN=11.0, degree=0)
    eng = Engine.from_problem(P, reorth=reorth)
    eng.solve()
    assert eng.meff()[0] == 3
    assert rel(eng.get_solution()[:, 0], f(d) * b) < 1e-9
    V = eng.get_basis()[0]
    assert orth_loss(V[:3]) < 1e-14
    eng.delete()
