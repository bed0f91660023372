"""GPU parity of the CUDA engine against the FP64 oracle (through the C ABI).

Tolerances: FP64 engine vs FP64 oracle 1e-10 relative (the FP64 parity
tolerance); mixed engine vs FP64 oracle 1e-6 relative.  Sizes are such that the
oracle finishes in well under a second per case.
"""
import numpy as np
import pytest
import scipy.sparse as sp

from gpumatfun_gb300 import Engine, GmError, LanczosEngine, params, workloads
from oracle import fab, known

pytestmark = pytest.mark.gpu

FP64_TOL = 1e-10
MIXED_TOL = 1e-6


def rel(a, b):
    return float(np.linalg.norm(np.asarray(a) - np.asarray(b)) / max(np.linalg.norm(b), 1e-300))


def oracle_for(P, **kw):
    cs = kw.pop("col_scale", np.ones(P.R))
    return fab.OracleEngine(A=P.A, U0=P.U, Q=P.Q, m=P.m, gamma=P.gamma, gs_re=P.gs_re, gs_im=P.gs_im,
                            flam=P.flam, wts=P.wts, shifts=P.shifts, col_scale=cs, **kw)


@pytest.mark.parametrize("R", [1, 2, 4])
@pytest.mark.parametrize("degree", [0, 3])
def test_stepwise_parity_fp64(engine_lib, R, degree):
    # m = 12 keeps alpha/beta well conditioned on this grid: past the point where
    # Ritz values converge, a 1e-16 change in rounding moves alpha/beta by ~1e-2
    # while f(A)b stays within 1e-15, so longer runs are compared on the solution.
    P = workloads.config1_small(N=20, k=3, m=12, C=20, R=R, degree=degree, seed=3)
    eng = Engine.from_problem(P, precision="fp64")
    ora = oracle_for(P)
    np.testing.assert_allclose(eng.get_U(), ora.get_U(), rtol=0, atol=1e-14)
    assert rel(eng.get_update(), ora.update) < FP64_TOL
    eng.build_subspace()
    ora.build_subspace()
    ab_g, ab_o = eng.get_aabb(), ora.aabb()
    assert rel(ab_g, ab_o) < FP64_TOL, rel(ab_g, ab_o)
    eng.lin_sys_solves()
    ora.lin_sys_solves()
    yr, yi = eng.get_y()
    assert rel(yr + 1j * yi, ora.Yr + 1j * ora.Yi) < FP64_TOL
    eng.apply_V()
    ora.apply_V()
    assert rel(eng.get_xsol(), ora.X) < FP64_TOL
    assert rel(eng.get_solution(), ora.X + ora.update) < FP64_TOL
    eng.delete()


@pytest.mark.parametrize("degree", [0, 2])
def test_fused_solve_matches_exact(engine_lib, degree):
    N = 24
    P = workloads.config1_small(N=N, k=4, m=60, C=32, R=2, degree=degree, seed=5)
    eng = Engine.from_problem(P)
    eng.solve()
    x = eng.get_solution()
    for r in range(2):
        ex = known.dst_fab_2d(P.U[:, r], N, P.funcs[r], scale=(N + 1.0) ** 2)
        assert rel(x[:, r], ex) < 1e-9


def test_reference_api_time_steps(engine_lib):
    """lanczosEngine drop-in: CSC input, [1, dt] column scaling, update_U steps."""
    P = workloads.config1_small(N=16, k=3, m=24, C=16, R=2, degree=1, seed=7)
    dt = 0.1
    rng = np.random.default_rng(0)
    U = rng.random((P.n, 2)) * 0.5
    mass = 1.0 + 0.1 * rng.random(P.n)
    L = LanczosEngine(U, sp.csc_matrix(P.A), P.Q, P.lam, P.m, P.gamma, P.gs_re, P.gs_im,
                      P.flam[:, 0], P.flam[:, 1], dt, np.zeros(P.n), 0, 0, 0, 0, 1, 0, 0, 0, 0,
                      mass, P.wts[0], P.wts[1], P.shifts)
    ora = fab.OracleEngine(A=P.A, U0=U, Q=P.Q, m=P.m, gamma=P.gamma, gs_re=P.gs_re, gs_im=P.gs_im,
                           flam=P.flam, wts=P.wts, shifts=P.shifts, dt=dt, mass=mass)
    for _ in range(3):
        L.build_subspace(); ora.build_subspace()
        L.lin_sys_solves(); ora.lin_sys_solves()
        L.apply_V(); ora.apply_V()
        assert rel(L.get_xsol(), ora.get_xsol()) < FP64_TOL
        L.update_U(); ora.update_U()
        assert rel(L.get_U(), ora.get_U()) < FP64_TOL
        assert np.all(L.get_xsol() == 0.0)
    L.delete()


def test_monodomain_steps(engine_lib):
    P = workloads.config1_small(N=16, k=3, m=24, C=16, R=2, degree=0, seed=9)
    fhn = dict(aode=0.005, bode=-0.01, code=0.0, vrest=0.1, vamp=1.0, vth=0.0, vpeak=1.0, c1ion=-1.0, c2ion=0.0)
    dt = 0.05
    rng = np.random.default_rng(1)
    xh = (rng.random(P.n) > 0.7).astype(float)
    ode = 0.1 * (rng.random(P.n) > 0.5)
    yh = fhn["c1ion"] * xh * (xh - fhn["vrest"]) * (xh - fhn["vpeak"]) - ode
    U = np.stack([xh, yh], 1)
    L = LanczosEngine(U, P.A, P.Q, P.lam, P.m, P.gamma, P.gs_re, P.gs_im, P.flam[:, 0], P.flam[:, 1],
                      dt, ode, fhn["aode"], fhn["bode"], fhn["code"], fhn["vrest"], fhn["vamp"], fhn["vth"],
                      fhn["vpeak"], fhn["c1ion"], fhn["c2ion"], np.ones(P.n), P.wts[0], P.wts[1], P.shifts)
    ora = fab.OracleEngine(A=P.A, U0=U, Q=P.Q, m=P.m, gamma=P.gamma, gs_re=P.gs_re, gs_im=P.gs_im,
                           flam=P.flam, wts=P.wts, shifts=P.shifts, dt=dt, ode=ode.copy(),
                           fhn=(fhn["aode"], fhn["bode"], fhn["code"], fhn["vrest"], fhn["vamp"],
                                fhn["vth"], fhn["vpeak"], fhn["c1ion"]))
    for _ in range(3):
        for o in (L, ora):
            o.build_subspace(); o.lin_sys_solves(); o.apply_V(); o.update_U_monodomain()
        assert rel(L.get_U(), ora.get_U()) < FP64_TOL
    L.delete()


def test_set_y_apply(engine_lib):
    # arbitrary y exposes every Krylov vector individually, so m stays in the
    # range where V itself (not only f(A)b) is rounding-stable
    P = workloads.config1_small(N=16, k=2, m=10, C=12, R=2, degree=2, seed=2)
    eng = Engine.from_problem(P)
    ora = oracle_for(P)
    eng.build_subspace(); ora.build_subspace()
    rng = np.random.default_rng(3)
    yr, yi = rng.standard_normal((P.m, 2 * P.C)), rng.standard_normal((P.m, 2 * P.C))
    eng.set_y(yr, yi)
    ora.Yr, ora.Yi = yr, yi
    eng.apply_V(); ora.apply_V()
    assert rel(eng.get_xsol(), ora.X) < FP64_TOL
    gyr, gyi = eng.get_y()
    np.testing.assert_array_equal(gyr, yr)


def test_repeated_fused_solve_is_idempotent(engine_lib):
    """gm_solve writes X (the MEX apply_V accumulates into X, as the reference)."""
    P = workloads.config1_small(N=16, k=2, m=20, C=12, R=1, degree=1, seed=6)
    eng = Engine.from_problem(P, sync=False)
    eng.solve()
    x1 = eng.get_solution()
    for _ in range(3):
        eng.solve()
    np.testing.assert_array_equal(eng.get_solution(), x1)
    eng.apply_V()
    np.testing.assert_allclose(eng.get_xsol(), 2 * (x1 - eng.get_update()), rtol=1e-13, atol=1e-300)


def test_oracle_golden_fd16(engine_lib):
    g = np.load(__import__("os").path.join(__import__("os").path.dirname(__file__), "golden", "fd16_oracle.npz"))
    P = workloads.config1_small(N=16, k=3, m=24, C=16, R=2, degree=2)
    eng = Engine.from_problem(P)
    eng.solve()
    assert rel(eng.get_xsol(), g["X"]) < FP64_TOL


@pytest.mark.parametrize("case", ["circle1", "circle2"])
def test_fe_circle_golden(engine_lib, case):
    """FE meshes shipped with the reference: engine vs dense-eigh f(A)b."""
    import os
    g = np.load(os.path.join(os.path.dirname(__file__), "golden", "circle_fab.npz"))
    ptr, ind, dat = g[f"{case}_indptr"], g[f"{case}_indices"], g[f"{case}_data"]
    n = ptr.size - 1
    A = sp.csr_matrix((dat, ind, ptr), shape=(n, n))
    lam5 = g[f"{case}_lam"]
    Q = g[f"{case}_Q"]
    k = 4
    b = g[f"{case}_b"]
    lN = float(g[f"{case}_lmax"]) * 1.001
    f = params.frac_power(-0.8)
    P = workloads.make_problem(case, A, b[:, None], Q, lam5[:k], [f], m=min(n - k - 1, 120), C=48,
                               l1=float(lam5[k]), lN=lN, degree=0)
    eng = Engine.from_problem(P)
    eng.solve()
    x = eng.get_solution()[:, 0]
    ora = oracle_for(P)
    assert rel(x, ora.solve()[:, 0]) < FP64_TOL
    assert rel(x, g[f"{case}_x_pow"]) < 1e-6


@pytest.mark.parametrize("degree", [0, 4])
def test_mixed_precision_large_scale_operator(engine_lib, degree):
    """h^-2-scaled operator with a degree-4 polynomial: the polynomial
    coefficients and A^4 leave FP32's range unless the engine rescales."""
    N = 48
    P = workloads.fd2d_problem(N, 4, 40, 32, [params.frac_power(-0.8)], R=1, scale=1e6 * (N + 1.0) ** 2,
                               seed=3, degree=degree)
    want = oracle_for(P).solve()
    eng = Engine.from_problem(P, precision="mixed")
    eng.solve()
    assert rel(eng.get_solution(), want) < MIXED_TOL
    e64 = Engine.from_problem(P, precision="fp64")
    e64.build_subspace()
    eng.build_subspace()
    ab, ab64 = eng.get_aabb(), e64.get_aabb()
    assert rel(ab[:5], ab64[:5]) < 1e-5


def test_mixed_precision_config1_small(engine_lib):
    P = workloads.config1_small(N=32, k=4, m=60, C=32, R=2, degree=0, seed=4)
    ora = oracle_for(P)
    want = ora.solve()
    eng = Engine.from_problem(P, precision="mixed")
    eng.solve()
    got = eng.get_solution()
    assert rel(got, want) < MIXED_TOL, rel(got, want)


@pytest.mark.parametrize("R", [1, 2])
def test_config1_full_size_fp64(engine_lib, R):
    """The 256 x 256 plain workload at full size against the oracle."""
    P = workloads.config1(R=R)
    ora = oracle_for(P)
    want = ora.solve()
    eng = Engine.from_problem(P)
    eng.solve()
    got = eng.get_solution()
    assert rel(got, want) < FP64_TOL
    ab = eng.get_aabb()
    assert rel(ab, ora.aabb()) < FP64_TOL


def test_breakdown_eigenvector_rhs(engine_lib):
    """b in a 3-dimensional invariant subspace: Lanczos stops at m_eff = 3
    (the reference would divide by beta = 0) and f(A)b is still exact."""
    N = 12
    A = workloads.problems.laplacian_2d(N, "D", 1.0)
    lam, Qe = workloads.problems.laplacian_2d_eigpairs(N, 6, "D", 1.0)
    b = Qe[:, [0, 3, 5]] @ np.array([1.0, 0.5, 0.25])
    f = params.frac_exp(0.1, 1.5)
    P = workloads.make_problem("bd", A, b[:, None], np.zeros((N * N, 0)), np.zeros(0), [f], m=20, C=40,
                               l1=float(lam[0]) * 0.9, lN=8.0, degree=0)
    # rounding residue of the analytic eigenvectors grows to beta_3 ~ 2e-12
    eng = Engine.from_problem(P, breakdown_tol=1e-10)
    eng.solve()
    assert eng.meff()[0] == 3
    x = eng.get_solution()[:, 0]
    assert rel(x, known.dense_fab(A, b, f)) < 1e-9


def test_exact_breakdown_default_tolerance(engine_lib):
    """Diagonal A and b on 3 coordinates: the Krylov space is exactly
    3-dimensional, beta_3 is at rounding level and the default tolerance stops."""
    n = 64
    d = np.linspace(1.0, 10.0, n)
    A = sp.diags(d).tocsr()
    b = np.zeros(n)
    b[[3, 20, 50]] = [1.0, -2.0, 0.5]
    f = params.frac_power(-0.8)
    P = workloads.make_problem("diag", A, b[:, None], np.zeros((n, 0)), np.zeros(0), [f], m=12, C=40,
                               l1=0.9, lN=11.0, degree=0)
    eng = Engine.from_problem(P)
    eng.solve()
    assert eng.meff()[0] == 3
    assert rel(eng.get_solution()[:, 0], f(d) * b) < 1e-9


def test_zero_rhs(engine_lib):
    P = workloads.config1_small(N=12, k=2, m=10, C=8, R=1)
    eng = Engine.from_problem(P)
    eng.set_U(np.zeros((P.n, 1)))
    eng.solve()
    assert eng.meff() == [0]
    assert np.all(eng.get_solution() == 0.0)


@pytest.mark.parametrize("degree", [0, 3, 6])
def test_sync_policies_agree(engine_lib, degree):
    """Neighbour waits between SpMV passes (default) and grid barriers, with
    the SELL column indices staged in shared memory by TMA or read directly,
    give the same bits: the passes compute identical values in identical order.
    The grid is large (hundreds of blocks, several Horner passes in both the
    Lanczos and the apply phase) so that an ordering race would show."""
    N = 180
    P = workloads.fd2d_problem(N, 3, 24, 24, [params.frac_exp(1e-3, 1.5)] * 2, R=2, scale=(N + 1.0) ** 2,
                               seed=2, degree=degree)
    want = oracle_for(P).solve()
    out = []
    for pol, stg in ((0, 1), (1, 1), (0, 2), (1, 2)):   # and column staging off / on
        eng = Engine.from_problem(P, sync_policy=pol, threads=128, sync=False, col_staging=stg)
        info = eng.info()
        assert info["grid_blocks"] > 200
        assert info["neighbour_waits"] == (1 if pol == 0 else 0)
        assert (info["col_stage_groups"] > 0) == (stg == 2)
        for _ in range(3):
            eng.solve()
            out.append(eng.get_solution())
        eng.set_U(P.U)  # X = 0 again: apply_V accumulates
        eng.build_subspace(); eng.lin_sys_solves(); eng.apply_V()
        out.append(eng.get_solution())
        eng.delete()
    for x in out[1:]:
        np.testing.assert_array_equal(x, out[0])
    assert rel(out[0], want) < FP64_TOL


def test_info_ex_reports_l2_window_and_staging(engine_lib):
    """gm_info_ex: the L2 window and the column staging each engine chose
    (auto: window when the matrix and one pass's vectors fit L2; staging
    without a window, and with one in the FP64 engine but not in the mixed
    one), and a count below the total fills only that many."""
    import ctypes as ct
    P = workloads.fd2d_problem(64, 2, 24, 24, [params.frac_exp(1e-3, 1.5)], R=1, scale=65.0 ** 2, seed=3)
    for prec, win, stg in (("fp64", 0, 0), ("fp64", 1, 0), ("fp64", 2, 0), ("fp64", 1, 2), ("fp64", 0, 1),
                           ("mixed", 0, 0), ("mixed", 1, 0)):
        mat_bytes = (8 if prec == "fp64" else 4) * P.A.nnz
        eng = Engine.from_problem(P, precision=prec, l2_window=win, col_staging=stg)
        info = eng.info()
        if win == 1:
            assert info["l2_window_bytes"] == 0
            assert (info["col_stage_groups"] > 0) == (stg in (0, 2))
        else:
            assert info["l2_window_bytes"] >= mat_bytes
            assert (info["col_stage_groups"] > 0) == (prec == "fp64" and stg == 0)
        v = (ct.c_int64 * 19)(*([-7] * 19))
        assert engine_lib.gm_info_ex(eng._h, v, 3) == 0
        assert list(v)[:3] == [P.n, 1, P.m] and list(v)[3:] == [-7] * 16
        eng.delete()


def test_no_deflation_and_sigma_sorted(engine_lib):
    P = workloads.fd2d_problem(20, 0, 40, 24, [params.frac_exp(1e-3, 1.5)], R=1, scale=441.0, seed=8)
    ora = oracle_for(P)
    want = ora.solve()
    for sigma in (0, 64):
        eng = Engine.from_problem(P, sell_sigma=sigma, threads=256, blocks_per_sm=1)
        eng.solve()
        assert rel(eng.get_solution(), want) < FP64_TOL


def test_solve_host_end_to_end(engine_lib):
    P = workloads.config1_small(N=16, k=3, m=30, C=20, R=2, degree=1)
    eng = Engine.from_problem(P, sync=False)
    rng = np.random.default_rng(4)
    b = np.asfortranarray(rng.random((P.n, 2)))
    x = eng.solve_host(b)
    P.U = b
    ora = oracle_for(P)
    assert rel(x, ora.solve()) < FP64_TOL
    t = eng.phase_times()
    assert t["solve"] > 0


def test_create_errors(engine_lib):
    P = workloads.config1_small(N=8, k=1, m=6, C=4, R=2)
    with pytest.raises(GmError, match="bad_shifts"):
        Engine(P.A, P.U, P.Q, P.lam, P.flam, P.m, P.gamma, P.gs_re, P.gs_im, P.wts, P.shifts[:-2])
    eng = Engine.from_problem(P)
    with pytest.raises(GmError, match="GM_ERR_STATE"):
        eng.apply_V()
