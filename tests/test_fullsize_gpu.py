"""Parity at the workloads' full sizes (through the C ABI).

- 1M-node FE disk (FP64 and mixed) against the FP64 oracle;
- 3D variable-coefficient Laplacian: FP64 engine against the oracle at 128^3,
  mixed engine against the FP64 engine at 256^3 (16.8M rows, 117M nnz);
- the 64-problem uneven batch (R = 4, mixed and FP64) against the
  per-problem oracle;
- the 512^2 fractional monodomain at the reference's Krylov-dimension rule
  (tol = 1/N^2 gives m = 1012, run_script.m:15) against the oracle's steps;
- the adjoint on a 2k-node submesh cut from the 250k-node disk mesh against
  the dense FP64 (Daleckii-Krein) gradient.

Tolerances: FP64 engine vs FP64 oracle 1e-10 relative; mixed engine vs FP64
(oracle or engine) 1e-6 relative; adjoint as in the 2k-disk tests (x and
dL/db 1e-9, dL/dkappa 1e-7).
"""
import numpy as np
import pytest

from gpumatfun_gb300 import BatchEngine, Engine, LanczosEngine, adjoint, params, problems, workloads
from oracle import adjoint as oadj
from oracle import fab

pytestmark = pytest.mark.gpu

FP64_TOL = 1e-10
MIXED_TOL = 1e-6


def rel(a, b):
    return float(np.linalg.norm(np.asarray(a) - np.asarray(b)) / np.linalg.norm(b))


def worst_col(a, b):
    a, b = np.asarray(a), np.asarray(b)
    return float(np.max(np.linalg.norm(a - b, axis=0) / np.linalg.norm(b, axis=0)))


def oracle_solve(P):
    return fab.OracleEngine(A=P.A, U0=P.U, Q=P.Q, m=P.m, gamma=P.gamma, gs_re=P.gs_re, gs_im=P.gs_im,
                            flam=P.flam, wts=P.wts, shifts=P.shifts, col_scale=np.ones(P.R)).solve()


def engine_solve(P, precision, **kw):
    eng = Engine.from_problem(P, precision=precision, **kw)
    eng.solve()
    x = eng.get_solution()
    eng.delete()
    return x


def test_fe_disk_1M_against_oracle(engine_lib):
    """The 1M-node FE disk (997,710 rows, 7.0M nnz, degree 8, m = 80,
    C = 48, k = 20 deflated pairs)."""
    P = workloads.cached_problem("fe-disk-1M", R=1)
    assert P.n > 990_000 and P.k == 20 and P.d == 8
    want = oracle_solve(P)
    x64 = engine_solve(P, "fp64")
    e64 = rel(x64, want)
    xm = engine_solve(P, "mixed")
    em = rel(xm, want)
    print(f"1M disk: fp64 {e64:.2e} mixed {em:.2e} vs oracle")
    assert e64 < FP64_TOL
    assert em < MIXED_TOL


def test_fd3d_128_fp64_against_oracle(engine_lib):
    P = workloads.config3(N=128)
    want = oracle_solve(P)
    x = engine_solve(P, "fp64")
    assert rel(x, want) < FP64_TOL


def test_fd3d_256_mixed_against_fp64_engine(engine_lib):
    """The 256^3 workload at full size: mixed (FP32 matrix and basis) against
    the FP64 engine on the same b."""
    P = workloads.config3(N=256)
    assert P.n == 256 ** 3 and P.A.nnz == 117_047_296
    x64 = engine_solve(P, "fp64")
    xm = engine_solve(P, "mixed")
    e = rel(xm, x64)
    print(f"256^3 mixed vs fp64 engine: {e:.2e}")
    assert e < MIXED_TOL


def test_batch64_against_per_problem_oracle(engine_lib):
    """All 64 problems (N from 64 to 1024, 11.7M rows in total), 4
    right-hand sides each, in one launch, in both precisions."""
    probs = workloads.config5_batch()
    assert len(probs) == 64 and all(P.R == 4 for P in probs)
    xs = {}
    for prec in ("mixed", "fp64"):
        eng = BatchEngine(probs, precision=prec, sync=False)
        eng.solve()
        xs[prec] = eng.split(eng.get_solution())
        eng.delete()
    worst = {"mixed": 0.0, "fp64": 0.0}
    for i, P in enumerate(probs):
        want = oracle_solve(P)
        for prec in worst:
            worst[prec] = max(worst[prec], worst_col(xs[prec][i], want))
    print(f"batch-64 worst problem: mixed {worst['mixed']:.2e} fp64 {worst['fp64']:.2e}")
    assert worst["fp64"] < FP64_TOL
    assert worst["mixed"] < MIXED_TOL


def test_monodomain_512_reference_m_rule(engine_lib):
    """Two CUDA-graph time steps of the 512^2 FitzHugh-Nagumo monodomain at
    the reference's m rule (m = 1012) against two oracle steps."""
    P, dt, ode, fhn = workloads.monodomain_problem(512)
    assert P.m > 1000
    steps = 2
    ora = fab.OracleEngine(A=P.A, U0=P.U, Q=P.Q, m=P.m, gamma=P.gamma, gs_re=P.gs_re, gs_im=P.gs_im,
                           flam=P.flam, wts=P.wts, shifts=P.shifts, dt=dt, ode=ode.copy(),
                           fhn=(fhn["aode"], fhn["bode"], fhn["code"], fhn["vrest"], fhn["vamp"], fhn["vth"],
                                fhn["vpeak"], fhn["c1ion"]))
    for _ in range(steps):
        ora.build_subspace(); ora.lin_sys_solves(); ora.apply_V(); ora.update_U_monodomain()
    want = ora.get_U()
    for prec, tol in (("fp64", FP64_TOL), ("mixed", MIXED_TOL)):
        e = LanczosEngine(P.U, P.A, P.Q, P.lam, P.m, P.gamma, P.gs_re, P.gs_im, P.flam[:, 0], P.flam[:, 1],
                          dt, ode, fhn["aode"], fhn["bode"], fhn["code"], fhn["vrest"], fhn["vamp"], fhn["vth"],
                          fhn["vpeak"], fhn["c1ion"], fhn["c2ion"], np.ones(P.n), P.wts[0], P.wts[1], P.shifts,
                          precision=prec, sync=False)
        e.time_loop(steps, monodomain=True, graph=True)
        got = e.get_U()
        e.delete()
        err = rel(got[:, 0], want[:, 0])
        print(f"monodomain 512^2 {prec}: u after {steps} steps {err:.2e} vs oracle")
        assert err < tol


def test_adjoint_on_2k_submesh_of_250k_mesh(engine_lib):
    """The adjoint workload's mesh (250k nodes) and coefficient fields, cut to
    the ~2k interior nodes within radius 0.095 of (0.25, -0.15): the GPU
    gradient against the dense FP64 gradient."""
    torch = pytest.importorskip("torch")
    mesh, kappa, kstar, _ = workloads.adjoint_case(250_000)
    sub, keep = problems.submesh(mesh, center=(0.25, -0.15), radius=0.095)
    ks, kss = kappa[keep], kstar[keep]
    n = int((~sub.boundary).sum())
    assert 1800 < n < 2400
    rng = np.random.default_rng(21)
    b = rng.random(n)
    b /= np.linalg.norm(b)
    f = params.frac_power(-0.8)
    fprime = lambda z: -0.8 * np.power(z, -1.8)
    A_star, *_ = oadj.fe_parts(sub, kss)
    lam, Q = np.linalg.eigh(A_star.toarray())
    xs = Q @ (f(lam) * (Q.T @ b))
    d = xs + 0.01 * np.linalg.norm(xs) / np.sqrt(n) * rng.standard_normal(n)
    op = adjoint.FracFEOperator(sub, ks, alpha=1.6, m=200, C=32, degree=8, margin=1.25)
    cu = lambda a: torch.as_tensor(np.asarray(a, dtype=np.float64), device="cuda")
    x = op.forward(cu(ks), cu(b))
    dk, db = op.backward(cu(ks), cu(b), x - cu(d))
    op.delete()
    _, x_ref, dk_ref, db_ref = oadj.dense_grad(sub, ks, b, d, f, fprime)
    ex, edb, edk = rel(x.cpu().numpy(), x_ref), rel(db.cpu().numpy(), db_ref), rel(dk.cpu().numpy(), dk_ref)
    print(f"2k submesh of the 250k disk: x {ex:.2e} dL/db {edb:.2e} dL/dkappa {edk:.2e}")
    assert ex < 1e-9
    assert edb < 1e-9
    assert edk < 1e-7
