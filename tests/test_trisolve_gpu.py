"""Shifted tridiagonal solves at extreme scales (lanczos_impl.cu:292-406).

Scaling T, beta_0 and every shift by s leaves y = -beta_0 w (T - sigma)^{-1} e1
unchanged.  With s a power of two the scaling is exact in floating point, so
the GPU solve must return the same bits at s = 2^-530 (|T| ~ 1e-160),
s = 1 and s = 2^530 (|T| ~ 1e160), and match the oracle's banded LU
(oracle/fab.py::tridiag_solves) to the FP64 tolerance at every scale.  A
reciprocal formed as conj(g) / |g|^2, or a Schur update formed with beta^2,
overflows or underflows at these scales.
"""
import ctypes as ct

import numpy as np
import pytest

from gpumatfun_gb300 import Engine, params, workloads
from oracle import fab

pytestmark = pytest.mark.gpu

FP64_TOL = 1e-10


def rel(a, b):
    return float(np.linalg.norm(np.asarray(a) - np.asarray(b)) / max(np.linalg.norm(b), 1e-300))


def _solve_gpu(lib, m, R, C, aabb, wts_flat, shifts):
    """y through gm_lin_sys_solves_noalloc (the engine's solve phase on caller buffers)."""
    import torch
    fn = lib.gm_lin_sys_solves_noalloc
    fn.argtypes = [ct.c_int, ct.c_int, ct.c_int] + [ct.c_void_p] * 7
    fn.restype = ct.c_int
    dev = torch.device("cuda", torch.cuda.current_device())
    d_aabb = torch.tensor(aabb.T.reshape(-1), dtype=torch.float64, device=dev)
    d_wts = torch.tensor(wts_flat, dtype=torch.float64, device=dev)
    d_sh = torch.tensor(shifts, dtype=torch.float64, device=dev)
    d_yr = torch.full((R * C, m), np.nan, dtype=torch.float64, device=dev)
    d_yi = torch.full((R * C, m), np.nan, dtype=torch.float64, device=dev)
    rc = fn(m, R, C, d_aabb.data_ptr(), None, d_wts.data_ptr(), d_sh.data_ptr(), d_yr.data_ptr(),
            d_yi.data_ptr(), torch.cuda.current_stream().cuda_stream)
    assert rc == 0, lib.gm_last_error(None)
    torch.cuda.synchronize()
    return d_yr.cpu().numpy().T, d_yi.cpu().numpy().T


@pytest.mark.parametrize("R", [1, 4])
def test_solves_exact_under_power_of_two_scaling(engine_lib, R):
    P = workloads.config1_small(N=20, k=3, m=30, C=24, R=R, degree=0, seed=11)
    eng = Engine.from_problem(P, precision="fp64")
    eng.build_subspace()
    aabb = eng.get_aabb()
    eng.delete()
    m, C = P.m, P.C
    wts_flat = np.concatenate([np.asarray(w).reshape(C, 2).T.reshape(-1) for w in P.wts])
    base = None
    for e in (0, 530, -530):
        s = 2.0 ** e
        a_s = aabb * s
        sh_s = np.asarray(P.shifts) * s
        yr, yi = _solve_gpu(engine_lib, m, R, C, a_s, wts_flat, sh_s)
        y = yr + 1j * yi
        assert np.all(np.isfinite(y)), f"scale 2^{e}: non-finite solution"
        oyr, oyi = fab.tridiag_solves(a_s[:, :R].T, a_s[:, R:].T, P.wts, sh_s, m=m)
        assert rel(y, oyr + 1j * oyi) < FP64_TOL, (e, rel(y, oyr + 1j * oyi))
        if base is None:
            base = y
        else:
            np.testing.assert_array_equal(y, base)


def test_engine_on_operator_scaled_by_2_pow_490(engine_lib):
    """The whole engine on A * 2^490 (|T| ~ 1e150; the Lanczos norms reach
    ~1e302, still inside FP64), with f evaluated on the unscaled spectrum:
    f_s(lambda) = f(lambda / s), so f_s(sA) b = f(A) b.  Stepwise against the
    oracle on the same scaled inputs, and the solution against the unscaled
    problem's."""
    N = 20
    s = 2.0 ** 490
    f = params.frac_exp(1e-3, 1.5)
    fs = lambda x: f(np.asarray(x) / s)
    base = workloads.fd2d_problem(N, 0, 40, 32, [f], R=1, scale=(N + 1.0) ** 2, seed=6)
    P = workloads.make_problem("fd-scaled", base.A * s, base.U, base.Q, base.lam, [fs], base.m, base.C,
                               base.l1 * s, base.lN * s, degree=0)
    eng = Engine.from_problem(P, precision="fp64")
    ora = fab.OracleEngine(A=P.A, U0=P.U, Q=P.Q, m=P.m, gamma=P.gamma, gs_re=P.gs_re, gs_im=P.gs_im,
                           flam=P.flam, wts=P.wts, shifts=P.shifts, col_scale=np.ones(1))
    eng.build_subspace()
    ora.build_subspace()
    assert rel(eng.get_aabb(), ora.aabb()) < FP64_TOL
    eng.lin_sys_solves()
    ora.lin_sys_solves()
    yr, yi = eng.get_y()
    assert np.all(np.isfinite(yr)) and np.all(np.isfinite(yi))
    assert rel(yr + 1j * yi, ora.Yr + 1j * ora.Yi) < FP64_TOL
    eng.apply_V()
    x = eng.get_solution()
    eng.delete()
    e0 = Engine.from_problem(base, precision="fp64")
    e0.solve()
    x0 = e0.get_solution()
    e0.delete()
    assert rel(x, x0) < FP64_TOL
