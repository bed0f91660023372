"""gm_lin_sys_solves_noalloc against gm_lin_sys_solves (through the C ABI).

The no-allocation entry point serves callers that cannot allocate device
memory themselves during a call -- applications whose device memory all
belongs to their own allocator (MATLAB's gpuArray manager, a framework's
caching pool) and latency-critical loops that cannot afford cudaMalloc's
implicit synchronisation.  They pass their own device buffers; the solve's
only scratch is a fixed file-scope device table.  This file is collected last
so that a failure here does not hide the rest of the suite; it also passes
when run on its own.
"""
import ctypes as ct

import numpy as np
import pytest

from gpumatfun_gb300 import Engine, workloads

pytestmark = pytest.mark.gpu

TOL = 1e-13


def _noalloc(lib):
    fn = lib.gm_lin_sys_solves_noalloc
    fn.argtypes = [ct.c_int, ct.c_int, ct.c_int, ct.c_void_p, ct.c_void_p, ct.c_void_p, ct.c_void_p,
                   ct.c_void_p, ct.c_void_p, ct.c_void_p]
    fn.restype = ct.c_int
    return fn


def _engine_reference(P):
    """y from the existing entry point gm_lin_sys_solves (and its inputs)."""
    eng = Engine.from_problem(P, precision="fp64")
    eng.build_subspace()
    eng.lin_sys_solves()
    aabb = eng.get_aabb()
    yr, yi = eng.get_y()
    meff = eng.meff()
    eng.delete()
    return aabb, yr, yi, meff


@pytest.mark.parametrize("R", [1, 2, 4])
def test_noalloc_solves_match_engine_two_calls(engine_lib, R):
    import torch
    fn = _noalloc(engine_lib)
    dev = torch.device("cuda", torch.cuda.current_device())
    outs = []
    for seed in (3, 4):  # two calls in a row, different inputs
        P = workloads.config1_small(N=20, k=3, m=30, C=24, R=R, degree=2, seed=seed)
        aabb, yr_ref, yi_ref, meff = _engine_reference(P)
        wts = np.concatenate([np.asarray(w).reshape(P.C, 2).T.reshape(-1) for w in P.wts])
        d_aabb = torch.tensor(aabb.T.reshape(-1), dtype=torch.float64, device=dev)   # column-major
        d_wts = torch.tensor(wts, dtype=torch.float64, device=dev)
        d_sh = torch.tensor(P.shifts, dtype=torch.float64, device=dev)
        d_meff = torch.tensor(meff, dtype=torch.int32, device=dev)
        d_yr = torch.full((R * P.C, P.m), np.nan, dtype=torch.float64, device=dev)
        d_yi = torch.full((R * P.C, P.m), np.nan, dtype=torch.float64, device=dev)
        stream = torch.cuda.current_stream().cuda_stream
        rc = fn(P.m, R, P.C, d_aabb.data_ptr(), d_meff.data_ptr(), d_wts.data_ptr(), d_sh.data_ptr(),
                d_yr.data_ptr(), d_yi.data_ptr(), stream)
        assert rc == 0, engine_lib.gm_last_error(None)
        torch.cuda.synchronize()
        yr = d_yr.cpu().numpy().T
        yi = d_yi.cpu().numpy().T
        y, yref = yr + 1j * yi, yr_ref + 1j * yi_ref
        assert np.linalg.norm(y - yref) / np.linalg.norm(yref) < TOL
        outs.append(y)
    assert not np.allclose(outs[0], outs[1])  # the second call did not return the first call's contents


def test_noalloc_rejects_oversize(engine_lib):
    fn = _noalloc(engine_lib)
    m, C, R = 300, 64, 4  # m * R * C = 76800 > GM_NOALLOC_MAX_ENTRIES
    rc = fn(m, R, C, 1, None, 1, 1, 1, 1, None)  # rejected before any pointer is touched
    assert rc == 1
    assert "exceeds the fixed scratch" in engine_lib.gm_last_error(None).decode()
