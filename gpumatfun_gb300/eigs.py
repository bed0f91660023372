"""Deflation pairs on the GPU: the k smallest eigenpairs of the operator.

The reference computes the deflation vectors at set-up with MATLAB's
``eigs(K, M, k, 'sm')`` (process_nonuniform.m:38-40, 106-110), a shift-invert
eigensolve on the host.  ``deflation_pairs`` computes them on the GPU through
``gm_deflation_pairs`` (Chebyshev-filtered subspace iteration over a block of
32 vectors, FP64, Rayleigh-Ritz on the GPU); see include/gpumatfun.h.
"""
from __future__ import annotations

import ctypes as ct

import numpy as np
import scipy.sparse as sp

from .engine import GmError, load_library

__all__ = ["deflation_pairs", "MAX_K"]

MAX_K = 24
_STATS = ("iterations", "block_spmvs", "device_s", "max_rel_residual", "gershgorin_bound", "filter_cut",
          "block_top_ritz", "nnz", "block_spmvs_float_float")


def deflation_pairs(A, k: int, tol: float = 1e-8, max_degree: int = 1000, max_iter: int = 200, seed: int = 0,
                    raise_on_noconv: bool = True, float_float_filter: bool = True):
    """(lambda (k,), Q (n, k), stats dict) for the k smallest eigenpairs of the
    symmetric sparse A, computed on the current CUDA device.  With
    ``float_float_filter`` the early filter applications run in float-float
    arithmetic on the FP32 pipe; otherwise every step is FP64."""
    lib = load_library()
    A = sp.csr_matrix(A)
    A.sort_indices()
    n = A.shape[0]
    rp = np.ascontiguousarray(A.indptr, dtype=np.int64)
    ci = np.ascontiguousarray(A.indices, dtype=np.int32)
    va = np.ascontiguousarray(A.data, dtype=np.float64)
    lam = np.empty(k)
    Q = np.empty((n, k), order="F")
    stats = (ct.c_double * 9)()
    deg = int(max_degree) if float_float_filter else -int(max_degree)
    rc = lib.gm_deflation_pairs(n, rp.ctypes.data, ci.ctypes.data, va.ctypes.data, int(k), float(tol),
                                deg, int(max_iter), int(seed), lam.ctypes.data, Q.ctypes.data, stats)
    info = dict(zip(_STATS, list(stats)))
    if rc != 0 and not (rc == 9 and not raise_on_noconv):
        raise GmError(rc, (lib.gm_last_error(None) or b"").decode())
    info["converged"] = rc == 0
    return lam, Q, info
