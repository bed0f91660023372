"""Loader for the C/OpenMP restatement of the reference CPU path (cpu_fab.c).

Test infrastructure and timed CPU baseline only: ``bench.py`` times it as the
reference arm (the reference's own CPU path is MATLAB and cannot run here) and
tests check it against the numpy oracle.  ``build()`` compiles it with gcc
into oracle/_lib/ (not tracked).
"""
from __future__ import annotations

import ctypes as ct
import os
import shutil
import subprocess
from pathlib import Path

import numpy as np
import scipy.sparse as sp

HERE = Path(__file__).resolve().parent
SRC = HERE / "cpu_fab.c"
LIB = HERE / "_lib" / "libcpufab.so"
_lib = None


def build(force: bool = False) -> Path:
    if LIB.exists() and not force and LIB.stat().st_mtime >= SRC.stat().st_mtime:
        return LIB
    LIB.parent.mkdir(exist_ok=True)
    cc = os.environ.get("CC") or shutil.which("gcc") or "cc"
    tmp = LIB.with_suffix(f".tmp{os.getpid()}")
    cmd = [cc, "-O3", "-fopenmp", "-fPIC", "-shared", "-std=c11", "-o", str(tmp), str(SRC), "-lm"]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"cpu_fab build failed:\n{res.stderr}")
    os.replace(tmp, LIB)
    return LIB


def load():
    global _lib
    if _lib is None:
        build()
        lib = ct.CDLL(str(LIB))
        dp, lp, ip = ct.POINTER(ct.c_double), ct.POINTER(ct.c_long), ct.POINTER(ct.c_int)
        lib.cpu_fab.argtypes = [ct.c_long, lp, ip, dp, ct.c_int, dp, ct.c_int, ct.c_int, dp, ct.c_int,
                                dp, dp, dp, dp, dp, ct.c_int]
        lib.cpu_fab.restype = ct.c_int
        lib.cpu_fab_max_threads.restype = ct.c_int
        _lib = lib
    return _lib


def max_threads() -> int:
    return load().cpu_fab_max_threads()


def run(A, U_deflated, m, gamma, gs_re, gs_im, wts, sigma, threads: int = 0) -> np.ndarray:
    """sum_j Im(q_j(A) V y_j) for each (deflated) column of U, by the reference
    CPU algorithm (nicksmethodcpu.m).  Returns (n, R)."""
    lib = load()
    A = sp.csr_matrix(A)
    n = A.shape[0]
    rp = np.ascontiguousarray(A.indptr, dtype=np.int64)
    ci = np.ascontiguousarray(A.indices, dtype=np.int32)
    va = np.ascontiguousarray(A.data, dtype=np.float64)
    U = np.asfortranarray(np.asarray(U_deflated, dtype=np.float64).reshape(n, -1))
    R = U.shape[1]
    gamma = np.ascontiguousarray(gamma, dtype=np.float64)
    gr = np.asfortranarray(np.asarray(gs_re, dtype=np.float64))
    gi = np.asfortranarray(np.asarray(gs_im, dtype=np.float64))
    C = gr.shape[1]
    w = np.concatenate([np.asarray(x, dtype=np.float64).reshape(C, 2).T.reshape(-1) for x in wts])
    sg = np.empty(2 * C)
    sg[0::2] = np.real(sigma)
    sg[1::2] = np.imag(sigma)
    out = np.zeros((n, R), order="F")
    dp = ct.POINTER(ct.c_double)
    rc = lib.cpu_fab(n, rp.ctypes.data_as(ct.POINTER(ct.c_long)), ci.ctypes.data_as(ct.POINTER(ct.c_int)),
                     va.ctypes.data_as(dp), R, U.ctypes.data_as(dp), int(m), gamma.size, gamma.ctypes.data_as(dp),
                     C, gr.ctypes.data_as(dp), gi.ctypes.data_as(dp), w.ctypes.data_as(dp), sg.ctypes.data_as(dp),
                     out.ctypes.data_as(dp), int(threads))
    if rc != 0:
        raise MemoryError("cpu_fab: allocation failed")
    return np.ascontiguousarray(out)
