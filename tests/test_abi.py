"""C ABI: the library loads and exports every symbol of include/gpumatfun.h;
argument checks that run before any device call (no GPU needed)."""
import ctypes as ct
import os
import re

import numpy as np

from gpumatfun_gb300 import engine as E

HDR = os.path.join(os.path.dirname(os.path.dirname(__file__)), "include", "gpumatfun.h")


def header_functions():
    txt = open(HDR).read()
    return sorted(set(re.findall(r"^\s*(?:const\s+)?\w+\**\s+\**(gm_\w+)\s*\(", txt, re.M)))


def test_exports_every_header_symbol(engine_lib):
    names = header_functions()
    assert len(names) >= 20
    for nm in names:
        assert hasattr(engine_lib, nm), nm
    assert sorted(E.EXPORTED_SYMBOLS) == names
    assert b"sm_103a" in engine_lib.gm_version()


def test_struct_layout_matches_header(engine_lib):
    a = E.CreateArgs()
    engine_lib.gm_default_args(ct.byref(a))
    assert a.struct_version == 1 and a.nrhs == 2 and a.sync_mode == 1 and a.format == 0
    assert a.vamp == 1.0 and a.dt == 1.0


def _args(**over):
    a = E.CreateArgs()
    E.load_library().gm_default_args(ct.byref(a))
    for k, v in over.items():
        setattr(a, k, v)
    return a


def test_create_rejects_bad_arguments_before_device(engine_lib):
    h = ct.c_void_p()
    ptr = np.array([0, 1], dtype=np.int64)
    ind = np.array([0], dtype=np.int64)
    val = np.array([2.0])
    U = np.ones(1)
    g = np.ones(1)
    base = dict(n=1, ptr=ptr.ctypes.data_as(E._lp), ind=ind.ctypes.data_as(E._lp),
                values=val.ctypes.data_as(E._dp), U=U.ctypes.data_as(E._dp), nrhs=1,
                subspace_size=1, gamma_size=1, gamma=g.ctypes.data_as(E._dp), contour_size=1,
                gamma_s_real=g.ctypes.data_as(E._dp), gamma_s_imag=g.ctypes.data_as(E._dp),
                wts=g.ctypes.data_as(E._dp), shifts=g.ctypes.data_as(E._dp))
    cases = [(dict(nrhs=3), "nrhs"), (dict(struct_version=7), "struct_version"), (dict(n=0), "inputNotSquare"),
             (dict(subspace_size=0), "bad_N"), (dict(gamma_size=0), "bad_gamma"), (dict(precision=5), "precision"),
             (dict(num_eigs=2), "badQ"), (dict(format=9), "format"), (dict(reorth=3), "reorth"),
             (dict(reorth=-1), "reorth")]
    for over, msg in cases:
        kw = dict(base)
        kw.update(over)
        rc = engine_lib.gm_lanczos_create(ct.byref(_args(**kw)), ct.byref(h))
        assert rc == 1, (over, rc)
        assert msg in engine_lib.gm_last_error(None).decode(), engine_lib.gm_last_error(None)
        assert not h.value
    assert engine_lib.gm_lanczos_create(None, ct.byref(h)) == 1


def test_deflation_pairs_argument_checks(engine_lib):
    """gm_deflation_pairs rejects bad sizes before any device work."""
    rp = np.zeros(2, dtype=np.int64)
    ci = np.zeros(1, dtype=np.int32)
    va = np.zeros(1)
    out = np.zeros(4)
    f = engine_lib.gm_deflation_pairs
    f.argtypes = [ct.c_int64, ct.c_void_p, ct.c_void_p, ct.c_void_p, ct.c_int, ct.c_double, ct.c_int, ct.c_int,
                  ct.c_uint64, ct.c_void_p, ct.c_void_p, ct.c_void_p]
    for n, k, tol in ((10, 2, 1e-8), (1000, 0, 1e-8), (1000, 25, 1e-8), (1000, 4, 0.0)):
        rc = f(n, rp.ctypes.data, ci.ctypes.data, va.ctypes.data, k, tol, 100, 10, 0, out.ctypes.data,
               out.ctypes.data, None)
        assert rc == 1, (n, k, tol)
        assert b"deflation_pairs" in engine_lib.gm_last_error(None)
