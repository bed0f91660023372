"""Python host side of the f(A)b engine over its C ABI (include/gpumatfun.h).

``LanczosEngine`` mirrors the reference's MATLAB handle class
(lanczosEngine.m:1-56): the same constructor arguments in the same order and
the same methods (build_subspace, lin_sys_solves, apply_V, update_U,
update_U_monodomain, get_U, get_xsol, get_aabb, set_y).  ``Engine`` is the
generalised handle (any of 1/2/4 right-hand sides, precision choice, fused
solve).  Both call the CUDA library directly; there is no CPU fallback: a
missing library raises immediately.
"""
from __future__ import annotations

import ctypes as ct
from typing import Sequence

import numpy as np
import scipy.sparse as sp

from . import build as _build

__all__ = ["GmError", "Engine", "LanczosEngine", "load_library", "EXPORTED_SYMBOLS",
           "GM_FP64", "GM_MIXED"]

GM_FP64, GM_MIXED = 0, 1
GM_CSC, GM_CSR = 0, 1
_STATUS = {0: "GM_OK", 1: "GM_ERR_ARG", 2: "GM_ERR_OOM", 3: "GM_ERR_CUDA", 4: "GM_ERR_BREAKDOWN",
           5: "GM_ERR_TIMEOUT", 6: "GM_ERR_STATE", 7: "GM_ERR_NONFINITE", 8: "GM_ERR_UNSUPPORTED",
           9: "GM_ERR_NOCONV"}

EXPORTED_SYMBOLS = [
    "gm_default_args", "gm_lanczos_create", "gm_lanczos_delete", "gm_build_subspace",
    "gm_lin_sys_solves", "gm_apply_V", "gm_update_U", "gm_update_U_monodomain", "gm_get_U",
    "gm_get_xsol", "gm_get_aabb", "gm_set_y", "gm_get_y", "gm_set_U", "gm_set_U_device", "gm_get_update",
    "gm_get_solution", "gm_solve", "gm_solve_host", "gm_sync", "gm_set_stream",
    "gm_phase_times", "gm_info", "gm_info_ex", "gm_get_meff", "gm_last_error", "gm_version",
    "gm_lin_sys_solves_noalloc", "gm_batch_create", "gm_time_loop", "gm_fe_attach", "gm_fe_assemble",
    "gm_fe_gradient", "gm_get_solution_device", "gm_fe_forward", "gm_fe_backward",
    "gm_fe_backward_stored", "gm_get_basis", "gm_get_ode", "gm_set_state", "gm_deflation_pairs",
]

_dp = ct.POINTER(ct.c_double)
_lp = ct.POINTER(ct.c_int64)


class CreateArgs(ct.Structure):
    """ctypes mirror of gm_create_args (field order and types as in the header)."""
    _fields_ = [
        ("struct_version", ct.c_int),
        ("n", ct.c_int64), ("nnz", ct.c_int64), ("format", ct.c_int),
        ("ptr", _lp), ("ind", _lp), ("values", _dp),
        ("nrhs", ct.c_int), ("U", _dp),
        ("num_eigs", ct.c_int), ("Q", _dp), ("lambda_", _dp), ("flam", _dp),
        ("subspace_size", ct.c_int), ("gamma_size", ct.c_int), ("gamma", _dp),
        ("contour_size", ct.c_int), ("gamma_s_real", _dp), ("gamma_s_imag", _dp),
        ("wts", _dp), ("shifts", _dp),
        ("dt", ct.c_double), ("col_scale", _dp), ("mass", _dp), ("ode", _dp),
        ("aode", ct.c_double), ("bode", ct.c_double), ("code", ct.c_double),
        ("vrest", ct.c_double), ("vamp", ct.c_double), ("vth", ct.c_double),
        ("vpeak", ct.c_double), ("c1ion", ct.c_double), ("c2ion", ct.c_double),
        ("precision", ct.c_int), ("sync_mode", ct.c_int), ("threads_per_block", ct.c_int),
        ("blocks_per_sm", ct.c_int), ("sell_sigma", ct.c_int),
        ("barrier_timeout_s", ct.c_double), ("breakdown_tol", ct.c_double),
        ("sync_policy", ct.c_int), ("col_staging", ct.c_int), ("keep_entry_map", ct.c_int),
        ("l2_window", ct.c_int),
        ("row_weight", _dp), ("diag_compensation", ct.c_int),
        ("max_blocks", ct.c_int), ("matrix_powers", ct.c_int), ("reorth", ct.c_int),
        ("val_prefetch", ct.c_int),
    ]


class BatchProblem(ct.Structure):
    """ctypes mirror of gm_batch_problem."""
    _fields_ = [
        ("n", ct.c_int64), ("format", ct.c_int), ("ptr", _lp), ("ind", _lp), ("values", _dp),
        ("U", _dp), ("gamma", _dp), ("gamma_s_real", _dp), ("gamma_s_imag", _dp),
        ("wts", _dp), ("shifts", _dp),
    ]


_LIB = None


def load_library(build_if_missing: bool = False) -> ct.CDLL:
    """Load libgpumatfun.so from the package tree (raises if it is absent)."""
    global _LIB
    if _LIB is not None:
        return _LIB
    path = _build.LIB
    if not path.exists():
        if build_if_missing:
            _build.build()
        else:
            raise RuntimeError(f"engine library missing: {path} (run __graft_entry__.build())")
    lib = ct.CDLL(str(path))
    h = ct.c_void_p
    lib.gm_default_args.argtypes = [ct.POINTER(CreateArgs)]
    lib.gm_default_args.restype = None
    lib.gm_lanczos_create.argtypes = [ct.POINTER(CreateArgs), ct.POINTER(h)]
    lib.gm_batch_create.argtypes = [ct.c_int, ct.POINTER(BatchProblem), ct.POINTER(CreateArgs), ct.POINTER(h)]
    for name in ("gm_lanczos_delete", "gm_build_subspace", "gm_lin_sys_solves", "gm_apply_V",
                 "gm_update_U", "gm_update_U_monodomain", "gm_solve", "gm_sync"):
        getattr(lib, name).argtypes = [h]
    for name in ("gm_get_U", "gm_get_xsol", "gm_get_aabb", "gm_get_update", "gm_get_solution", "gm_get_basis"):
        getattr(lib, name).argtypes = [h, _dp]
    lib.gm_set_U.argtypes = [h, _dp]
    lib.gm_get_ode.argtypes = [h, _dp]
    lib.gm_set_state.argtypes = [h, _dp, _dp]
    lib.gm_set_U_device.argtypes = [h, ct.c_void_p]
    lib.gm_set_y.argtypes = [h, _dp, _dp]
    lib.gm_get_y.argtypes = [h, _dp, _dp]
    lib.gm_solve_host.argtypes = [h, _dp, _dp]
    lib.gm_set_stream.argtypes = [h, ct.c_void_p]
    lib.gm_time_loop.argtypes = [h, ct.c_int, ct.c_int, ct.c_int]
    lib.gm_fe_attach.argtypes = [h, ct.c_int64, ct.c_void_p, ct.c_void_p, ct.c_void_p, ct.c_void_p, ct.c_void_p]
    lib.gm_fe_assemble.argtypes = [h, ct.c_void_p]
    lib.gm_fe_gradient.argtypes = [h, ct.c_void_p]
    lib.gm_get_solution_device.argtypes = [h, ct.c_void_p]
    lib.gm_fe_forward.argtypes = [h, ct.c_void_p, ct.c_void_p, ct.c_void_p]
    lib.gm_fe_backward.argtypes = [h, ct.c_void_p, ct.c_void_p, ct.c_void_p, ct.c_void_p, ct.c_void_p]
    lib.gm_fe_backward_stored.argtypes = [h, ct.c_void_p, ct.c_void_p, ct.c_void_p]
    lib.gm_phase_times.argtypes = [h, ct.POINTER(ct.c_float)]
    lib.gm_info.argtypes = [h, _lp]
    lib.gm_info_ex.argtypes = [h, _lp, ct.c_int]
    lib.gm_get_meff.argtypes = [h, ct.POINTER(ct.c_int)]
    lib.gm_deflation_pairs.argtypes = [ct.c_int64, ct.c_void_p, ct.c_void_p, ct.c_void_p, ct.c_int, ct.c_double,
                                       ct.c_int, ct.c_int, ct.c_uint64, ct.c_void_p, ct.c_void_p, _dp]
    lib.gm_last_error.argtypes = [h]
    lib.gm_last_error.restype = ct.c_char_p
    lib.gm_version.restype = ct.c_char_p
    _LIB = lib
    return lib


STREAM_LEGACY = 1  # cudaStreamLegacy


class GmError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"{_STATUS.get(code, code)}: {msg}")
        self.code = code


def _f64(a) -> np.ndarray:
    return np.ascontiguousarray(np.asarray(a, dtype=np.float64))


def _ptr(a: np.ndarray | None, typ=_dp):
    return None if a is None else a.ctypes.data_as(typ)


class Engine:
    """Handle over the CUDA engine (one per problem, owns its device memory)."""

    def __init__(self, A, U, Q, lam, flam, m, gamma, gs_re, gs_im, wts: Sequence, shifts,
                 dt: float = 1.0, col_scale=None, mass=None, ode=None, fhn: dict | None = None,
                 precision: str | int = "fp64", sync: bool = True, threads: int = 0,
                 blocks_per_sm: int = 0, sell_sigma: int = 0, timeout_s: float = 0.0,
                 breakdown_tol: float = 0.0, matrix_format: str = "csr", sync_policy: int = 0,
                 col_staging: int = 0, keep_entry_map: bool = False, l2_window: int = 0,
                 row_weight=None, diag_compensation: int = 0, matrix_powers: int = 0, max_blocks: int = 0,
                 reorth: int = 0, val_prefetch: int = 0):
        self._lib = load_library()
        self._h = ct.c_void_p()
        n = A.shape[0]
        if A.shape[0] != A.shape[1]:
            raise GmError(1, "lanczos_create:inputNotSquare: Sparse matrix must be square.")
        if matrix_format == "csc":
            M = sp.csc_matrix(A)
            fmt = GM_CSC
        else:
            M = sp.csr_matrix(A)
            fmt = GM_CSR
        ptr = np.ascontiguousarray(M.indptr, dtype=np.int64)
        ind = np.ascontiguousarray(M.indices, dtype=np.int64)
        val = _f64(M.data)
        U = _f64(np.asarray(U).reshape(n, -1).T).reshape(-1)  # column-major n x R
        R = U.size // n
        Q = _f64(np.asarray(Q).reshape(n, -1).T).reshape(-1) if Q is not None and np.size(Q) else np.zeros(0)
        k = Q.size // n if n else 0
        flam = _f64(np.asarray(flam).reshape(k, R).T).reshape(-1) if k else np.zeros(0)
        lam = _f64(lam) if lam is not None and np.size(lam) else np.zeros(max(k, 1))
        gamma = _f64(gamma).reshape(-1)
        gs_re = _f64(np.asarray(gs_re).reshape(gamma.size, -1).T).reshape(-1)  # (d+1) x C col-major
        gs_im = _f64(np.asarray(gs_im).reshape(gamma.size, -1).T).reshape(-1)
        C = gs_re.size // gamma.size
        wts = _f64(np.concatenate([_f64(w).reshape(C, 2).T.reshape(-1) for w in wts]))
        shifts = _f64(shifts).reshape(-1)
        if wts.size != 2 * C * R:
            raise GmError(1, "lanczos_create:bad_wts1: one C x 2 weight block per right-hand side")
        if shifts.size != 2 * m * C * R:
            raise GmError(1, "lanczos_create:bad_shifts: Invalid shifts input argument c.")
        cs = _f64(col_scale) if col_scale is not None else None
        mass = _f64(mass) if mass is not None else None
        ode = _f64(ode) if ode is not None else None
        prec = {"fp64": GM_FP64, "mixed": GM_MIXED}.get(precision, precision)
        a = CreateArgs()
        self._lib.gm_default_args(ct.byref(a))
        a.n, a.nnz, a.format = n, int(ptr[-1]), fmt
        a.ptr, a.ind, a.values = _ptr(ptr, _lp), _ptr(ind, _lp), _ptr(val)
        a.nrhs, a.U = R, _ptr(U)
        a.num_eigs, a.Q, a.lambda_, a.flam = k, _ptr(Q) if k else None, _ptr(lam), _ptr(flam) if k else None
        a.subspace_size, a.gamma_size, a.gamma = int(m), gamma.size, _ptr(gamma)
        a.contour_size, a.gamma_s_real, a.gamma_s_imag = C, _ptr(gs_re), _ptr(gs_im)
        a.wts, a.shifts = _ptr(wts), _ptr(shifts)
        a.dt, a.col_scale, a.mass, a.ode = float(dt), _ptr(cs), _ptr(mass), _ptr(ode)
        f = dict(aode=0.0, bode=0.0, code=0.0, vrest=0.0, vamp=1.0, vth=0.0, vpeak=0.0, c1ion=0.0, c2ion=0.0)
        f.update(fhn or {})
        for key, v in f.items():
            setattr(a, key, float(v))
        a.precision, a.sync_mode = int(prec), 1 if sync else 0
        a.threads_per_block, a.blocks_per_sm, a.sell_sigma = threads, blocks_per_sm, sell_sigma
        a.barrier_timeout_s, a.breakdown_tol = timeout_s, breakdown_tol
        a.sync_policy = int(sync_policy)
        a.col_staging = int(col_staging)
        a.keep_entry_map = 1 if keep_entry_map else 0
        a.l2_window = int(l2_window)
        rw = _f64(row_weight) if row_weight is not None else None
        a.row_weight = _ptr(rw) if rw is not None else None
        a.diag_compensation = int(diag_compensation)
        a.matrix_powers = int(matrix_powers)
        a.max_blocks = int(max_blocks)
        a.reorth = int(reorth)
        a.val_prefetch = int(val_prefetch)
        self._keep = (ptr, ind, val, U, Q, lam, flam, gamma, gs_re, gs_im, wts, shifts, cs, mass, ode, rw)
        rc = self._lib.gm_lanczos_create(ct.byref(a), ct.byref(self._h))
        self._keep = None
        if rc != 0:
            raise GmError(rc, self._lib.gm_last_error(None).decode())
        self.n, self.R, self.m, self.C, self.k, self.d = n, R, int(m), C, k, gamma.size - 1
        self.precision = prec

    # -- helpers
    def _check(self, rc: int):
        if rc != 0:
            raise GmError(rc, self._lib.gm_last_error(self._h).decode())

    def _out(self, fn, shape=None) -> np.ndarray:
        out = np.empty(self.n * self.R)
        self._check(fn(self._h, _ptr(out)))
        return out.reshape(self.R, self.n).T.copy()

    @property
    def handle(self) -> int:
        return self._h.value

    # -- reference methods (lanczosEngine.m:12-55)
    def build_subspace(self):
        self._check(self._lib.gm_build_subspace(self._h))

    def lin_sys_solves(self):
        self._check(self._lib.gm_lin_sys_solves(self._h))

    def apply_V(self):
        self._check(self._lib.gm_apply_V(self._h))

    def update_U(self):
        self._check(self._lib.gm_update_U(self._h))

    def update_U_monodomain(self):
        self._check(self._lib.gm_update_U_monodomain(self._h))

    def get_U(self) -> np.ndarray:
        return self._out(self._lib.gm_get_U)

    def get_xsol(self) -> np.ndarray:
        return self._out(self._lib.gm_get_xsol)

    def get_aabb(self) -> np.ndarray:
        out = np.empty((self.m + 1) * 2 * self.R)
        self._check(self._lib.gm_get_aabb(self._h, _ptr(out)))
        return out.reshape(2 * self.R, self.m + 1).T.copy()

    def set_y(self, yreal, yimag):
        yr = _f64(np.asarray(yreal).reshape(self.m, -1).T).reshape(-1)
        yi = _f64(np.asarray(yimag).reshape(self.m, -1).T).reshape(-1)
        if yr.size != self.m * self.R * self.C or yi.size != yr.size:
            raise GmError(1, "set_y: Yreal/Yimag must be m x (nrhs*C)")
        self._check(self._lib.gm_set_y(self._h, _ptr(yr), _ptr(yi)))

    def get_y(self):
        cnt = self.m * self.R * self.C
        yr, yi = np.empty(cnt), np.empty(cnt)
        self._check(self._lib.gm_get_y(self._h, _ptr(yr), _ptr(yi)))
        return yr.reshape(-1, self.m).T.copy(), yi.reshape(-1, self.m).T.copy()

    # -- additions
    def get_basis(self) -> np.ndarray:
        """The Krylov basis of the last build, shape (nrhs, m, n), as FP64."""
        out = np.empty(self.R * self.m * self.n)
        self._check(self._lib.gm_get_basis(self._h, _ptr(out)))
        return out.reshape(self.R, self.m, self.n)

    def get_state(self):
        """Checkpoint of a time loop: (Usol as get_U returns it, ode)."""
        ode = np.empty(self.n)
        self._check(self._lib.gm_get_ode(self._h, _ptr(ode)))
        return self.get_U(), ode

    def set_state(self, U, ode=None):
        """Resume from get_state(): Usol without column scaling, and ode."""
        u = _f64(np.asarray(U).reshape(self.n, -1).T).reshape(-1)
        if u.size != self.n * self.R:
            raise GmError(1, "set_state: U must be n x nrhs")
        o = _f64(np.asarray(ode).reshape(-1)) if ode is not None else None
        if o is not None and o.size != self.n:
            raise GmError(1, "set_state: ode must have n entries")
        self._check(self._lib.gm_set_state(self._h, _ptr(u), _ptr(o) if o is not None else None))

    def set_U(self, U):
        u = _f64(np.asarray(U).reshape(self.n, -1).T).reshape(-1)
        if u.size != self.n * self.R:
            raise GmError(1, "set_U: U must be n x nrhs")
        self._check(self._lib.gm_set_U(self._h, _ptr(u)))

    def set_U_device(self, ptr: int):
        """New right-hand sides from a device pointer (column-major n x nrhs
        FP64 on this handle's device, e.g. ``tensor.data_ptr()``)."""
        self._check(self._lib.gm_set_U_device(self._h, ct.c_void_p(ptr)))

    def solve(self):
        """Fused build_subspace + lin_sys_solves + apply_V in one launch."""
        self._check(self._lib.gm_solve(self._h))

    def get_solution(self) -> np.ndarray:
        return self._out(self._lib.gm_get_solution)

    def get_solution_device(self, ptr: int):
        """Solution (column-major n x nrhs FP64) into device memory at ``ptr``."""
        self._check(self._lib.gm_get_solution_device(self._h, ct.c_void_p(ptr)))

    def fe_attach(self, ntri: int, ent_ptr, ent_tri, ent_coef, tri_nodes, tri_kc):
        """Finite-element structure of A(kappa) (engine created with
        keep_entry_map=True from a CSR matrix); see gm_fe_attach."""
        arrs = (np.ascontiguousarray(ent_ptr, dtype=np.int64), np.ascontiguousarray(ent_tri, dtype=np.int32),
                _f64(ent_coef), np.ascontiguousarray(tri_nodes, dtype=np.int64), _f64(tri_kc))
        self._check(self._lib.gm_fe_attach(self._h, int(ntri), *[a.ctypes.data_as(ct.c_void_p) for a in arrs]))

    def fe_assemble(self, kappa_ptr: int):
        """A <- A(kappa), kappa a device pointer to ntri doubles."""
        self._check(self._lib.gm_fe_assemble(self._h, ct.c_void_p(kappa_ptr)))

    def fe_gradient(self, dkappa_ptr: int):
        """dL/dkappa (device pointer, ntri doubles) after solving for U = [b, g]."""
        self._check(self._lib.gm_fe_gradient(self._h, ct.c_void_p(dkappa_ptr)))

    def fe_forward(self, kappa: int, b: int, x: int):
        """x = f(A(kappa)) b; arguments are pointers (host or device)."""
        self._check(self._lib.gm_fe_forward(self._h, ct.c_void_p(kappa), ct.c_void_p(b), ct.c_void_p(x)))

    def fe_backward(self, kappa: int, b: int, g: int, dkappa: int, db: int | None):
        """dL/dkappa and dL/db for dL/dx = g; arguments are pointers (host or device)."""
        self._check(self._lib.gm_fe_backward(self._h, ct.c_void_p(kappa), ct.c_void_p(b), ct.c_void_p(g),
                                             ct.c_void_p(dkappa), ct.c_void_p(db or 0)))

    def fe_backward_stored(self, g: int, dkappa: int, db: int | None):
        """Backward at the kappa and b of the last fe_forward (nrhs = 1 engine),
        reusing its stored Krylov state."""
        self._check(self._lib.gm_fe_backward_stored(self._h, ct.c_void_p(g), ct.c_void_p(dkappa),
                                                    ct.c_void_p(db or 0)))

    def get_update(self) -> np.ndarray:
        return self._out(self._lib.gm_get_update)

    def solve_host(self, b: np.ndarray, out: np.ndarray | None = None) -> np.ndarray:
        """f(A) b end to end: host b (n x R, column-major buffer) -> host x."""
        b = np.asarray(b, dtype=np.float64)
        bc = b if (b.flags.f_contiguous and b.ndim == 2) else np.asfortranarray(b.reshape(self.n, -1))
        if out is None:
            out = np.empty((self.n, self.R), order="F")
        self._check(self._lib.gm_solve_host(self._h, bc.ctypes.data_as(_dp), out.ctypes.data_as(_dp)))
        return out

    def time_loop(self, nsteps: int, monodomain: bool = False, graph: bool = True):
        """nsteps exponential-Euler steps (fused solve + update_U or
        update_U_monodomain), replayed from a cached CUDA graph by default."""
        self._check(self._lib.gm_time_loop(self._h, int(nsteps), 1 if monodomain else 0, 1 if graph else 0))

    def sync(self):
        self._check(self._lib.gm_sync(self._h))

    def set_stream(self, stream_ptr: int | None):
        """Launch on an external stream.  None restores the handle's own stream;
        0 (the legacy default stream, e.g. torch's default stream) is passed
        as CUDA's cudaStreamLegacy handle so that it is not taken for None."""
        if stream_ptr is None:
            handle = 0
        elif stream_ptr == 0:
            handle = STREAM_LEGACY
        else:
            handle = stream_ptr
        self._check(self._lib.gm_set_stream(self._h, ct.c_void_p(handle)))

    def phase_times(self) -> dict:
        ms = (ct.c_float * 5)()
        self._check(self._lib.gm_phase_times(self._h, ms))
        return dict(zip(("deflate", "build_subspace", "lin_sys_solves", "apply_V", "solve"), list(ms)))

    nprob = 1

    def info(self) -> dict:
        keys = ("n", "nrhs", "m", "d", "C", "k", "precision", "grid_blocks", "threads",
                "sell_padded", "device_bytes", "launches", "problems", "matrix_powers",
                "value_prefetch_bytes", "reorth", "l2_window_bytes", "col_stage_groups",
                "neighbour_waits")
        v = (ct.c_int64 * len(keys))()
        self._check(self._lib.gm_info_ex(self._h, v, len(keys)))
        return dict(zip(keys, list(v)))

    def meff(self) -> list:
        v = (ct.c_int * (self.R * self.nprob))()
        self._check(self._lib.gm_get_meff(self._h, v))
        return list(v)

    def delete(self):
        if getattr(self, "_h", None) and self._h.value:
            self._lib.gm_lanczos_delete(self._h)
            self._h = ct.c_void_p()

    close = delete

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.delete()

    def __del__(self):
        try:
            self.delete()
        except Exception:
            pass

    @classmethod
    def from_problem(cls, P, **kw) -> "Engine":
        """Engine for a ``workloads.FabProblem``."""
        kw.setdefault("row_weight", getattr(P, "row_weight", None))
        return cls(P.A, P.U, P.Q, P.lam, P.flam, P.m, P.gamma, P.gs_re, P.gs_im, P.wts, P.shifts,
                   col_scale=P.col_scale if P.col_scale is not None else np.ones(P.R), **kw)


class LanczosEngine(Engine):
    """Drop-in for the reference's MATLAB handle (lanczosEngine.m:8-10): the
    same 25 constructor arguments in the same order (valvec is implicit)."""

    def __init__(self, U, A, Q, lambda_, N, gamma, gamma_s_real, gamma_s_imag, exp_lambda,
                 phi_lambda, dt, ode, aode, bode, code, vrest, vamp, vth, vpeak, c1ion, c2ion,
                 mass, wts1, wts2, shifts, **kw):
        U = np.asarray(U, dtype=np.float64)
        if U.ndim != 2 or U.shape[1] != 2:
            raise GmError(1, "lanczos_create:badU: Invalid U input argument.")
        k = 0 if Q is None else np.asarray(Q).reshape(U.shape[0], -1).shape[1]
        if k and (np.size(exp_lambda) != k or np.size(phi_lambda) != k):
            raise GmError(1, "lanczos_create:bad_exp_lambda: Invalid exp_lambda input argument.")
        flam = np.stack([np.ravel(exp_lambda), np.ravel(phi_lambda)], axis=1) if k else np.zeros((0, 2))
        fhn = dict(aode=aode, bode=bode, code=code, vrest=vrest, vamp=vamp, vth=vth, vpeak=vpeak,
                   c1ion=c1ion, c2ion=c2ion)
        kw.setdefault("matrix_format", "csc")
        super().__init__(A, U, Q, lambda_, flam, int(N), gamma, gamma_s_real, gamma_s_imag,
                         [wts1, wts2], shifts, dt=dt, col_scale=None, mass=mass, ode=ode, fhn=fhn, **kw)


class BatchEngine(Engine):
    """Several independent problems (uneven sizes) in one engine: every launch
    runs all of them at once (gm_batch_create).  All problems share m, C, the
    polynomial degree and the number of right-hand sides; vectors are the
    problems' rows stacked in order."""

    def __init__(self, problems: Sequence, precision: str | int = "fp64", sync: bool = True,
                 threads: int = 0, blocks_per_sm: int = 0, sell_sigma: int = 0, timeout_s: float = 0.0,
                 sync_policy: int = 0, col_staging: int = 0, diag_compensation: int = 0, reorth: int = 0,
                 val_prefetch: int = 0):
        self._lib = load_library()
        self._h = ct.c_void_p()
        P0 = problems[0]
        R, m, C, d1 = P0.R, P0.m, P0.C, P0.gamma.size
        keep = []
        arr = (BatchProblem * len(problems))()
        for i, P in enumerate(problems):
            if P.R != R or P.m != m or P.C != C or P.gamma.size != d1 or P.k != 0:
                raise GmError(1, "batch_create: problems must share nrhs, m, C and degree, without deflation")
            M = sp.csr_matrix(P.A)
            ptr = np.ascontiguousarray(M.indptr, dtype=np.int64)
            ind = np.ascontiguousarray(M.indices, dtype=np.int64)
            val = _f64(M.data)
            U = _f64(np.asarray(P.U).reshape(P.n, -1).T).reshape(-1)
            gam = _f64(P.gamma)
            gsr = _f64(np.asarray(P.gs_re).T).reshape(-1)
            gsi = _f64(np.asarray(P.gs_im).T).reshape(-1)
            wts = _f64(np.concatenate([_f64(w).reshape(C, 2).T.reshape(-1) for w in P.wts]))
            sh = _f64(P.shifts)
            keep.extend([ptr, ind, val, U, gam, gsr, gsi, wts, sh])
            arr[i] = BatchProblem(P.n, GM_CSR, _ptr(ptr, _lp), _ptr(ind, _lp), _ptr(val), _ptr(U), _ptr(gam),
                                  _ptr(gsr), _ptr(gsi), _ptr(wts), _ptr(sh))
        a = CreateArgs()
        self._lib.gm_default_args(ct.byref(a))
        cs = np.ones(R)
        keep.append(cs)
        a.nrhs, a.subspace_size, a.gamma_size, a.contour_size = R, m, d1, C
        a.col_scale = _ptr(cs)
        a.precision = int({"fp64": GM_FP64, "mixed": GM_MIXED}.get(precision, precision))
        a.sync_mode = 1 if sync else 0
        a.threads_per_block, a.blocks_per_sm, a.sell_sigma = threads, blocks_per_sm, sell_sigma
        a.barrier_timeout_s, a.sync_policy, a.col_staging = timeout_s, int(sync_policy), int(col_staging)
        a.diag_compensation = int(diag_compensation)
        a.reorth = int(reorth)
        a.val_prefetch = int(val_prefetch)
        rc = self._lib.gm_batch_create(len(problems), arr, ct.byref(a), ct.byref(self._h))
        del keep
        if rc != 0:
            raise GmError(rc, self._lib.gm_last_error(None).decode())
        self.nprob = len(problems)
        self.sizes = [P.n for P in problems]
        self.row0 = np.concatenate([[0], np.cumsum(self.sizes)])
        self.n, self.R, self.m, self.C, self.k, self.d = int(self.row0[-1]), R, m, C, 0, d1 - 1
        self.precision = a.precision

    def split(self, X: np.ndarray) -> list:
        """Per-problem row blocks of a stacked (n_total, R) array."""
        return [X[self.row0[p]:self.row0[p + 1]] for p in range(self.nprob)]

    def get_aabb(self) -> np.ndarray:
        """(nprob, m+1, 2R): alpha columns then beta columns per problem."""
        out = np.empty((self.m + 1) * 2 * self.R * self.nprob)
        self._check(self._lib.gm_get_aabb(self._h, _ptr(out)))
        return out.reshape(self.nprob, 2 * self.R, self.m + 1).transpose(0, 2, 1).copy()

    def get_y(self):
        cnt = self.m * self.R * self.C * self.nprob
        yr, yi = np.empty(cnt), np.empty(cnt)
        self._check(self._lib.gm_get_y(self._h, _ptr(yr), _ptr(yi)))
        return yr.reshape(-1, self.m).T.copy(), yi.reshape(-1, self.m).T.copy()
