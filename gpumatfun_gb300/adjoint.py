"""Adjoint of x = f(A(kappa)) b for the P1 finite-element fractional operator.

The operator is the nonuniform-diffusion one of problem_startup_nonuniform.m
and process_nonuniform.m:90-91:
- A(kappa) = M^{-1/2} K(kappa) M^{-1/2} on the interior nodes of a P1
  triangle mesh (homogeneous Dirichlet boundary);
- K(kappa) = sum_e kappa_e K_e, with one diffusion coefficient per triangle;
- M is the lumped mass.

The reference treats A as a fixed input and has no derivative. This module
adds the gradient of a loss on f(A(kappa)) b with respect to b and kappa. It
reuses the engine's contour nodes and shifted solves through the Frechet form
of the resolvent:

    d f(A) b = Im sum_j w_j (xi_j - A)^{-1} dA (xi_j - A)^{-1} b.

The engine kernels behind it:
- ``gm_fe_assemble`` rebuilds A's stored values from kappa on the GPU. It
  gathers a fixed list of triangle contributions per stored entry, in a
  fixed order and without atomics, so the same kappa always gives the same
  bits.
- ``gm_fe_gradient`` takes a solve for U = [b, g] (g = dL/dx). It lifts the
  shifted solutions of both columns, applies the shifted polynomial, and
  reduces per triangle.

By default the operator's engine has one right-hand side, and it keeps the
forward solve's Krylov state: its basis and shifted solutions. A backward
call at the same κ and b then costs one more solve, for g.
`store_basis=False` recomputes that state instead: a two-column engine solves
[b, g] together. This needs one basis of memory instead of two and costs more
time.

``FracFEOperator`` owns one engine for one mesh. ``FracFESolve`` is the
``torch.autograd.Function`` over it. The functions act on CUDA float64
tensors and run on the caller's current stream.
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np
import scipy.sparse as sp

from . import params, problems
from .engine import Engine

__all__ = ["FEStructure", "fe_structure", "FracFEOperator", "FracFESolve", "frac_fe_solve"]


@dataclass
class FEStructure:
    """Sparsity and per-entry triangle contributions of A(kappa)."""
    n: int                   # interior nodes (rows of A)
    ntri: int
    indptr: np.ndarray       # CSR pattern of A (sorted columns)
    indices: np.ndarray
    ent_ptr: np.ndarray      # (nnz+1,) contributions of each stored entry
    ent_tri: np.ndarray      # triangle of each contribution (sorted within an entry)
    ent_coef: np.ndarray     # msi_a K_e[a][c] msi_c of each contribution
    tri_nodes: np.ndarray    # (ntri, 3) row of each vertex, -1 on the boundary
    tri_kc: np.ndarray       # (ntri, 9) msi_a K_e[a][c] msi_c
    inner: np.ndarray        # mesh node of each row
    msqrt: np.ndarray        # M^{1/2} per row

    def values(self, kappa: np.ndarray) -> np.ndarray:
        """Stored values of A(kappa) in CSR order (host, FP64)."""
        kappa = np.asarray(kappa, dtype=np.float64)
        contrib = kappa[self.ent_tri] * self.ent_coef
        out = np.zeros(self.indices.size)
        np.add.at(out, np.repeat(np.arange(self.indices.size), np.diff(self.ent_ptr)), contrib)
        return out

    def matrix(self, kappa: np.ndarray) -> sp.csr_matrix:
        return sp.csr_matrix((self.values(kappa), self.indices, self.indptr), shape=(self.n, self.n))


def fe_structure(mesh: problems.FEMesh) -> FEStructure:
    """Entry lists of A(kappa) for ``mesh`` (problems.fe_operator's operator)."""
    nodes, tris = mesh.nodes, np.asarray(mesh.tris, dtype=np.int64)
    nt = tris.shape[0]
    area, G = problems.p1_element_grads(nodes, tris)
    K1 = np.einsum("tid,tjd->tij", G, G) * area[:, None, None]
    nn = nodes.shape[0]
    M = np.bincount(tris.ravel(), weights=np.repeat(area / 3.0, 3), minlength=nn)
    inner = np.flatnonzero(~mesh.boundary)
    idx = np.full(nn, -1, dtype=np.int64)
    idx[inner] = np.arange(inner.size)
    ms = np.sqrt(M[inner])
    msi = np.zeros(nn)
    msi[inner] = 1.0 / ms
    kc = K1 * msi[tris][:, :, None] * msi[tris][:, None, :]
    rows = np.broadcast_to(idx[tris][:, :, None], (nt, 3, 3))
    cols = np.broadcast_to(idx[tris][:, None, :], (nt, 3, 3))
    tid = np.broadcast_to(np.arange(nt)[:, None, None], (nt, 3, 3))
    ok = (rows >= 0) & (cols >= 0)
    r, c, t, coef = rows[ok], cols[ok], tid[ok], kc[ok]
    order = np.lexsort((t, c, r))
    r, c, t, coef = r[order], c[order], t[order], coef[order]
    n = inner.size
    key = r * n + c
    first = np.concatenate([[True], key[1:] != key[:-1]])
    starts = np.flatnonzero(first)
    ent_ptr = np.concatenate([starts, [key.size]]).astype(np.int64)
    er, ec = r[starts], c[starts]
    indptr = np.concatenate([[0], np.cumsum(np.bincount(er, minlength=n))]).astype(np.int64)
    return FEStructure(n=n, ntri=nt, indptr=indptr, indices=ec.astype(np.int64), ent_ptr=ent_ptr,
                       ent_tri=t.astype(np.int32), ent_coef=np.ascontiguousarray(coef),
                       tri_nodes=np.ascontiguousarray(idx[tris]), tri_kc=np.ascontiguousarray(kc.reshape(nt, 9)),
                       inner=inner, msqrt=ms)


class FracFEOperator:
    """x = f(A(kappa)) b with f(x) = x^(-alpha/2), and its adjoint, on one mesh.

    The contour (C nodes on [l1, lN]) and the polynomial preconditioner
    (degree ``degree`` on [0, lN]) are fixed at construction, so every kappa
    evaluates the same approximation of f.  ``matrix_powers`` runs two Horner
    levels of the degree-``degree`` polynomial per SpMV pass (bit-identical
    results; a few percent faster on meshes of a few 100k nodes). [l1, lN] must enclose the
    spectrum of every A(kappa) used. By default it is the spectrum of
    A(kappa0), widened by ``margin``.
    """

    def __init__(self, mesh: problems.FEMesh, kappa0: np.ndarray, alpha: float = 1.6, m: int = 150,
                 C: int = 32, degree: int = 16, l1: float | None = None, lN: float | None = None,
                 margin: float = 2.0, precision: str = "fp64", store_basis: bool = True,
                 matrix_powers: int = 1, **engine_kw):
        self.st = fe_structure(mesh)
        self.alpha = float(alpha)
        self.f = params.frac_power(-alpha / 2)
        A0 = self.st.matrix(kappa0)
        if l1 is None or lN is None:
            import scipy.sparse.linalg as sla
            hi = float(sla.eigsh(A0, k=1, which="LA", return_eigenvectors=False, tol=1e-6)[0])
            lo = float(sla.eigsh(A0, k=1, sigma=0.0, which="LM", return_eigenvectors=False)[0])
            l1 = lo / margin if l1 is None else l1
            lN = hi * margin if lN is None else lN
        self.l1, self.lN = float(l1), float(lN)
        self.contour = params.hht_contour(self.l1, self.lN, C)
        self.gamma = params.polynomial_coeffs(degree, self.lN / 4.0)
        gs, sigma = params.shifted_poly_coeffs(self.gamma, self.contour.xi)
        w = self.contour.weights_mat(self.f)
        self.m, self.C, self.degree = int(m), int(C), int(degree)
        n = self.st.n
        R = 1 if store_basis else 2
        self.store_basis = bool(store_basis)
        self.engine = Engine(A0, np.zeros((n, R)), None, None, None, m, self.gamma, gs.real, gs.imag, [w] * R,
                             params.shifts_vector(sigma, m, R), col_scale=np.ones(R), precision=precision,
                             sync=False, keep_entry_map=True, row_weight=self.st.msqrt,
                             matrix_powers=matrix_powers, **engine_kw)
        self._fwd_key = None
        st = self.st
        self.engine.fe_attach(st.ntri, st.ent_ptr, st.ent_tri, st.ent_coef, st.tri_nodes, st.tri_kc)
        self.n, self.ntri = n, st.ntri
        self._stream = None

    def _on_current_stream(self):
        """Launch on the caller's current stream, so that the engine's kernels
        are ordered with the torch kernels that make and consume its tensors
        (the legacy default stream is handle 0 in torch)."""
        import torch
        s = torch.cuda.current_stream().cuda_stream
        if s != self._stream:
            self.engine.set_stream(s)
            self._stream = s

    def forward(self, kappa, b):
        """f(A(kappa)) b (CUDA float64 tensors) through gm_fe_forward."""
        import torch
        self._on_current_stream()
        kappa = kappa.detach().to(torch.float64).contiguous()
        b = b.detach().to(torch.float64).contiguous()
        x = torch.empty_like(b)
        self.engine.fe_forward(kappa.data_ptr(), b.data_ptr(), x.data_ptr())
        self._fwd_key = self._key(kappa, b) if self.store_basis else None
        return x

    @staticmethod
    def _key(kappa, b):
        return (kappa.data_ptr(), kappa._version, tuple(kappa.shape), b.data_ptr(), b._version, tuple(b.shape))

    def backward(self, kappa, b, gx):
        """(dL/dkappa, dL/db) for dL/dx = gx through gm_fe_backward."""
        import torch
        self._on_current_stream()
        kappa = kappa.detach().to(torch.float64).contiguous()
        b = b.detach().to(torch.float64).contiguous()
        gx = gx.detach().to(torch.float64).contiguous()
        dk = torch.empty(self.ntri, dtype=torch.float64, device=b.device)
        db = torch.empty_like(b)
        if self._fwd_key is not None and self._fwd_key == self._key(kappa, b):
            self.engine.fe_backward_stored(gx.data_ptr(), dk.data_ptr(), db.data_ptr())
        else:
            self.engine.fe_backward(kappa.data_ptr(), b.data_ptr(), gx.data_ptr(), dk.data_ptr(), db.data_ptr())
            self._fwd_key = self._key(kappa, b) if self.store_basis else None
        return dk, db

    def delete(self):
        self.engine.delete()


class _FracFESolveFn:
    """Built lazily so that importing this module does not need torch."""
    cls = None


def _make_fn():
    import torch

    class FracFESolve(torch.autograd.Function):
        """x = f(A(kappa)) b; backward gives dL/dkappa (per triangle) and dL/db."""

        @staticmethod
        def forward(ctx, kappa, b, op):
            ctx.op = op
            ctx.save_for_backward(kappa, b)
            return op.forward(kappa, b)

        @staticmethod
        def backward(ctx, gx):
            kappa, b = ctx.saved_tensors
            if not (ctx.needs_input_grad[0] or ctx.needs_input_grad[1]):
                return None, None, None
            dk, db = ctx.op.backward(kappa, b, gx.contiguous())
            return (dk if ctx.needs_input_grad[0] else None, db if ctx.needs_input_grad[1] else None, None)

    return FracFESolve


def __getattr__(name):
    if name == "FracFESolve":
        if _FracFESolveFn.cls is None:
            _FracFESolveFn.cls = _make_fn()
        return _FracFESolveFn.cls
    raise AttributeError(name)


def frac_fe_solve(kappa, b, op: FracFEOperator):
    """Differentiable x = f(A(kappa)) b through ``op``."""
    return __getattr__("FracFESolve").apply(kappa, b, op)
