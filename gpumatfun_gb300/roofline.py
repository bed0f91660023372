"""Algorithmic HBM traffic and arithmetic of the engine's kernels.

The counts are what the algorithm must move, not what the implementation
happens to move: every matrix entry (value + column index) is read once per
SpMV pass, every vector a pass reads or writes is counted once (perfect
reuse of gathered x entries), and padding of the SELL slices is excluded.
ncu's dram__bytes for the same launch, divided by these figures, shows how
close the kernels come to that ideal.

Units: n rows, nnz stored entries, R right-hand sides, m Krylov dimension,
d polynomial degree, C contour nodes, k deflation vectors.
"""
from __future__ import annotations

from dataclasses import dataclass


@dataclass
class Sizes:
    n: int
    nnz: int
    R: int
    m: int
    d: int
    C: int
    k: int
    mixed: bool = False
    reorth: int = 0     # Gram-Schmidt passes per Lanczos step (0, 1 or 2)

    @property
    def vb(self):   # matrix value bytes
        return 4 if self.mixed else 8

    @property
    def sb(self):   # Krylov basis / Lanczos work-vector element bytes
        return 4 if self.mixed else 8

    hb = 8          # Horner/lift element bytes (FP64 or float-float)


def spmv_matrix_bytes(s: Sizes) -> float:
    return s.nnz * (s.vb + 4) + 4.0 * (s.n + 1)


def lanczos_bytes(s: Sizes) -> float:
    """build_subspace: prologue + m steps of (d+1) SpMV passes and the
    alpha/beta update pass."""
    nR = float(s.n) * s.R
    M = spmv_matrix_bytes(s)
    tot = 8 * nR + s.sb * nR  # prologue: read U, write W
    for j in range(s.m):
        prev = s.sb * nR if j > 0 else 0.0
        if s.d == 0:
            tot += M + s.sb * nR + s.sb * nR + prev + s.sb * nR      # gather W, write V_j, read V_{j-1}, write W
        else:
            tot += M + s.sb * nR + s.sb * nR + s.hb * nR            # pass 1: gather W, write V_j, write H
            tot += (s.d - 1) * (M + s.hb * nR + s.sb * nR + s.hb * nR)  # Horner: gather H, read V_j, write H
            tot += M + s.hb * nR + s.sb * nR + prev + s.sb * nR    # final: gather H, V_j, V_{j-1}, write W
        tot += 3 * s.sb * nR                                        # pass B: read W, V_j, write W
        tot += reorth_step_bytes(s, j)
    return tot


def reorth_step_bytes(s: Sizes, j: int) -> float:
    """Gram-Schmidt of step j against V_0..V_j, s.reorth times: per pass the
    dots read w (in the Horner buffer) and V_0..V_j, and the correction reads
    w and V_0..V_j again and writes w (the last pass writes the work vector
    in storage precision instead)."""
    if s.reorth <= 0:
        return 0.0
    nR = float(s.n) * s.R
    per = 2 * (j + 1) * s.sb * nR + 2 * s.hb * nR + s.hb * nR
    return s.reorth * per + s.hb * nR   # + pass B writing w unrounded


def solve_bytes(s: Sizes) -> float:
    """lin_sys_solves: tridiagonals, shifts, weights in; Y and coefficients out."""
    sys = s.R * s.C
    return 8.0 * (2 * (s.m + 1) * s.R + 2 * s.m * sys + 2 * s.C * s.R + 2 * s.m * sys + 2 * (s.d + 1) * s.C) \
        + 8.0 * 2 * s.R * (s.d + 1) * s.m


def apply_bytes(s: Sizes) -> float:
    nR = float(s.n) * s.R
    tot = s.m * s.sb * nR                   # V read once
    if s.d > 0:
        tot += (s.d + 1) * s.hb * nR        # P written
        tot += s.d * (spmv_matrix_bytes(s) + 3 * s.hb * nR)  # Horner: gather, read P_h, write
    tot += 8 * nR * 3                       # read update, write X and S
    return tot


def deflate_bytes(s: Sizes) -> float:
    nR = float(s.n) * s.R
    return 2 * 8.0 * s.n * s.k + 8 * nR * 5


def fused_solve_bytes(s: Sizes) -> float:
    """One fused launch: build_subspace + lin_sys_solves + apply_V."""
    return lanczos_bytes(s) + solve_bytes(s) + apply_bytes(s)


def fused_solve_flops(s: Sizes) -> float:
    """Floating-point operations (an FMA counts 2) of one fused launch."""
    spmv = 2.0 * s.nnz * s.R
    per_step = (s.d + 1) * spmv + 2.0 * s.n * s.R * (2 + s.d + 3)
    apply = 2.0 * s.n * s.R * s.m * (s.d + 1) + s.d * spmv
    reorth = sum(s.reorth * 2 * 2.0 * s.n * s.R * (j + 1) for j in range(s.m))
    return s.m * per_step + apply + reorth
