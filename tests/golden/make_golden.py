"""Generate the golden fixtures in this directory.

Run with GPUMATFUN_REF set to a checkout of the GPUMatfun sources (it reads
the FE meshes circle1.mat / circle2.mat shipped there); the outputs are
committed so tests never need the reference at run time.

circle_fab.npz: for each mesh, the operator A = M^{-1/2} K M^{-1/2} restricted
to the mesh's internal nodes (homogeneous Dirichlet), a seeded b, its 4
smallest eigenpairs and the exact f(A) b by dense eigendecomposition for
f(x) = x^-0.8 and f(x) = exp(-0.01 x^0.75).

fd16_oracle.npz: outputs of the oracle (aabb, Yreal, Yimag, X, update) on the
16 x 16 Dirichlet Laplacian case of tests/test_engine_gpu.py, pinning the
oracle itself against drift.
"""
import os
import sys

import numpy as np
import scipy.linalg as sla

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
REF = os.environ.get("GPUMATFUN_REF")


def circle_case(name, seed):
    from gpumatfun_gb300.problems import load_fe_mat
    A = load_fe_mat(os.path.join(REF, name + ".mat")).A
    Ad = A.toarray()
    lam, Qf = sla.eigh(0.5 * (Ad + Ad.T))
    rng = np.random.default_rng(seed)
    b = rng.random(A.shape[0])
    b /= np.linalg.norm(b)
    f1 = lam ** -0.8
    f2 = np.exp(-0.01 * lam ** 0.75)
    x1 = Qf @ (f1 * (Qf.T @ b))
    x2 = Qf @ (f2 * (Qf.T @ b))
    return {f"{name}_indptr": A.indptr.astype(np.int64), f"{name}_indices": A.indices.astype(np.int64),
            f"{name}_data": A.data, f"{name}_b": b, f"{name}_lam": lam[:5], f"{name}_Q": Qf[:, :4],
            f"{name}_lmax": np.array(lam[-1]), f"{name}_x_pow": x1, f"{name}_x_exp": x2}


def main():
    if not REF or not os.path.isdir(REF):
        raise SystemExit("set GPUMATFUN_REF to a checkout of the GPUMatfun sources (for circle1.mat, circle2.mat)")
    out = {}
    out.update(circle_case("circle1", 11))
    out.update(circle_case("circle2", 12))
    np.savez_compressed(os.path.join(HERE, "circle_fab.npz"), **out)
    from gpumatfun_gb300 import workloads
    from oracle import fab
    P = workloads.config1_small(N=16, k=3, m=24, C=16, R=2, degree=2)
    eng = fab.OracleEngine(A=P.A, U0=P.U, Q=P.Q, m=P.m, gamma=P.gamma, gs_re=P.gs_re, gs_im=P.gs_im,
                           flam=P.flam, wts=P.wts, shifts=P.shifts, col_scale=np.ones(2))
    eng.solve()
    np.savez_compressed(os.path.join(HERE, "fd16_oracle.npz"), aabb=eng.aabb(), Yr=eng.Yr, Yi=eng.Yi,
                        X=eng.X, update=eng.update, U=P.U)
    print("wrote", sorted(out)[:4], "...")


if __name__ == "__main__":
    main()
