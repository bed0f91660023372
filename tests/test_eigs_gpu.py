"""GPU deflation pairs (gm_deflation_pairs) against known eigenpairs.

The reference computes its deflation vectors with eigs(K, M, k, 'sm')
(process_nonuniform.m:38-40, 106-110).  Checks:
- the 2D Dirichlet Laplacian, whose eigenpairs are known in closed form and
  come in equal pairs (lambda_ij = lambda_ji): eigenvalues to 1e-10 relative,
  the invariant subspace to the analytic one;
- an FE disk operator against host shift-invert eigsh;
- the 1M-node FE disk of the f(A)b workload against its eigsh pairs:
  eigenvalues to 1e-8 relative, every relative residual below 1e-6, and the
  same invariant subspace;
- the engine fed with the GPU pairs gives the same f(A)b as with eigsh's.
"""
import numpy as np
import pytest
import scipy.sparse as sp
import scipy.sparse.linalg as sla

from gpumatfun_gb300 import Engine, eigs, problems, workloads
from gpumatfun_gb300.engine import GmError

pytestmark = pytest.mark.gpu


def subspace_cos_min(Qa, Qb):
    """Smallest cosine of the principal angles between span(Qa) and span(Qb)."""
    return float(np.linalg.svd(Qa.T @ Qb, compute_uv=False).min())


def rel_residuals(A, lam, Q):
    return np.linalg.norm(A @ Q - Q * lam, axis=0) / np.abs(lam)


def test_fd_laplacian_with_double_eigenvalues(engine_lib):
    N = 60
    A = problems.laplacian_2d(N, "D", 1.0)
    lam_ref, Q_ref = problems.laplacian_2d_eigpairs(N, 40, "D", 1.0)
    o = np.argsort(lam_ref)
    lam_ref, Q_ref = lam_ref[o], Q_ref[:, o]
    k = 20
    assert lam_ref[k] - lam_ref[k - 1] > 1e-3 * lam_ref[k]     # the 20 lowest form an invariant subspace
    assert np.min(np.diff(lam_ref[:k])) < 1e-12                 # with equal pairs inside it
    lam, Q, st = eigs.deflation_pairs(A, k, tol=1e-9)
    assert st["converged"]
    np.testing.assert_allclose(lam, lam_ref[:k], rtol=1e-10)
    assert rel_residuals(A, lam, Q).max() <= 1e-9
    assert subspace_cos_min(Q_ref[:, :k], Q) > 1 - 1e-12
    np.testing.assert_allclose(Q.T @ Q, np.eye(k), atol=1e-12)


def test_fe_disk_against_eigsh(engine_lib):
    mesh = problems.disk_mesh(30000, seed=4)
    cent = mesh.nodes[mesh.tris].mean(axis=1)
    kappa = np.exp(problems.gaussian_random_field(cent, sigma=1.0, ell=0.1, seed=5))
    A, _, _ = problems.fe_operator(mesh, kappa)
    k = 12
    lu = sla.splu(sp.csc_matrix(A))
    op = sla.LinearOperator(A.shape, matvec=lu.solve, dtype=np.float64)
    lam_ref, Q_ref = sla.eigsh(A, k=k, sigma=0.0, which="LM", OPinv=op, tol=1e-12)
    o = np.argsort(lam_ref)
    lam_ref, Q_ref = lam_ref[o], Q_ref[:, o]
    for ff in (True, False):   # float-float filter until 1e-7, then FP64; or FP64 throughout
        lam, Q, st = eigs.deflation_pairs(A, k, float_float_filter=ff)
        assert (st["block_spmvs_float_float"] > 0) == ff
        np.testing.assert_allclose(lam, lam_ref, rtol=1e-10)
        assert rel_residuals(A, lam, Q).max() <= 1e-8
        assert subspace_cos_min(Q_ref, Q) > 1 - 1e-10


def test_fe_disk_1M_against_eigsh_and_in_the_engine(engine_lib):
    """The 1M-node FE disk (997,710 rows, k = 20): the GPU pairs against the
    workload's shift-invert eigsh pairs, then one f(A)b with each set."""
    P = workloads.cached_problem("fe-disk-1M", R=1)
    lam, Q, st = eigs.deflation_pairs(P.A, P.k)
    print(f"1M disk GPU deflation pairs: {st['iterations']:.0f} iterations, {st['block_spmvs']:.0f} block "
          f"SpMVs ({st['block_spmvs_float_float']:.0f} float-float), {st['device_s']:.2f} s, "
          f"max rel residual {st['max_rel_residual']:.2e}")
    assert st["converged"]
    err = np.max(np.abs(lam - P.lam) / P.lam)
    assert err <= 1e-8, err
    assert rel_residuals(P.A, lam, Q).max() <= 1e-6
    assert subspace_cos_min(P.Q, Q) > 1 - 1e-8
    # the engine with the GPU pairs: the same f(A)b as with eigsh's pairs
    P2 = workloads.make_problem(P.name, P.A, P.U, Q, lam, P.funcs, P.m, P.C, P.l1, P.lN, degree=P.d,
                                prob_dim=P.lN / 4, row_weight=P.row_weight)
    xs = []
    for prob in (P, P2):
        e = Engine.from_problem(prob, precision="fp64")
        e.solve()
        xs.append(e.get_solution())
        e.delete()
    assert np.linalg.norm(xs[1] - xs[0]) / np.linalg.norm(xs[0]) < 1e-10


def test_not_converged_and_argument_errors(engine_lib):
    A = problems.laplacian_2d(40, "D", 1.0)
    lam, Q, st = eigs.deflation_pairs(A, 10, max_iter=1, raise_on_noconv=False)
    assert not st["converged"] and st["iterations"] == 1
    with pytest.raises(GmError) as err:
        eigs.deflation_pairs(A, 10, max_iter=1)
    assert err.value.code == 9
    bad = A.copy()
    bad.data[3] = np.nan
    with pytest.raises(GmError) as err:
        eigs.deflation_pairs(bad, 4)
    assert err.value.code == 1
