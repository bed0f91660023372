"""CPU checks of the adjoint's host side and of its oracles.

The entry lists of A(kappa) must assemble exactly the operator of
problems.fe_operator. The dense Daleckii-Krein gradient is pinned by central
finite differences of the dense loss. The contour gradient with exact solves
must agree with the dense one to the quadrature error.
"""
import numpy as np
import pytest

from gpumatfun_gb300 import adjoint, params, problems
from oracle import adjoint as oadj


def _setup(nt=400, seed=3, sg=0.5):
    mesh = problems.disk_mesh(nt, seed=seed)
    cent = mesh.nodes[mesh.tris].mean(axis=1)
    kappa = np.exp(problems.gaussian_random_field(cent, sigma=sg, ell=0.2, seed=seed + 1))
    return mesh, kappa


def test_structure_assembles_fe_operator():
    mesh, kappa = _setup()
    st = adjoint.fe_structure(mesh)
    A_ref, ms, inner = problems.fe_operator(mesh, kappa)
    A = st.matrix(kappa)
    assert A.shape == A_ref.shape
    np.testing.assert_array_equal(A.indptr, A_ref.indptr)
    np.testing.assert_array_equal(A.indices, A_ref.indices)
    np.testing.assert_allclose(A.data, A_ref.data, rtol=1e-13, atol=1e-13 * abs(A_ref.data).max())
    np.testing.assert_array_equal(st.inner, inner)
    np.testing.assert_allclose(st.msqrt, ms, rtol=1e-15)
    # every contribution of a triangle to the entry lists is one of its 9 local pairs
    assert st.ent_ptr[-1] == st.ent_tri.size
    assert np.all(np.diff(st.ent_ptr) >= 1)
    # boundary vertices carry -1
    assert st.tri_nodes.min() == -1 and st.tri_nodes.max() == st.n - 1


def _loss_dense(mesh, kappa, b, d, f):
    A, *_ = oadj.fe_parts(mesh, kappa)
    lam, Q = np.linalg.eigh(A.toarray())
    x = Q @ (f(lam) * (Q.T @ b))
    return 0.5 * float((x - d) @ (x - d))


def test_dense_gradient_matches_finite_differences():
    mesh, kappa = _setup(nt=150)
    alpha = 1.6
    f = params.frac_power(-alpha / 2)
    fp = lambda x: (-alpha / 2) * np.power(x, -alpha / 2 - 1)
    rng = np.random.default_rng(0)
    n = int((~mesh.boundary).sum())
    b = rng.random(n)
    d = rng.random(n) * 0.01
    L, x, dk, db = oadj.dense_grad(mesh, kappa, b, d, f, fp)
    for _ in range(4):
        v = kappa * rng.standard_normal(kappa.size)
        h = 1e-6
        fd = (_loss_dense(mesh, kappa + h * v, b, d, f) - _loss_dense(mesh, kappa - h * v, b, d, f)) / (2 * h)
        assert abs(fd - dk @ v) <= 1e-6 * abs(fd) + 1e-12
        u = rng.standard_normal(n)
        fdb = (_loss_dense(mesh, kappa, b + h * u, d, f) - _loss_dense(mesh, kappa, b - h * u, d, f)) / (2 * h)
        assert abs(fdb - db @ u) <= 1e-6 * abs(fdb) + 1e-12


def test_contour_gradient_matches_dense():
    mesh, kappa = _setup(nt=300)
    alpha = 1.6
    f = params.frac_power(-alpha / 2)
    fp = lambda x: (-alpha / 2) * np.power(x, -alpha / 2 - 1)
    A, *_ = oadj.fe_parts(mesh, kappa)
    lam = np.linalg.eigvalsh(A.toarray())
    con = params.hht_contour(lam[0] / 2, lam[-1] * 2, 32)
    w = con.weights(f)
    rng = np.random.default_rng(1)
    b = rng.random(A.shape[0])
    d = rng.random(A.shape[0]) * 0.01
    L0, x0, dk0, _ = oadj.dense_grad(mesh, kappa, b, d, f, fp)
    L1, x1, dk1 = oadj.contour_grad(mesh, kappa, b, d, con.xi, w)
    assert np.linalg.norm(x1 - x0) <= 1e-8 * np.linalg.norm(x0)
    assert np.linalg.norm(dk1 - dk0) <= 1e-7 * np.linalg.norm(dk0)


@pytest.mark.parametrize("degree,m", [(0, 80), (4, 40)])
def test_krylov_gradient_formula_matches_dense(degree, m):
    """The formula the GPU gradient follows (Krylov lifts, shifted polynomial
    by Horner) reproduces the dense gradient once Lanczos has converged."""
    from oracle import fab
    mesh, kappa = _setup(nt=300, sg=0.5)
    alpha = 1.6
    f = params.frac_power(-alpha / 2)
    fp = lambda x: (-alpha / 2) * np.power(x, -alpha / 2 - 1)
    A, *_ = oadj.fe_parts(mesh, kappa)
    lam = np.linalg.eigvalsh(A.toarray())
    con = params.hht_contour(lam[0] / 2, lam[-1] * 2, 32)
    gamma = params.polynomial_coeffs(degree, lam[-1] * 2 / 4)
    gs, sigma = params.shifted_poly_coeffs(gamma, con.xi)
    wm = con.weights_mat(f)
    rng = np.random.default_rng(5)
    b = rng.random(A.shape[0])
    d = rng.random(A.shape[0]) * 0.01
    L0, x0, dk0, db0 = oadj.dense_grad(mesh, kappa, b, d, f, fp)
    g = x0 - d
    o = fab.OracleEngine(A=A, U0=np.stack([b, g], axis=1), Q=None, m=m, gamma=gamma, gs_re=gs.real,
                         gs_im=gs.imag, flam=np.zeros((0, 2)), wts=[wm, wm],
                         shifts=params.shifts_vector(sigma, m, 2), col_scale=np.ones(2))
    o.build_subspace(); o.lin_sys_solves(); o.apply_V()
    dk = oadj.krylov_grad(mesh, kappa, o.V, o.Yr, o.Yi, gs, con.weights(f))
    assert np.linalg.norm(o.get_xsol()[:, 1] - db0) <= 1e-7 * np.linalg.norm(db0)
    assert np.linalg.norm(dk - dk0) <= 1e-6 * np.linalg.norm(dk0)


def test_submesh_cut_is_a_closed_dirichlet_mesh():
    """problems.submesh: kept triangles all inside the radius, every edge of
    the cut that only one kept triangle has is on the Dirichlet boundary, and
    the restricted operator is SPD."""
    mesh = problems.disk_mesh(20000, seed=3)
    sub, keep = problems.submesh(mesh, center=(0.2, -0.1), radius=0.3)
    cent = np.array([0.2, -0.1])
    assert np.all(np.hypot(*(mesh.nodes[mesh.tris[keep]] - cent).transpose(2, 0, 1)) < 0.3)
    np.testing.assert_array_equal(sub.nodes[sub.tris], mesh.nodes[mesh.tris[keep]])
    e = np.sort(np.concatenate([sub.tris[:, [0, 1]], sub.tris[:, [1, 2]], sub.tris[:, [2, 0]]]), axis=1)
    uniq, cnt = np.unique(e, axis=0, return_counts=True)
    assert np.all(sub.boundary[uniq[cnt == 1].ravel()])
    assert cnt.max() == 2
    A, *_ = problems.fe_operator(sub, np.ones(sub.tris.shape[0]))
    assert A.shape[0] == int((~sub.boundary).sum()) > 1000
    assert np.linalg.eigvalsh(A.toarray()).min() > 0
