"""MATLAB .mat mesh ingest (the layout of the reference's circle*.mat files),
checked on a mesh written here, so no reference file is needed at run time."""
import numpy as np
import pytest
import scipy.io as sio
import scipy.sparse as sp

from gpumatfun_gb300 import problems


def write_mesh(path, n_target=300, seed=3):
    mesh = problems.disk_mesh(n_target, seed=seed)
    kappa = np.ones(mesh.tris.shape[0])
    K, M = problems.p1_assemble(mesh, kappa)
    inner = np.flatnonzero(~mesh.boundary)
    sio.savemat(path, {"K": sp.csc_matrix(K), "M": sp.csc_matrix(sp.diags(M)), "nodes": mesh.nodes,
                       "elements": (mesh.tris + 1).astype(np.float64),
                       "internal_nodes": (inner + 1)[None, :].astype(np.float64)})
    return mesh, kappa


def test_load_fe_mat_matches_operator(tmp_path):
    path = str(tmp_path / "mesh.mat")
    mesh, kappa = write_mesh(path)
    fx = problems.load_fe_mat(path)
    A, ms, inner = problems.fe_operator(mesh, kappa)
    np.testing.assert_array_equal(fx.kept, inner)
    assert abs(fx.A - A).max() < 1e-12 * abs(A).max()
    np.testing.assert_allclose(fx.msqrt, ms, rtol=1e-15)
    np.testing.assert_array_equal(fx.elements, mesh.tris)
    # SPD after the Dirichlet restriction
    assert np.linalg.eigvalsh(fx.A.toarray()).min() > 0


def test_load_fe_mat_neumann_keeps_all_nodes(tmp_path):
    path = str(tmp_path / "mesh.mat")
    mesh, _ = write_mesh(path)
    fx = problems.load_fe_mat(path, dirichlet=False)
    assert fx.A.shape[0] == mesh.nodes.shape[0]
    # K's rows sum to zero (constant null vector), so A (M^{1/2} 1) = 0
    assert np.abs(fx.A @ fx.msqrt).max() < 1e-10 * abs(fx.A).max()


def test_load_fe_mat_missing_variable(tmp_path):
    path = str(tmp_path / "bad.mat")
    sio.savemat(path, {"K": sp.csc_matrix(np.eye(3))})
    with pytest.raises(ValueError, match="no variable"):
        problems.load_fe_mat(path)
