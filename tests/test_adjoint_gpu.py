"""Adjoint of x = f(A(kappa)) b on the GPU.

The checks are:
- GPU assembly of A(kappa) against the host assembly;
- the gradient against the same formula restated in FP64 on the oracle's
  Krylov state (kernel parity);
- the gradient against the dense Daleckii-Krein gradient (2k-node disk);
- central finite differences on 64 random directions (step 1e-6);
- the torch.autograd.Function path;
- the mixed-precision gradient against the FP64 one.
"""
import numpy as np
import pytest

from gpumatfun_gb300 import adjoint, params, problems
from gpumatfun_gb300.engine import Engine, GmError
from oracle import adjoint as oadj
from oracle import fab

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")

ALPHA = 1.6
M2K = 200   # Krylov dimension at which the 2k-node case has converged (degree-8 polynomial)


def rel(a, b):
    return float(np.linalg.norm(np.asarray(a) - np.asarray(b)) / np.linalg.norm(b))


def fprime(x):
    return (-ALPHA / 2) * np.power(x, -ALPHA / 2 - 1)


def make_case(nt, seed=0, sg=1.0):
    """Mesh, current kappa, b and data d from a ground-truth kappa* plus 1% noise."""
    mesh = problems.disk_mesh(nt, seed=seed)
    cent = mesh.nodes[mesh.tris].mean(axis=1)
    kstar = np.exp(problems.gaussian_random_field(cent, sigma=sg, ell=0.1, seed=seed + 1))
    kappa = np.exp(problems.gaussian_random_field(cent, sigma=sg, ell=0.1, seed=seed + 7))
    n = int((~mesh.boundary).sum())
    rng = np.random.default_rng(seed + 2)
    b = rng.random(n)
    b /= np.linalg.norm(b)
    A, *_ = oadj.fe_parts(mesh, kstar)
    lam, Q = np.linalg.eigh(A.toarray()) if n <= 4000 else (None, None)
    f = params.frac_power(-ALPHA / 2)
    if lam is not None:
        xs = Q @ (f(lam) * (Q.T @ b))
    else:
        xs = np.zeros(n)
    d = xs + 0.01 * np.linalg.norm(xs) / np.sqrt(n) * rng.standard_normal(n)
    return mesh, kappa, b, d


@pytest.fixture(scope="module")
def case2k():
    return make_case(2000)


@pytest.fixture(scope="module")
def op2k(engine_lib, case2k):
    mesh, kappa, b, d = case2k
    op = adjoint.FracFEOperator(mesh, kappa, alpha=ALPHA, m=M2K, C=32, degree=8, margin=1.25)
    yield op
    op.delete()


def cuda(a):
    return torch.as_tensor(np.asarray(a, dtype=np.float64), device="cuda")


def test_gpu_assembly_matches_host(op2k, case2k):
    mesh, kappa, b, d = case2k
    k2 = kappa * np.exp(0.3 * np.sin(np.arange(kappa.size)))
    x_gpu = op2k.forward(cuda(k2), cuda(b)).cpu().numpy()
    # an engine created from the host-assembled A(k2) with the same method parameters
    op_h = adjoint.FracFEOperator(mesh, k2, alpha=ALPHA, m=M2K, C=32, degree=8, l1=op2k.l1, lN=op2k.lN)
    U = np.zeros((b.size, op_h.engine.R))
    U[:, 0] = b
    op_h.engine.set_U(U)
    op_h.engine.solve()
    x_host = op_h.engine.get_solution()[:, 0]
    op_h.delete()
    assert rel(x_gpu, x_host) < 1e-13


@pytest.mark.parametrize("store_basis", [True, False])
def test_gradient_matches_krylov_restatement(engine_lib, store_basis):
    """Kernel parity: same Krylov state, same formula, FP64 on the host.
    store_basis: a one-column engine with two stored Krylov states (b, g);
    otherwise a two-column engine solving [b, g] together."""
    mesh, kappa, b, d = make_case(500, seed=4)
    op = adjoint.FracFEOperator(mesh, kappa, alpha=ALPHA, m=30, C=24, degree=3, store_basis=store_basis)
    x = op.forward(cuda(kappa), cuda(b)).cpu().numpy()
    g = x - d
    dk, db = op.backward(cuda(kappa), cuda(b), cuda(g))
    dk, db = dk.cpu().numpy(), db.cpu().numpy()
    A = op.st.matrix(kappa)
    gs, sigma = params.shifted_poly_coeffs(op.gamma, op.contour.xi)
    w = op.contour.weights(op.f)
    wm = op.contour.weights_mat(op.f)
    o = fab.OracleEngine(A=A, U0=np.stack([b, g], axis=1), Q=None, m=op.m, gamma=op.gamma, gs_re=gs.real,
                         gs_im=gs.imag, flam=np.zeros((0, 2)), wts=[wm, wm],
                         shifts=params.shifts_vector(sigma, op.m, 2), col_scale=np.ones(2))
    o.build_subspace()
    o.lin_sys_solves()
    o.apply_V()
    dk_o = oadj.krylov_grad(mesh, kappa, o.V, o.Yr, o.Yi, gs, w)
    assert rel(db, o.get_xsol()[:, 1]) < 1e-10
    assert rel(dk, dk_o) < 1e-10
    op.delete()


def test_gradient_matches_dense_oracle(op2k, case2k):
    mesh, kappa, b, d = case2k
    x = op2k.forward(cuda(kappa), cuda(b)).cpu().numpy()
    dk, db = op2k.backward(cuda(kappa), cuda(b), cuda(x - d))
    L, x_ref, dk_ref, db_ref = oadj.dense_grad(mesh, kappa, b, d, op2k.f, fprime)
    ex, edb, edk = rel(x, x_ref), rel(db.cpu().numpy(), db_ref), rel(dk.cpu().numpy(), dk_ref)
    print(f"vs dense oracle: x {ex:.2e} dL/db {edb:.2e} dL/dkappa {edk:.2e}")
    assert ex < 1e-9
    assert edb < 1e-9
    assert edk < 1e-7


def test_finite_differences_64_directions(op2k, case2k):
    mesh, kappa, b, d = case2k
    kt, bt, dt = cuda(kappa), cuda(b), cuda(d)

    def loss(k):
        x = op2k.forward(k, bt)
        return 0.5 * float(torch.sum((x - dt) ** 2))

    x = op2k.forward(kt, bt)
    dk, _ = op2k.backward(kt, bt, x - dt)
    gen = torch.Generator(device="cuda").manual_seed(11)
    h = 1e-6
    fds, ads = [], []
    for _ in range(64):
        v = kt * torch.randn(kt.shape, generator=gen, device="cuda", dtype=torch.float64)
        fds.append((loss(kt + h * v) - loss(kt - h * v)) / (2 * h))
        ads.append(float(torch.dot(dk, v)))
    fds, ads = np.array(fds), np.array(ads)
    # error of each direction relative to the typical directional derivative
    err = np.abs(fds - ads) / np.sqrt(np.mean(ads ** 2))
    print(f"FD 64 directions: max {err.max():.2e} median {np.median(err):.2e}")
    assert err.max() < 1e-6


def test_autograd_function(op2k, case2k):
    mesh, kappa, b, d = case2k
    kt = cuda(kappa).requires_grad_(True)
    bt = cuda(b).requires_grad_(True)
    x = adjoint.frac_fe_solve(kt, bt, op2k)
    loss = 0.5 * torch.sum((x - cuda(d)) ** 2)
    loss.backward()
    dk, db = op2k.backward(cuda(kappa), cuda(b), (x - cuda(d)).detach())
    assert torch.equal(kt.grad, dk)
    assert torch.equal(bt.grad, db)


def test_mixed_precision_gradient(engine_lib, case2k):
    mesh, kappa, b, d = case2k
    ops = [adjoint.FracFEOperator(mesh, kappa, alpha=ALPHA, m=M2K, C=32, degree=8, margin=1.25, precision=p)
           for p in ("fp64", "mixed")]
    grads = []
    for op in ops:
        x = op.forward(cuda(kappa), cuda(b))
        dk, db = op.backward(cuda(kappa), cuda(b), x - cuda(d))
        grads.append((dk.cpu().numpy(), db.cpu().numpy()))
        op.delete()
    eb, ek = rel(grads[1][1], grads[0][1]), rel(grads[1][0], grads[0][0])
    print(f"mixed vs FP64: dL/db {eb:.2e} dL/dkappa {ek:.2e}")
    assert eb < 1e-5
    assert ek < 1e-4


def test_errors(engine_lib, case2k):
    mesh, kappa, b, d = case2k
    st = adjoint.fe_structure(mesh)
    A = st.matrix(kappa)
    P = dict(m=10, gamma=[1.0], gs_re=np.ones((1, 8)), gs_im=np.zeros((1, 8)),
             wts=[np.ones((8, 2))] * 2, shifts=np.ones(2 * 10 * 8 * 2))
    eng = Engine(A, np.ones((A.shape[0], 2)), None, None, None, P["m"], P["gamma"], P["gs_re"], P["gs_im"],
                 P["wts"], P["shifts"], col_scale=np.ones(2))
    with pytest.raises(GmError):
        eng.fe_attach(st.ntri, st.ent_ptr, st.ent_tri, st.ent_coef, st.tri_nodes, st.tri_kc)
    eng.delete()
    eng = Engine(A, np.ones((A.shape[0], 2)), None, None, None, P["m"], P["gamma"], P["gs_re"], P["gs_im"],
                 P["wts"], P["shifts"], col_scale=np.ones(2), keep_entry_map=True)
    dk = torch.empty(st.ntri, dtype=torch.float64, device="cuda")
    with pytest.raises(GmError):
        eng.fe_gradient(dk.data_ptr())          # before attach
    bad = st.ent_tri.copy()
    bad[0] = st.ntri
    with pytest.raises(GmError):
        eng.fe_attach(st.ntri, st.ent_ptr, bad, st.ent_coef, st.tri_nodes, st.tri_kc)
    eng.fe_attach(st.ntri, st.ent_ptr, st.ent_tri, st.ent_coef, st.tri_nodes, st.tri_kc)
    with pytest.raises(GmError):
        eng.fe_gradient(dk.data_ptr())          # before a solve
    eng.delete()


def test_host_pointer_entries(op2k, case2k):
    """gm_fe_forward / gm_fe_backward (the MEX backward entry) with host
    buffers give the same bits as with device buffers."""
    mesh, kappa, b, d = case2k
    x_dev = op2k.forward(cuda(kappa), cuda(b))
    dk_dev, db_dev = op2k.backward(cuda(kappa), cuda(b), x_dev - cuda(d))
    torch.cuda.synchronize()
    eng = op2k.engine
    eng.set_stream(None)
    op2k._stream = None
    kh, bh = np.ascontiguousarray(kappa), np.ascontiguousarray(b)
    xh = np.empty_like(bh)
    eng.fe_forward(kh.ctypes.data, bh.ctypes.data, xh.ctypes.data)
    gh = xh - d
    dkh = np.empty(op2k.ntri)
    dbh = np.empty_like(bh)
    eng.fe_backward(kh.ctypes.data, bh.ctypes.data, gh.ctypes.data, dkh.ctypes.data, dbh.ctypes.data)
    np.testing.assert_array_equal(xh, x_dev.cpu().numpy())
    np.testing.assert_array_equal(dkh, dk_dev.cpu().numpy())
    np.testing.assert_array_equal(dbh, db_dev.cpu().numpy())


def test_stored_forward_state_is_reused(op2k, case2k):
    """backward at the forward's kappa and b reuses the stored Krylov state
    (one solve instead of two) and gives the same bits as recomputing it."""
    mesh, kappa, b, d = case2k
    kt, bt = cuda(kappa), cuda(b)
    x = op2k.forward(kt, bt)
    launches0 = op2k.engine.info()["launches"]
    dk1, db1 = op2k.backward(kt, bt, x - cuda(d))          # same tensors: stored state
    used_stored = op2k.engine.info()["launches"] - launches0
    dk2, db2 = op2k.backward(cuda(kappa), cuda(b), x - cuda(d))   # new tensors: recomputed
    used_full = op2k.engine.info()["launches"] - launches0 - used_stored
    assert used_stored < used_full
    assert torch.equal(dk1, dk2) and torch.equal(db1, db2)
    # a fresh forward on other inputs invalidates the stored state
    op2k.forward(cuda(kappa * 1.01), bt)
    with pytest.raises(GmError):
        op2k.engine.fe_assemble(cuda(kappa).data_ptr())
        op2k.engine.fe_backward_stored((x - cuda(d)).data_ptr(), dk1.data_ptr(), db1.data_ptr())
