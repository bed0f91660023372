"""Edge cases of the GPU engine against the FP64 oracle:
- sizes that are not multiples of the 32-row SELL slice, down to n = 1;
- uneven rows (one dense row, empty off-diagonals);
- a CSC input with unsorted row indices;
- a batch whose problems include a zero right-hand side;
- the autotuner on the GPU.
"""
import numpy as np
import pytest
import scipy.sparse as sp

from gpumatfun_gb300 import BatchEngine, Engine, autotune, params, workloads
from oracle import fab

pytestmark = pytest.mark.gpu


def rel(a, b):
    return float(np.linalg.norm(np.asarray(a) - np.asarray(b)) / max(np.linalg.norm(b), 1e-300))


def spd(n, seed, density=0.2, dense_row=False, drop_diag=None):
    rng = np.random.default_rng(seed)
    B = sp.random(n, n, density=density, random_state=rng, format="csr")
    A = B @ B.T + sp.identity(n) * (0.5 + rng.random())
    if dense_row and n > 2:
        v = rng.random(n) * 0.01
        D = sp.lil_matrix((n, n))
        D[0, :] = v
        D[:, 0] = v[:, None]
        A = A + D.tocsr() + sp.identity(n) * 0.1
    A = sp.csr_matrix((A + A.T) / 2)
    A.sort_indices()
    return A


def problem(A, R=2, m=None, C=16, degree=0, seed=0, f=None):
    n = A.shape[0]
    lam = np.linalg.eigvalsh(A.toarray())
    m = m or min(n, 12)
    f = f or params.frac_power(-0.5)
    rng = np.random.default_rng(seed)
    U = rng.random((n, R))
    return workloads.make_problem("edge", A, U, np.zeros((n, 0)), np.zeros(0), [f] * R, m, C,
                                  lam[0] * 0.9, lam[-1] * 1.1, degree=degree, prob_dim=lam[-1] * 1.1 / 4)


def oracle(P):
    return fab.OracleEngine(A=P.A, U0=P.U, Q=None, m=P.m, gamma=P.gamma, gs_re=P.gs_re, gs_im=P.gs_im,
                            flam=np.zeros((0, P.R)), wts=P.wts, shifts=P.shifts, col_scale=np.ones(P.R)).solve()


@pytest.mark.parametrize("n", [1, 2, 5, 31, 32, 33, 65, 97])
@pytest.mark.parametrize("R", [1, 2, 4])
def test_odd_sizes(engine_lib, n, R):
    A = spd(n, seed=n + 7 * R)
    P = problem(A, R=R, m=min(n, 8), seed=n)
    eng = Engine.from_problem(P, sync=False)
    eng.solve()
    assert rel(eng.get_solution(), oracle(P)) < 1e-10
    eng.delete()


def test_dense_row_and_sorted_slices(engine_lib):
    A = spd(200, seed=3, density=0.02, dense_row=True)
    P = problem(A, R=2, m=10, degree=2)
    want = oracle(P)
    for sigma in (0, 64):
        eng = Engine.from_problem(P, sell_sigma=sigma, sync=False)
        eng.solve()
        assert rel(eng.get_solution(), want) < 1e-10
        eng.delete()


def test_csc_unsorted_input(engine_lib):
    A = spd(150, seed=11, density=0.05)
    P = problem(A, R=1, m=10)
    want = oracle(P)
    C = sp.csc_matrix(A)
    rng = np.random.default_rng(0)
    # shuffle the row indices inside every column (MATLAB keeps them sorted; the engine must not care)
    for j in range(C.shape[1]):
        a, b = C.indptr[j], C.indptr[j + 1]
        perm = rng.permutation(b - a)
        C.indices[a:b] = C.indices[a:b][perm]
        C.data[a:b] = C.data[a:b][perm]
    eng = Engine(C, P.U, None, None, None, P.m, P.gamma, P.gs_re, P.gs_im, P.wts, P.shifts,
                 col_scale=np.ones(1), matrix_format="csc")
    eng.solve()
    assert rel(eng.get_solution(), want) < 1e-10
    eng.delete()


def test_batch_with_zero_column(engine_lib):
    probs = workloads.config5_batch(nprob=3, R=2, seed=9, lo=8, hi=30, m=12, C=12)
    probs[1].U[:, 1] = 0.0
    eng = BatchEngine(probs, sync=False)
    eng.solve()
    xs = eng.split(eng.get_solution())
    assert np.all(xs[1][:, 1] == 0.0)
    assert eng.meff()[1 * 2 + 1] == 0
    for i, (P, x) in enumerate(zip(probs, xs)):
        cols = [0, 1] if i != 1 else [0]
        for c in cols:
            P1 = workloads.make_problem(P.name, P.A, P.U[:, c:c + 1], P.Q, P.lam, P.funcs[:1], P.m, P.C,
                                        P.l1, P.lN, degree=P.d)
            assert rel(x[:, c], oracle(P1)[:, 0]) < 1e-10
    eng.delete()


def test_autotune_on_gpu(engine_lib, tmp_path):
    P = workloads.config1_small(N=40, k=0, m=20, C=16, R=1)
    space = [dict(threads=256, blocks_per_sm=0, col_staging=2, sync_policy=0),
             dict(threads=128, blocks_per_sm=0, col_staging=1, sync_policy=1)]
    cache = tmp_path / "tune.json"
    best = autotune.tune(P, precision="fp64", reps=2, cache_path=str(cache), space=space)
    assert not best["cached"] and best["ms"] > 0 and best["trials"] == 2
    again = autotune.tune(P, precision="fp64", reps=2, cache_path=str(cache), space=space)
    assert again["cached"] and again["threads"] == best["threads"]
    eng = Engine.from_problem(P, **{k: best[k] for k in ("threads", "blocks_per_sm", "col_staging", "sync_policy")})
    eng.solve()
    assert rel(eng.get_solution(), oracle(P)) < 1e-10
    eng.delete()


def test_wait_limit_reports_timeout_and_context_survives(engine_lib):
    """Failure detection without a GPU fault: with a 100 ns wait limit the
    bounded barrier and neighbour waits of a many-block launch run out; the
    kernel records GM_ERR_TIMEOUT and returns, the host reads the status, and
    the same context (and the same handle after gm_set_U) solves normally."""
    from gpumatfun_gb300.engine import GmError
    P = workloads.fd2d_problem(160, 0, 16, 12, [params.frac_exp(1e-3, 1.5)], R=1, scale=161.0 ** 2, seed=1)
    want = oracle(P)
    eng = None
    with pytest.raises(GmError) as err:
        # the create-time deflation launch may already run out; otherwise a solve does
        eng = Engine.from_problem(P, timeout_s=1e-7, threads=128, sync=True)
        for _ in range(20):           # a launch whose every wait is shorter than 100 ns is not an error
            eng.solve()
    assert err.value.code == 5, str(err.value)     # GM_ERR_TIMEOUT
    if eng is not None:
        eng.delete()
    ok = Engine.from_problem(P, threads=128, sync=True)
    ok.solve()
    assert rel(ok.get_solution(), want) < 1e-10
    ok.delete()


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
@pytest.mark.parametrize("R,degree", [(1, 8), (2, 5), (1, 3), (4, 6)])
def test_matrix_powers_passes_are_bit_identical(engine_lib, precision, R, degree):
    """Two Horner levels per pass (halo rows recomputed per block, the level
    in between in shared memory) run the same operations in the same order as
    one level per pass: the results agree bit for bit, on a grid of hundreds
    of blocks whose two-hop waits are exercised."""
    from gpumatfun_gb300 import adjoint
    mesh = __import__("gpumatfun_gb300").problems.disk_mesh(40000, seed=2)
    cent = mesh.nodes[mesh.tris].mean(axis=1)
    kappa = np.exp(__import__("gpumatfun_gb300").problems.gaussian_random_field(cent, sigma=1.0, ell=0.1, seed=3))
    A = adjoint.fe_structure(mesh).matrix(kappa)
    lam_hi = 1.05 * float(__import__("scipy.sparse.linalg", fromlist=["eigsh"]).eigsh(
        A, k=1, which="LA", return_eigenvectors=False, tol=1e-4)[0])
    f = params.frac_power(-0.8)
    rng = np.random.default_rng(R + degree)
    U = rng.random((A.shape[0], R))
    P = workloads.make_problem("mpk", A, U, np.zeros((A.shape[0], 0)), np.zeros(0), [f] * R, 12, 16,
                               lam_hi / 2e4, lam_hi, degree=degree, prob_dim=lam_hi / 4)
    out = []
    for mp in (0, 1):
        eng = Engine.from_problem(P, precision=precision, threads=128, sync=False, matrix_powers=mp)
        assert eng.info()["grid_blocks"] > 200
        assert eng.info()["matrix_powers"] == mp
        eng.solve()
        out.append(eng.get_solution())
        eng.delete()
    np.testing.assert_array_equal(out[0], out[1])
    if precision == "fp64" and R <= 2:
        assert rel(out[1], oracle(P)) < 1e-10
