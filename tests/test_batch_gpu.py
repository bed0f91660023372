"""Batched engine (several independent problems of uneven size in one
launch) against the per-problem FP64 oracle."""
import numpy as np
import pytest

from gpumatfun_gb300 import BatchEngine, Engine, workloads
from gpumatfun_gb300.engine import GmError
from oracle import fab

pytestmark = pytest.mark.gpu


def rel(a, b):
    return float(np.linalg.norm(np.asarray(a) - np.asarray(b)) / np.linalg.norm(b))


def oracle(P):
    return fab.OracleEngine(A=P.A, U0=P.U, Q=P.Q, m=P.m, gamma=P.gamma, gs_re=P.gs_re, gs_im=P.gs_im,
                            flam=P.flam, wts=P.wts, shifts=P.shifts, col_scale=np.ones(P.R)).solve()


@pytest.mark.parametrize("R,degree", [(1, 0), (4, 0), (2, 3)])
def test_batch_matches_per_problem_oracle(engine_lib, R, degree):
    probs = workloads.config5_batch(nprob=6, R=R, seed=3, lo=10, hi=70, m=24, C=24, degree=degree)
    eng = BatchEngine(probs, precision="fp64", sync=False, threads=128)
    assert eng.info()["problems"] == 6
    eng.solve()
    xs = eng.split(eng.get_solution())
    for P, x in zip(probs, xs):
        assert rel(x, oracle(P)) < 1e-10
    # the stepwise reference entry points work per problem as well
    eng.set_U(np.concatenate([P.U for P in probs]))
    eng.build_subspace(); eng.lin_sys_solves(); eng.apply_V()
    for P, x in zip(probs, eng.split(eng.get_solution())):
        assert rel(x, oracle(P)) < 1e-10
    ab = eng.get_aabb()
    assert ab.shape == (6, 25, 2 * R)
    assert len(eng.meff()) == 6 * R


def test_batch_agrees_with_single_engines(engine_lib):
    probs = workloads.config5_batch(nprob=4, R=2, seed=5, lo=12, hi=60, m=20, C=16)
    eng = BatchEngine(probs, sync=False)
    eng.solve()
    for P, x in zip(probs, eng.split(eng.get_solution())):
        e1 = Engine.from_problem(P)
        e1.solve()
        assert rel(x, e1.get_solution()) < 1e-12
        e1.delete()


def test_batch_mixed_precision(engine_lib):
    probs = workloads.config5_batch(nprob=5, R=4, seed=7, lo=16, hi=80, m=40, C=32)
    eng = BatchEngine(probs, precision="mixed", sync=False)
    eng.solve()
    for P, x in zip(probs, eng.split(eng.get_solution())):
        assert rel(x, oracle(P)) < 1e-6


def test_batch_rejects_mismatched_problems(engine_lib):
    a = workloads.config5_batch(nprob=1, R=2, seed=1, lo=10, hi=12, m=10, C=8)[0]
    b = workloads.config5_batch(nprob=1, R=2, seed=2, lo=10, hi=12, m=12, C=8)[0]
    with pytest.raises(GmError):
        BatchEngine([a, b])
