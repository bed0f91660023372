"""The C/OpenMP restatement of the reference CPU path (timed CPU baseline)
against the numpy oracle (no GPU)."""
import numpy as np
import pytest

from gpumatfun_gb300 import workloads
from oracle import cpu_fab, fab


@pytest.mark.parametrize("R,degree", [(1, 0), (2, 3), (4, 1)])
def test_cpu_fab_matches_oracle(R, degree):
    P = workloads.config1_small(N=18, k=3, m=30, C=20, R=R, degree=degree, seed=2)
    ora = fab.OracleEngine(A=P.A, U0=P.U, Q=P.Q, m=P.m, gamma=P.gamma, gs_re=P.gs_re, gs_im=P.gs_im,
                           flam=P.flam, wts=P.wts, shifts=P.shifts, col_scale=np.ones(R))
    want = ora.solve() - ora.update
    got = cpu_fab.run(P.A, ora.U, P.m, P.gamma, P.gs_re, P.gs_im, P.wts, P.sigma, threads=2)
    assert np.linalg.norm(got - want) / np.linalg.norm(want) < 1e-11
