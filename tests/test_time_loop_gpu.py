"""Time loop (fused solve + update per step), with and without CUDA-graph
replay, against the MEX-style call sequence and the oracle."""
import numpy as np
import pytest

from gpumatfun_gb300 import LanczosEngine, workloads
from oracle import fab

pytestmark = pytest.mark.gpu


def rel(a, b):
    return float(np.linalg.norm(np.asarray(a) - np.asarray(b)) / np.linalg.norm(b))


def make(P, dt, ode, fhn, **kw):
    return LanczosEngine(P.U, P.A, P.Q, P.lam, P.m, P.gamma, P.gs_re, P.gs_im, P.flam[:, 0], P.flam[:, 1],
                         dt, ode, fhn["aode"], fhn["bode"], fhn["code"], fhn["vrest"], fhn["vamp"], fhn["vth"],
                         fhn["vpeak"], fhn["c1ion"], fhn["c2ion"], np.ones(P.n), P.wts[0], P.wts[1], P.shifts, **kw)


@pytest.mark.parametrize("monodomain", [True, False])
def test_time_loop_graph_matches_calls_and_oracle(engine_lib, monodomain):
    P, dt, ode, fhn = workloads.monodomain_problem(24, k=4, m=30, C=16)
    steps = 4
    seq = make(P, dt, ode, fhn)
    for _ in range(steps):
        seq.build_subspace(); seq.lin_sys_solves(); seq.apply_V()
        seq.update_U_monodomain() if monodomain else seq.update_U()
    u_seq = seq.get_U()
    plain = make(P, dt, ode, fhn, sync=False)
    plain.time_loop(steps, monodomain=monodomain, graph=False)
    graph = make(P, dt, ode, fhn, sync=False)
    graph.time_loop(steps, monodomain=monodomain, graph=True)
    np.testing.assert_array_equal(plain.get_U(), u_seq)
    np.testing.assert_array_equal(graph.get_U(), u_seq)
    # a second replay of the cached graph continues the same trajectory
    graph.time_loop(steps, monodomain=monodomain, graph=True)
    plain.time_loop(steps, monodomain=monodomain, graph=False)
    np.testing.assert_array_equal(graph.get_U(), plain.get_U())
    ora = fab.OracleEngine(A=P.A, U0=P.U, Q=P.Q, m=P.m, gamma=P.gamma, gs_re=P.gs_re, gs_im=P.gs_im,
                           flam=P.flam, wts=P.wts, shifts=P.shifts, dt=dt, ode=ode.copy(),
                           fhn=(fhn["aode"], fhn["bode"], fhn["code"], fhn["vrest"], fhn["vamp"], fhn["vth"],
                                fhn["vpeak"], fhn["c1ion"]))
    for _ in range(2 * steps):
        ora.build_subspace(); ora.lin_sys_solves(); ora.apply_V()
        ora.update_U_monodomain() if monodomain else ora.update_U()
    assert rel(graph.get_U(), ora.get_U()) < 1e-10


def test_time_loop_graph_batch_of_many_blocks(engine_lib):
    """A graph replay on a grid with hundreds of blocks: the progress flags
    are reset inside the graph, so replays cannot see stale flags."""
    P, dt, ode, fhn = workloads.monodomain_problem(160, k=8, m=20, C=12)
    a = make(P, dt, ode, fhn, sync=False, threads=128)
    b = make(P, dt, ode, fhn, sync=False, threads=128)
    assert a.info()["grid_blocks"] > 150
    for _ in range(3):
        a.time_loop(2, monodomain=True, graph=True)
    b.time_loop(6, monodomain=True, graph=False)
    np.testing.assert_array_equal(a.get_U(), b.get_U())


@pytest.mark.parametrize("monodomain", [True, False])
def test_checkpoint_resume_continues_bit_for_bit(engine_lib, monodomain):
    """get_state after some steps, set_state on a fresh handle: the resumed
    run continues the same trajectory bit for bit (Usol and the recovery
    variable are the whole state of a time loop)."""
    P, dt, ode, fhn = workloads.monodomain_problem(24, k=4, m=30, C=16)
    a = make(P, dt, ode, fhn)
    a.time_loop(5, monodomain=monodomain, graph=False)
    U5, ode5 = a.get_state()
    a.time_loop(4, monodomain=monodomain, graph=True)
    b = make(P, dt, ode, fhn)
    b.set_state(U5, ode5)
    np.testing.assert_array_equal(b.get_U(), U5)
    b.time_loop(4, monodomain=monodomain, graph=True)
    np.testing.assert_array_equal(b.get_U(), a.get_U())
    np.testing.assert_array_equal(b.get_state()[1], a.get_state()[1])


def test_graph_on_legacy_stream_is_refused_and_handle_stays_synchronous(engine_lib):
    """A CUDA graph cannot be captured on the legacy default stream: the call
    is refused up front (GM_ERR_ARG) and the handle keeps its synchronous
    mode, so the next plain time loop returns with the stream drained and
    continues the trajectory as a fresh handle would."""
    import torch
    from gpumatfun_gb300.engine import GmError
    P, dt, ode, fhn = workloads.monodomain_problem(64, k=4, m=30, C=16)
    a = make(P, dt, ode, fhn, sync=True)
    a.set_stream(0)   # torch's default stream: the legacy default stream
    with pytest.raises(GmError) as err:
        a.time_loop(3, monodomain=True, graph=True)
    assert err.value.code == 1, str(err.value)
    a.time_loop(20, monodomain=True, graph=False)
    assert torch.cuda.default_stream().query()   # synchronous mode: nothing left in flight
    b = make(P, dt, ode, fhn)
    b.time_loop(20, monodomain=True, graph=False)
    np.testing.assert_array_equal(a.get_U(), b.get_U())
