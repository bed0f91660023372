"""The multi-GPU path is replicas only: independent problems per rank, a max
over ranks of the step time, and the job throughput over all ranks.  Checked
with two gloo ranks on CPU."""
import os
import socket

import pytest
import torch
import torch.multiprocessing as mp

from gpumatfun_gb300 import replicas


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, out):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        # rank r takes 10 + 5 r ms per step and solves 3 right-hand sides per step
        ms_local = 10.0 + 5.0 * rank
        vals = replicas.max_over_ranks([ms_local, 1.0 + rank])
        thr, ms = replicas.job_throughput(3, ms_local, world)
        out[rank] = (vals, thr, ms, replicas.rank0_only(rank))
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks_take_the_slowest_rank():
    world = 2
    ctx = mp.get_context("spawn")
    with ctx.Manager() as mgr:
        out = mgr.dict()
        mp.start_processes(_worker, args=(world, _free_port(), out), nprocs=world, start_method="spawn")
        res = dict(out)
    for rank in range(world):
        vals, thr, ms, only0 = res[rank]
        assert vals == [15.0, 2.0]             # element-wise max over the two ranks
        assert ms == 15.0
        assert thr == pytest.approx(2 * 3 * 1e3 / 15.0)   # all ranks' units over the slowest time
        assert only0 == (rank == 0)


def test_single_process_is_identity():
    assert replicas.max_over_ranks([4.0, 2.0]) == [4.0, 2.0]
    thr, ms = replicas.job_throughput(4, 20.0, 1)
    assert ms == 20.0 and thr == pytest.approx(200.0)
