"""The multi-GPU path of bench.py is replicas: every rank renders the same workload on its own GPU
and the job's time is the slowest rank's.  The reduction is checked here with two gloo ranks on
the CPU (no GPU needed)."""
import os
import socket

import pytest
import torch.distributed as dist
import torch.multiprocessing as mp

import bench


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank: int, world: int, port: int, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        mine = [10.0 + 5.0 * rank, 3.0 - rank]           # rank 1 is slower on the first timing
        out[rank] = bench.max_over_ranks(mine)
        dist.barrier()
    finally:
        dist.destroy_process_group()


def test_max_over_ranks_gloo_world2():
    port = _free_port()
    with mp.Manager() as m:
        out = m.dict()
        mp.spawn(_rank, args=(2, port, out), nprocs=2, join=True)
        got = dict(out)
    assert got[0] == got[1] == [15.0, 3.0]


def test_job_throughput_counts_every_rank():
    # 20 frames per rank on 4 ranks, slowest rank took 100 ms
    assert bench.job_throughput(20, 4, 100.0) == pytest.approx(800.0)
    assert bench.max_over_ranks([1.0, 2.0]) == [1.0, 2.0]   # no process group: identity
