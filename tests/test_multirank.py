"""The multi-GPU path of bench.py is replicas: each rank counts the whole
workload and the job time is the slowest rank's.  Exercised here with two
gloo ranks on the CPU (no GPU, no NCCL)."""
import os
import sys

import pytest
import torch.distributed as dist
import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _rank(rank, world, port, out):
    sys.path.insert(0, ROOT)
    import bench

    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    times = [1.0 + rank, 10.0 - rank]  # device-resident, end-to-end seconds on this rank
    got = bench.max_over_ranks(times, world)
    out[rank] = (got, bench.job_value(8, 3, world, got[0]))
    dist.barrier()
    dist.destroy_process_group()


def test_two_gloo_ranks_take_the_slowest_time():
    ctx = mp.get_context("spawn")
    with ctx.Manager() as m:
        out = m.dict()
        port = 29000 + (os.getpid() % 1000)
        procs = [ctx.Process(target=_rank, args=(r, 2, port, out)) for r in range(2)]
        for p in procs:
            p.start()
        for p in procs:
            p.join(120)
            assert p.exitcode == 0
        for r in range(2):
            got, value = out[r]
            assert got == [2.0, 10.0]
            assert value == pytest.approx(8 * 2 * 3 / 2.0)


def test_single_rank_needs_no_process_group():
    sys.path.insert(0, ROOT)
    import bench

    assert bench.max_over_ranks([3.0, 4.0], 1) == [3.0, 4.0]
    assert bench.job_value(8, 2, 1, 4.0) == 4.0
