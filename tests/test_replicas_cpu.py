"""The multi-GPU path is replicas only (halos are independent; the reference's only
exchange is the map all-reduce, not rebuilt): each rank paints its own catalogue and the
whole-job throughput takes the slowest rank.  That reduction runs here on two gloo
ranks on the CPU."""
import os
import sys

import pytest
import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _rank(rank, world, port, times, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                      WORLD_SIZE=str(world))
    sys.path.insert(0, ROOT)
    import torch.distributed as dist

    import bench
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        ms = bench.max_over_ranks(times[rank])
        out[rank] = (ms, bench.job_throughput(1000, world, ms))
    finally:
        dist.destroy_process_group()


def test_slowest_rank_sets_the_job_throughput():
    world, times = 2, [3.0, 5.0]
    port = 29500 + os.getpid() % 2000
    with mp.Manager() as mgr:
        out = mgr.dict()
        mp.spawn(_rank, args=(world, port, times, out), nprocs=world, join=True)
        res = dict(out)
    for r in range(world):
        ms, value = res[r]
        assert ms == max(times)
        assert value == pytest.approx(1000 * world / (max(times) * 1e-3))


def test_single_process_reduction_is_identity():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.max_over_ranks(2.5) == 2.5
    assert bench.job_throughput(10, 1, 1.0) == pytest.approx(1e4)
