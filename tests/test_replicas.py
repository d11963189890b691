"""Multi-GPU runs of bench.py are replicas: each rank mines the same job and
rank 0 reports the slowest rank's time over all ranks' jobs (and all ranks'
embeddings over that time).  The
reduction is checked here with two gloo ranks on the CPU."""
import os
import sys

import pytest
import torch.multiprocessing as mp

from helpers import ROOT


def _worker(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    sys.path.insert(0, ROOT)
    import torch.distributed as dist
    import bench
    dist.init_process_group("gloo", rank=rank, world_size=world)
    times = bench.max_over_ranks([100.0 + 50.0 * rank, 10.0 * (world - rank)])
    out[rank] = (times, bench.replica_value(world, 2_000_000, times[0]), bench.replica_ms_per_job(world, 5, times[0]))
    dist.destroy_process_group()


def test_two_rank_replica_reduction():
    port = 29500 + os.getpid() % 1000
    with mp.Manager() as man:
        out = man.dict()
        mp.spawn(_worker, args=(2, port, out), nprocs=2, join=True)
        res = dict(out)
    assert res[0][0] == [150.0, 20.0] and res[1][0] == [150.0, 20.0]
    assert res[0][1] == pytest.approx(2 * 2_000_000 / 0.150)
    assert res[0][2] == pytest.approx(150.0 / 10)


def test_single_process_is_identity():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.max_over_ranks([1.5, 2.5]) == [1.5, 2.5]
