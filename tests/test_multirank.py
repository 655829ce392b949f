"""The benchmark's multi-GPU path is replicas only (independent reconstructions, no collective on the
data path); its timing aggregation (max over ranks) runs here as two gloo ranks on the CPU."""
import os
import sys

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _worker(rank, world, port, out):
    sys.path.insert(0, ROOT)
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench

    t = bench.max_over_ranks(1.5 + rank, dist)  # rank 1 is the slow one
    out[rank] = bench.replica_throughput(1001, 4, world, t)
    dist.barrier()
    dist.destroy_process_group()


def test_two_gloo_ranks_take_the_slowest_rank():
    import random

    port = random.randint(20000, 40000)
    with mp.Manager() as m:
        out = m.dict()
        mp.spawn(_worker, args=(2, port, out), nprocs=2, join=True)
        vals = dict(out)
    assert vals[0] == vals[1] == pytest.approx(1001 * 4 * 2 / 2.5)


def test_single_process_is_identity():
    sys.path.insert(0, ROOT)
    import bench

    assert bench.max_over_ranks(3.25, None) == 3.25
    assert bench.replica_throughput(1001, 10, 1, 2.0) == pytest.approx(5005.0)
