"""The multi-GPU form of bench.py runs independent replicas (one per rank,
no data-path collective) and reports world * units / slowest rank's time.
This checks that aggregation with world_size 2 over gloo on the CPU."""
import os
import sys

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _rank(rank, world, port, out):
    sys.path.insert(0, ROOT)
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    # rank r pretends to have needed (r + 1) seconds for 1000 units
    value, t = bench.replica_throughput(rank + 1.0, 1000, world, dist, "cpu")
    out[rank] = (value, t)
    dist.barrier()
    dist.destroy_process_group()


def test_replica_throughput_uses_the_slowest_rank():
    world = 2
    port = 29500 + (os.getpid() % 1000)
    mgr = mp.Manager()
    out = mgr.dict()
    mp.spawn(_rank, args=(world, port, out), nprocs=world, join=True)
    for r in range(world):
        value, t = out[r]
        assert t == 2.0  # the slower rank
        assert value == world * 1000 / 2.0
