"""The multi-GPU form of the bench is replicas only: each rank advances its
own scene and the job's figures are the slowest rank's time and the summed
work.  This runs that host-side combination on two gloo ranks on the CPU."""
import os
import socket

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench

    ms, work = bench.combine_replicas(10.0 + 5.0 * rank, 1000 * (rank + 1), dist, "cpu")
    out[rank] = (ms, work)
    dist.destroy_process_group()


def test_two_replicas_combine_on_gloo():
    world = 2
    manager = mp.Manager()
    out = manager.dict()
    mp.start_processes(_rank, args=(world, _free_port(), out), nprocs=world, start_method="spawn")
    for r in range(world):
        assert out[r] == (15.0, 3000.0)


def test_single_rank_is_identity():
    import bench

    assert bench.combine_replicas(7.5, 42) == (7.5, 42)
