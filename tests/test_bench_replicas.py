"""bench.py's multi-GPU arm is replicas only: every rank assembles its own copy
of the workload and the job's time is the slowest rank's. The host logic runs
here on world-size-2 gloo process groups on the CPU."""
import os
import socket

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist
import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    import sys
    sys.path.insert(0, ROOT)
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    ms = bench.max_over_ranks(1.0 + rank, world, "cpu")
    out[rank] = (ms, bench.replica_value(1000, ms, world))
    dist.destroy_process_group()


def test_slowest_rank_sets_the_time_and_every_replica_counts():
    world = 2
    out = mp.Manager().dict()
    mp.spawn(_rank, args=(world, _free_port(), out), nprocs=world, join=True)
    for r in range(world):
        ms, value = out[r]
        assert ms == 2.0
        assert value == pytest.approx(world * 1000 / 2.0e-3)


def test_single_process_needs_no_group():
    import sys
    sys.path.insert(0, ROOT)
    import bench
    assert bench.max_over_ranks(3.5, 1, "cpu") == 3.5
    assert bench.replica_value(384000, 1.8, 1) == pytest.approx(384000 / 1.8e-3)
