"""Multi-GPU is replicas only: every rank clusters its own copy of the
workload and the bench reports world * units / (slowest rank's time).  The
aggregation runs here on CPU with two gloo ranks."""
import os
import socket
import sys

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, times, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    sys.path.insert(0, ROOT)
    import bench
    t, value = bench.aggregate(times[rank], 1000, world, "cpu")
    out[rank] = (t, value)
    dist.destroy_process_group()


def test_two_replicas_report_the_slowest_rank():
    world, times = 2, [0.5, 2.0]
    port = _free_port()
    out = mp.Manager().dict()
    mp.spawn(_rank, args=(world, port, times, out), nprocs=world, join=True)
    for r in range(world):
        t, value = out[r]
        assert t == pytest.approx(2.0)
        assert value == pytest.approx(world * 1000 / 2.0)


def test_one_rank_is_its_own_time():
    sys.path.insert(0, ROOT)
    import bench
    t, value = bench.aggregate(0.25, 1000, 1, "cpu")
    assert t == 0.25 and value == pytest.approx(4000.0)
