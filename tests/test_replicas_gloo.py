"""The replica (N > 1) bookkeeping of bench.py on CPU with two gloo ranks:
the reported time is the slowest rank's and the whole-job rate counts every
rank's units over it."""
import os
import socket
import sys

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _rank(rank, world, port, out):
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    sys.path.insert(0, ROOT)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    seconds = [2.0, 3.0][rank]
    t = bench.max_over_ranks(seconds, dist, device="cpu")
    out[rank] = (t, bench.whole_job_rate(1000.0, world, t))
    dist.barrier()
    dist.destroy_process_group()


def test_two_gloo_ranks_report_the_slowest_time_and_whole_job_rate():
    world, port = 2, _free_port()
    out = mp.Manager().dict()
    mp.spawn(_rank, args=(world, port, out), nprocs=world, join=True)
    for r in range(world):
        t, rate = out[r]
        assert t == 3.0
        assert rate == pytest.approx(2 * 1000.0 / 3.0)
