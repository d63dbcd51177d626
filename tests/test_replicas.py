"""The multi-GPU form of the benchmark runs independent replicas (the sweep
has no exchange step on one problem: replicas only).  Its host logic --
the slowest rank's time and the whole-job rate -- runs here on two gloo
ranks on the CPU."""
import os
import socket

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _rank(rank, world, port, out):
    import sys
    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    import bench
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    local_ms = 10.0 + 5.0 * rank          # rank 1 is the slower replica
    slowest = bench.max_over_ranks(local_ms, dist, "cpu")
    rate = bench.whole_job_rate(1000, 4, world, slowest)
    out[rank] = (slowest, rate)
    dist.barrier()
    dist.destroy_process_group()


def test_replica_timing_takes_the_slowest_rank():
    world = 2
    port = _free_port()
    out = mp.Manager().dict()
    mp.spawn(_rank, args=(world, port, out), nprocs=world, join=True)
    for r in range(world):
        slowest, rate = out[r]
        assert slowest == 15.0
        assert rate == pytest.approx(2 * 1000 * 4 / 15e-3)


def test_single_process_needs_no_group():
    import bench
    assert bench.max_over_ranks(3.5, None, "cpu") == 3.5
    assert bench.whole_job_rate(10, 2, 1, 20.0) == pytest.approx(1000.0)
