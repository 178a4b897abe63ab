"""The N>1 bench path (independent replicas, one per rank) on CPU: two gloo ranks."""
import os
import socket
import sys

import pytest
import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, ms, out):
    import torch.distributed as dist
    sys.path.insert(0, ROOT)
    import bench
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        ms_max, rate = bench.replica_rate(ms[rank], 1000.0, dist, device="cpu")
        out[rank] = (ms_max, rate)
    finally:
        dist.destroy_process_group()


def test_replica_rate_two_gloo_ranks():
    """Each rank times its own replica; both see the slowest rank's time, and the job rate
    is world x units / that time."""
    world, port = 2, _free_port()
    ms = [4.0, 5.0]
    ctx = mp.get_context("spawn")
    out = ctx.Manager().dict()
    procs = [ctx.Process(target=_rank, args=(r, world, port, ms, out)) for r in range(world)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
        assert p.exitcode == 0
    for r in range(world):
        ms_max, rate = out[r]
        assert ms_max == pytest.approx(5.0)
        assert rate == pytest.approx(world * 1000.0 / 5e-3)


def test_replica_rate_single_process():
    sys.path.insert(0, ROOT)
    import bench
    ms_max, rate = bench.replica_rate(2.0, 100.0, None, device="cpu")
    assert ms_max == 2.0 and rate == pytest.approx(100.0 / 2e-3)
