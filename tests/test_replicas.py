"""bench.py's multi-GPU path is replicas only: every rank runs the whole join
and the job is timed by its slowest rank.  The aggregation runs here on two
gloo ranks on the CPU (127.0.0.1 rendezvous)."""
import os
import socket
import sys

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    import torch.distributed as dist

    sys.path.insert(0, REPO)
    import bench

    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        step_s = 0.10 + 0.05 * rank  # rank 1 is the slow one
        slowest = bench.max_over_ranks(step_s, dist, "cpu")
        out[rank] = (slowest, bench.replica_value(1000, world, slowest))
    finally:
        dist.destroy_process_group()


def test_two_replicas_slowest_rank_sets_the_time():
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp

    port = _free_port()
    manager = mp.get_context("spawn").Manager()
    out = manager.dict()
    mp.spawn(_rank, args=(2, port, out), nprocs=2, join=True)
    for rank in range(2):
        slowest, value = out[rank]
        assert slowest == pytest.approx(0.15)
        assert value == pytest.approx(2 * 1000 / 0.15)


def test_single_process_is_its_own_maximum():
    sys.path.insert(0, REPO)
    import bench

    assert bench.max_over_ranks(0.25, None, "cpu") == 0.25
    assert bench.replica_value(10, 1, 0.5) == 20
