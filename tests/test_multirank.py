"""The multi-process path of bench.py on CPU (gloo, world size 2): every rank
gets the slowest rank's time, and the reported rate counts the units of all
ranks over that time (replicas: one process per GPU, no data-path
collective)."""

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


def _rank(rank, world, port, out):
    sys.path.insert(0, ROOT)
    import bench

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        ms = 10.0 + 5.0 * rank  # rank 1 is the slow one
        slowest = bench.max_over_ranks(ms, dist, "cpu")
        out[rank] = (slowest, bench.whole_job_rate(world, 1000, 4, slowest))
        dist.barrier()
    finally:
        dist.destroy_process_group()


def test_slowest_rank_sets_the_time_and_rates_add_up():
    world = 2
    port = _free_port()
    with mp.Manager() as m:
        out = m.dict()
        mp.spawn(_rank, args=(world, port, out), nprocs=world, join=True)
        res = dict(out)
    assert set(res) == {0, 1}
    for rank in (0, 1):
        slowest, rate = res[rank]
        assert slowest == 15.0
        assert rate == pytest.approx(2 * 1000 * 4 / 0.015)


def test_one_process_needs_no_collective():
    sys.path.insert(0, ROOT)
    import bench

    assert bench.max_over_ranks(7.5, None, "cpu") == 7.5
    assert bench.whole_job_rate(1, 500, 2, 10.0) == pytest.approx(1e5)
