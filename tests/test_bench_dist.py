"""CPU test of bench.py's multi-rank path with two gloo ranks: every rank
reconstructs its own volume, the elapsed time is the maximum over ranks and
the value counts the iterations of all ranks."""

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


def _worker(rank, world, port, out):
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    local_ms = 100.0 + 50.0 * rank  # rank 1 is slower
    ms = bench.max_over_ranks(local_ms, dist, "cpu")
    out[rank] = (ms, bench.whole_job_rate(10, world, ms))
    dist.barrier()
    dist.destroy_process_group()


def test_two_ranks_max_time_and_whole_job_value():
    world = 2
    port = _free_port()
    with mp.Manager() as mgr:
        out = mgr.dict()
        mp.spawn(_worker, args=(world, port, out), nprocs=world, join=True)
        res = dict(out)
    assert res[0][0] == res[1][0] == 150.0
    assert abs(res[0][1] - 2 * 10 / 0.150) < 1e-9


def test_single_rank_without_process_group():
    import bench
    assert bench.max_over_ranks(3.5, None, "cpu") == 3.5
    assert abs(bench.whole_job_rate(5, 1, 2000.0) - 2.5) < 1e-12
