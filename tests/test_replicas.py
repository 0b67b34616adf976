"""The multi-GPU form of the benchmark is replicas only (pixels and samples are
independent; no exchange step): each rank renders its own step and the job is
charged the slowest rank.  These world-size-2 gloo tests on the CPU cover the
cross-rank reduction and the whole-job throughput bench.py reports."""
import os
import socket

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank: int, world: int, port: int, results):
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    step_ms = 100.0 + 25.0 * rank  # rank 1 is the slowest
    slowest = bench.max_over_ranks(step_ms, "cpu")
    results[rank] = (slowest, bench.whole_job_mpaths(132_710_400, world, slowest))
    dist.barrier()
    dist.destroy_process_group()


def test_slowest_rank_charged_over_gloo():
    world = 2
    with mp.Manager() as m:
        results = m.dict()
        mp.spawn(_worker, args=(world, _free_port(), results), nprocs=world, join=True)
        got = dict(results)
    assert got[0] == got[1]
    slowest, mpaths = got[0]
    assert slowest == 125.0
    assert abs(mpaths - 2 * 132_710_400 / 125e3) < 1e-9


def test_single_process_needs_no_group():
    import bench
    assert bench.max_over_ranks(7.5, "cpu") == 7.5
    assert bench.whole_job_mpaths(1e6, 1, 1000.0) == 1.0
