"""The N > 1 path of bench.py (replicas, one image stream per rank, no
data-path collective): the job time is the slowest rank's, the throughput
counts every rank's units, and the reference arm runs on rank 0 only.
Exercised with two gloo ranks on the CPU."""
import os
import socket
import sys

import pytest
import torch
import torch.distributed as dist
import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _rank_main(rank, world, port, q):
    os.environ.update({"MASTER_ADDR": "127.0.0.1", "MASTER_PORT": str(port), "RANK": str(rank),
                       "WORLD_SIZE": str(world), "LOCAL_RANK": str(rank)})
    sys.path.insert(0, ROOT)
    import bench
    dist.init_process_group("gloo", init_method="env://", rank=rank, world_size=world)
    try:
        rank_ms = 1000.0 + 250.0 * rank  # rank 1 is the slow one
        total = bench.max_over_ranks(rank_ms)
        value = bench.job_throughput(world, 4, 0.25, total)
        q.put((rank, total, value, bench.dist_setup()))
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
        assert p.exitcode == 0
    got = sorted(q.get(timeout=10) for _ in range(2))
    for rank, total, value, (world, r, local) in got:
        assert total == 1250.0  # max over ranks
        assert value == pytest.approx(2 * 4 * 0.25 / 1.25)  # both ranks' units / slowest time
        assert (world, r, local) == (2, rank, rank)


def test_single_process_is_its_own_max():
    sys.path.insert(0, ROOT)
    import bench
    assert not dist.is_initialized()
    assert bench.max_over_ranks(12.5) == 12.5
    assert bench.job_throughput(1, 5, 0.262144, 1000.0) == pytest.approx(1.31072)


def test_reference_arm_other_ranks_exit_without_work(monkeypatch):
    sys.path.insert(0, ROOT)
    import bench
    monkeypatch.setenv("RANK", "1")
    monkeypatch.setenv("WORLD_SIZE", "2")
    called = []
    monkeypatch.setattr(bench, "workload", lambda *a, **k: called.append(1))

    class A:
        steps, warmup, gpus = 1, 0, 2
    assert bench.run_reference(A()) == 0
    assert not called
