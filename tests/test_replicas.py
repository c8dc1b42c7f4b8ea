"""The benchmark's N-GPU path is replicas only: every rank renders its own passes and
the job is timed by the slowest rank.  Its one collective (a max over ranks) and the
whole-job throughput run here on CPU with two gloo ranks; the reference arm's non-zero
ranks exit without work."""
import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, ws, port, q):
    import torch
    import torch.distributed as dist
    sys.path.insert(0, ROOT)
    import bench
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=ws)
    try:
        ms = bench.max_over_ranks(torch, 10.0 + 5.0 * rank, ws, device="cpu")
        q.put((rank, ms, bench.replica_throughput(ws, 1000, ms)))
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks_time_the_slowest_and_sum_the_work():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
        assert p.exitcode == 0
    got = sorted(q.get(timeout=10) for _ in range(2))
    assert [g[1] for g in got] == [15.0, 15.0]
    assert all(abs(g[2] - 2 * 1000 / 0.015) < 1e-6 for g in got)


def test_reference_arm_nonzero_rank_exits_without_work(monkeypatch):
    sys.path.insert(0, ROOT)
    import bench
    monkeypatch.setenv("RANK", "1")
    monkeypatch.setenv("WORLD_SIZE", "2")

    class A:
        steps, warmup = 3, 3
    assert bench.run_reference(A()) == 0


def test_single_rank_needs_no_process_group():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.max_over_ranks(None, 7.5, 1) == 7.5
    assert bench.replica_throughput(1, 2073600, 1000.0) == pytest.approx(2073600)
