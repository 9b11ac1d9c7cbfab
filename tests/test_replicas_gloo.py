"""Replica aggregation of bench.py with two gloo ranks on CPU: the timed value is all ranks'
rays over the slowest rank's time, and the reference arm does its work on rank 0 only."""
import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out):
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    sys.path.insert(0, ROOT)
    import bench
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        # rank r took (r + 1) seconds for its steps; every rank traced 1,000,000 rays per step
        slowest = bench.max_over_ranks(float(rank + 1), world, device="cpu")
        value = bench.job_value(1_000_000, 10, slowest, world)
        assert bench.dist_info() == (rank, world, rank)
        dist.barrier()
        out.put((rank, slowest, value))
    finally:
        dist.destroy_process_group()


def test_two_replicas_report_whole_job_over_slowest_rank():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=120)
    assert all(p.exitcode == 0 for p in procs), [p.exitcode for p in procs]
    got = sorted(q.get(timeout=5) for _ in range(2))
    for rank, slowest, value in got:
        assert slowest == 2.0
        assert value == pytest.approx(2 * 1_000_000 * 10 / 2.0 / 1e6)


def test_single_rank_needs_no_process_group():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.max_over_ranks(1.5, 1) == 1.5
    assert bench.job_value(7_476_193, 20, 0.066, 1) == pytest.approx(7_476_193 * 20 / 0.066 / 1e6)


def test_reference_arm_is_rank_zero_only(monkeypatch, capsys):
    sys.path.insert(0, ROOT)
    import bench
    monkeypatch.setenv("RANK", "1")
    monkeypatch.setenv("WORLD_SIZE", "2")

    class A:
        steps, warmup = 1, 0
    bench.run_reference(A())  # returns before loading anything
    assert capsys.readouterr().out == ""
