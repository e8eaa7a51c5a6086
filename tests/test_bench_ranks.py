"""The bench's multi-rank bookkeeping on CPU (gloo, world size 2): replicas
only -- each rank times its own copy of the workload, the job's time is the
slowest rank's and its throughput counts every rank's units; the reference
arm prints from rank 0 alone."""
import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    import torch.distributed as dist

    import bench
    dist.init_process_group("gloo", init_method="tcp://127.0.0.1:%d" % port, rank=rank, world_size=world)
    ms = bench.max_over_ranks(10.0 + 5.0 * rank, dist, "cpu")  # rank 1 is the slow one
    rate = bench.job_rate(1000.0, 20, world, ms / 1e3)
    out.put((rank, ms, rate))
    dist.barrier()
    dist.destroy_process_group()


def test_max_over_ranks_and_job_rate_gloo():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    # both ranks see the slowest rank's 15 ms; the job did 2 x 1000 x 20 units
    assert [r[1] for r in res] == [15.0, 15.0]
    assert all(abs(r[2] - 2 * 1000 * 20 / 0.015) < 1e-6 for r in res)


def test_alone_needs_no_process_group():
    import bench
    assert bench.max_over_ranks(3.5, None, "cpu") == 3.5
    assert bench.job_rate(10.0, 3, 1, 2.0) == 15.0


def test_reference_arm_prints_from_rank_0_only(monkeypatch, capsys):
    import bench
    monkeypatch.setenv("RANK", "1")
    monkeypatch.setenv("WORLD_SIZE", "2")
    monkeypatch.setattr(sys, "argv", ["bench.py", "--impl", "reference", "--gpus", "2", "--steps", "1", "--warmup", "0"])
    bench.run_reference(bench.parse())
    assert capsys.readouterr().out == ""
