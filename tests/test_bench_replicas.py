"""bench.py on N GPUs runs N independent replicas (the path has no exchange
step): each rank times its own series, the job's time is the slowest rank's,
and the value counts every rank's units.  Checked here with two gloo ranks on
the CPU; the reference arm runs on rank 0 only."""
import os
import socket
import sys

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, REPO)


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    import torch.distributed as dist

    import bench

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        # rank r took 10 + r ms for the step, 20 - r ms end to end
        got = bench.reduce_max_over_ranks([10.0 + rank, 20.0 - rank, 5.0], dist, "cpu")
        out.put((rank, got))
    finally:
        dist.destroy_process_group()


def test_two_replicas_take_the_slowest_rank():
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
    got = dict(q.get(timeout=10) for _ in range(2))
    assert got[0] == got[1] == [11.0, 20.0, 5.0]


def test_job_throughput_counts_every_replica():
    import bench

    one = bench.job_throughput(1.92e10, 3, 1, 30.0)
    assert one == pytest.approx(1.92e10 * 3 / 0.030 / 1e9)
    assert bench.job_throughput(1.92e10, 3, 4, 30.0) == pytest.approx(4 * one)


def test_single_rank_needs_no_process_group():
    import bench

    assert bench.reduce_max_over_ranks([1.5, 2.5], None, "cpu") == [1.5, 2.5]


def test_reference_arm_runs_on_rank_zero_only(capsys):
    import bench

    assert bench.run_reference(None, 1, 2) is None
    assert capsys.readouterr().out == ""
