"""bench.py's multi-rank logic on CPU: two gloo ranks, each with its own
replica time, agree on the max-over-ranks time and on the whole-job
throughput; the reference arm runs on rank 0 only."""
import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    sys.path.insert(0, ROOT)
    import torch.distributed as dist

    import bench

    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        ms = bench.max_over_ranks(100.0 + 25.0 * rank, dist)
        v = bench.throughput(2048000, 20, world, ms)
        q.put((rank, ms, v))
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks_agree_on_time_and_throughput():
    torch = pytest.importorskip("torch")
    mp = torch.multiprocessing.get_context("spawn")
    q = mp.Queue()
    port = _free_port()
    procs = [mp.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
        assert p.exitcode == 0
    out = sorted(q.get(timeout=10) for _ in range(2))
    for rank, ms, v in out:
        assert ms == 125.0
        assert v == pytest.approx(2048000 * 20 * 2 / 0.125)


def test_single_process_helpers():
    sys.path.insert(0, ROOT)
    import bench

    assert bench.max_over_ranks(3.5) == 3.5
    assert bench.throughput(1000, 10, 1, 1000.0) == 10000.0
    c = bench.workload_config(2048000, 80, 1)
    assert c["natoms"] == 2048000 and "80^3" in c["workload"]


def test_reference_arm_runs_on_rank_zero_only(capsys):
    sys.path.insert(0, ROOT)
    import bench

    class A:
        cells, steps, warmup, precision = 80, 1, 0, "mixed"

    bench.run_reference(A(), rank=1, world=2)
    assert capsys.readouterr().out == ""


def test_side_legs_report_their_failure_in_the_line():
    """A leg beside the headline that raises leaves an error entry instead of
    ending the run; a leg that succeeds returns its result unchanged."""
    sys.path.insert(0, ROOT)
    import bench

    assert bench.guarded(lambda: {"value": 1.0}) == {"value": 1.0}

    def broken():
        raise RuntimeError("leg failed")

    assert bench.guarded(broken) == {"error": "RuntimeError: leg failed"}
    assert set(bench.ACCUMULATION) == {"mixed", "fp64"}
    assert "FP32 per thread" in bench.ACCUMULATION["mixed"]
