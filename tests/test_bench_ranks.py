"""Multi-rank logic of bench.py on CPU: world size 2 over gloo (127.0.0.1).

Each rank reports its own step time; the job's time is the slowest rank's, and the
whole-job rate counts every rank's units over that time.  The reference arm runs on
rank 0 only; other ranks return 0 without output.
"""
import contextlib
import io
import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, out_q):
    os.environ.update({"MASTER_ADDR": "127.0.0.1", "MASTER_PORT": str(port), "RANK": str(rank),
                       "WORLD_SIZE": str(world), "LOCAL_RANK": str(rank)})
    sys.path.insert(0, ROOT)
    import bench
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        r, w, loc = bench.dist_env()
        my_ms = 100.0 + 50.0 * rank                     # rank 1 is the slow one
        total_ms = bench.max_over_ranks(my_ms, dist, "cpu")
        rate = bench.job_rate(1000, 4, w, total_ms)
        dist.barrier()
        # the reference arm: rank 0 alone runs; others exit 0 silently
        buf = io.StringIO()
        rc = None
        if rank != 0:
            class A:
                n, steps, warmup, ref_seconds = 256, 1, 0, 0.01
            with contextlib.redirect_stdout(buf):
                rc = bench.run_reference(A())
        out_q.put((rank, r, w, loc, total_ms, rate, rc, buf.getvalue()))
    finally:
        dist.destroy_process_group()


def test_two_ranks_max_time_and_job_rate():
    world = 2
    ctx = mp.get_context("spawn")
    q = ctx.SimpleQueue()
    mp.start_processes(_worker, args=(world, _free_port(), q), nprocs=world, join=True, start_method="spawn")
    res = sorted(q.get() for _ in range(world))
    for rank, r, w, loc, total_ms, rate, rc, out in res:
        assert (r, w, loc) == (rank, world, rank)
        assert total_ms == 150.0                       # slowest rank's time on every rank
        assert rate == pytest.approx(1000 * 4 * world / 0.150)
        if rank != 0:
            assert rc == 0 and out == ""


def test_single_rank_helpers():
    import bench
    assert bench.max_over_ranks(12.5, None, "cpu") == 12.5
    assert bench.job_rate(10, 2, 1, 1000.0) == pytest.approx(20.0)
