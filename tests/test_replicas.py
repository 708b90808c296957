"""bench.py's multi-GPU mode runs independent replicas (the render path has
no exchange step); its only cross-rank operation is the max-over-ranks
timing reduction.  Checked here with two gloo ranks on the CPU."""

import os
import socket

import pytest


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, out):
    import torch.distributed as dist

    import bench

    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    got = bench.max_over_ranks(10.0 + 5.0 * rank, dist, "cpu")
    out.put((rank, got))
    dist.destroy_process_group()


def test_max_over_ranks_gloo_two_ranks():
    import torch.multiprocessing as mp

    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    res = dict(q.get(timeout=10) for _ in range(2))
    assert res == {0: 15.0, 1: 15.0}


def test_whole_job_time_per_step():
    import bench

    assert bench.whole_job_ms_per_step(400.0, 100, 1) == pytest.approx(4.0)
    assert bench.whole_job_ms_per_step(400.0, 100, 4) == pytest.approx(1.0)
    assert bench.max_over_ranks(3.5) == 3.5
