"""The multi-rank path of bench.py on CPU (gloo, 2 ranks): every rank learns the
slowest replica's time, the whole-job rate counts all replicas, and the
reference arm runs on rank 0 only."""
import io
import contextlib
import socket
import types

import pytest

import bench


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, q):
    import os

    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        q.put((rank, bench.max_over_ranks(1.5 + rank, world)))
        dist.barrier()
    finally:
        dist.destroy_process_group()


def test_slowest_replica_time_reaches_every_rank():
    mp = pytest.importorskip("torch.multiprocessing")
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=120)
    assert all(p.exitcode == 0 for p in procs)
    got = dict(q.get(timeout=5) for _ in range(2))
    assert got == {0: 2.5, 1: 2.5}


def test_whole_job_rate_counts_every_replica():
    one = bench.whole_job_rate(2_097_152, 0.875, 1)
    assert one == pytest.approx(2_097_152 * 5 / 0.875e-3)
    assert bench.whole_job_rate(2_097_152, 0.875, 4) == pytest.approx(4 * one)
    assert bench.max_over_ranks(3.0, 1) == 3.0


def test_reference_arm_runs_on_rank_zero_only():
    args = types.SimpleNamespace(warmup=1, steps=1, gpus=2)
    out = io.StringIO()
    with contextlib.redirect_stdout(out):
        bench.reference_arm(args, rank=1, world=2)
    assert out.getvalue() == ""
