"""Host logic of the replicated (N > 1) bench run, on CPU with two gloo
ranks: the slowest rank's time is every rank's, and the reference arm runs
on rank 0 only (the other ranks exit without output)."""
import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, q):
    import io
    import contextlib
    sys.path.insert(0, ROOT)
    import torch.distributed as dist
    import bench
    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank, world_size=world)
    try:
        got = bench.max_over_ranks(1.5 + rank, dist)
        os.environ.update(WORLD_SIZE=str(world), RANK=str(rank), LOCAL_RANK=str(rank))
        out = io.StringIO()
        rc = None
        if rank != 0:  # rank 0 would run the CPU reference workload here
            with contextlib.redirect_stdout(out):
                rc = bench.run_reference(type("A", (), {"steps": 1, "warmup": 0})())
        q.put((rank, got, rc, out.getvalue()))
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks():
    import multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [r[1] for r in res] == [2.5, 2.5]
    assert res[1][2] == 0 and res[1][3] == ""


def test_single_process_max_is_identity():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.max_over_ranks(3.25) == 3.25
