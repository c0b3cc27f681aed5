"""The benchmark's multi-process host logic on CPU ranks (gloo, world size 2).

The timed path runs one process per GPU.  The whole job's time is the
slowest rank's (`max_over_ranks`), every rank's units count toward the
value, and in the reference arm rank 0 alone works and prints.  Nothing
here touches a GPU.
"""
from __future__ import annotations

import io
import os
import socket
import sys
from contextlib import redirect_stdout
from pathlib import Path

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402

ROOT = Path(__file__).resolve().parents[1]


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank: int, world: int, port: int, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    sys.path.insert(0, str(ROOT))
    import bench
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        # rank r took r + 1.5 s: the job took the slowest rank's 2.5 s
        t = bench.max_over_ranks(rank + 1.5, world)
        # the reference arm: rank 0 alone runs (here stopped before any work
        # by a rank other than 0)
        buf = io.StringIO()
        if rank != 0:
            with redirect_stdout(buf):
                bench.run_reference(None, rank, world)
        out.put((rank, t, buf.getvalue()))
    finally:
        dist.destroy_process_group()


def test_max_over_ranks_and_reference_arm_on_two_gloo_ranks():
    ctx = mp.get_context("spawn")
    out = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, out)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(out.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [r for r, _, _ in res] == [0, 1]
    assert all(t == 2.5 for _, t, _ in res)
    assert res[1][2] == ""  # rank 1 of the reference arm printed nothing


def test_single_process_keeps_its_time():
    sys.path.insert(0, str(ROOT))
    import bench
    assert bench.max_over_ranks(1.25, 1) == 1.25
