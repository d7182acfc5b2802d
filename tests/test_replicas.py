"""The N > 1 path of bench.py on CPU: N independent replicas (no data-path
collective), the job time is the slowest replica's, the whole-job rate is
N x per-replica bytes / that time.  Two gloo ranks on 127.0.0.1."""
from __future__ import annotations

import os
import socket
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    sys.path.insert(0, str(ROOT))
    import torch.distributed as dist

    import bench

    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        local = 1.0 + rank  # rank 1 is the slow replica
        ms = bench.max_over_ranks(local, world, "cpu")
        out.put((rank, ms, bench.job_rate(world, 2e9, ms)))
    finally:
        dist.destroy_process_group()


def test_two_replicas_report_the_slowest():
    mp = pytest.importorskip("torch.multiprocessing")
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    got = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [g[1] for g in got] == [2.0, 2.0]
    assert all(abs(g[2] - 2 * 2e9 / 2e-3 / 1e9) < 1e-9 for g in got)  # 2000 GB/s for the job
