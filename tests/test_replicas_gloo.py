"""Replica path of bench.py on CPU: two gloo ranks (world size 2).

The multi-GPU mode of this path is replicas only: every rank runs the same
workload on its own GPU with no collective on the data path; the bench only
needs a barrier around the timed region and the maximum of the ranks'
times.  These tests run that host logic (bench.Dist) as two processes on
the gloo backend, and check that the reference arm does its work on rank 0
only.
"""
from __future__ import annotations

import os
import socket
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]


def _free_port() -> int:
    with socket.socket(socket.AF_INET, socket.SOCK_STREAM) as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank: int, world: int, port: int, q):
    os.environ.update({"RANK": str(rank), "WORLD_SIZE": str(world), "LOCAL_RANK": str(rank),
                       "MASTER_ADDR": "127.0.0.1", "MASTER_PORT": str(port)})
    sys.path.insert(0, str(ROOT))
    import bench
    d = bench.Dist("gloo")
    try:
        d.barrier()
        t_max = d.max(1.5 + rank)          # per-rank "times"
        d.barrier()

        class A:
            pass
        args = A()
        ref = bench.run_reference(args, d) if rank != 0 else "skipped"
        q.put((rank, d.world, t_max, ref))
    finally:
        d.close()


def test_two_gloo_ranks_barrier_and_max():
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    results = {}
    for _ in range(2):
        rank, world, t_max, ref = q.get(timeout=120)
        results[rank] = (world, t_max, ref)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert results[0][0] == results[1][0] == 2
    # max over ranks: both ranks see the slower rank's time
    assert results[0][1] == results[1][1] == 2.5
    # the reference arm runs on rank 0 only; other ranks return nothing
    assert results[1][2] is None


def test_single_process_dist_is_identity(monkeypatch):
    monkeypatch.delenv("WORLD_SIZE", raising=False)
    monkeypatch.delenv("RANK", raising=False)
    sys.path.insert(0, str(ROOT))
    import bench
    d = bench.Dist("gloo")
    assert d.world == 1 and d.rank == 0
    d.barrier()
    assert d.max(3.25) == 3.25
    d.close()
