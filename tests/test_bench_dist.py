"""The multi-rank form of ``bench.py`` on CPU ranks (gloo, world size 2).

The path does not shard: every rank runs an independent replica of the step,
and the job's step time is the slowest replica's (``_max_over_ranks``), which
rank 0 prints.  The reference arm runs on rank 0 alone; the other ranks
return without work.  Ranks are separate processes started with ``spawn``
and meet at 127.0.0.1.
"""

from __future__ import annotations

import multiprocessing as mp
import os
import socket
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank: int, world: int, port: int, queue) -> None:
    os.environ.update(RANK=str(rank), WORLD_SIZE=str(world), LOCAL_RANK=str(rank), MASTER_ADDR="127.0.0.1",
                      MASTER_PORT=str(port))
    sys.path.insert(0, str(ROOT))
    import torch
    import torch.distributed as dist

    import bench

    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        ws, r, local = bench._dist()
        slowest = bench._max_over_ranks(0.5 + rank, torch.device("cpu"))
        args = type("A", (), {"workload": "siam10", "steps": 1, "warmup": 0})()
        ref = bench.run_reference(args) if rank != 0 else "rank 0 runs it"
        dist.barrier()
        queue.put((rank, ws, r, local, slowest, ref))
    finally:
        dist.destroy_process_group()


def test_replicas_report_the_slowest_rank_and_rank0_alone_runs_the_reference():
    pytest.importorskip("torch.distributed")
    ctx = mp.get_context("spawn")
    queue = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, queue)) for r in range(2)]
    for p in procs:
        p.start()
    results = sorted(queue.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [r[:4] for r in results] == [(0, 2, 0, 0), (1, 2, 1, 1)]
    assert all(r[4] == 1.5 for r in results)
    assert results[1][5] is None
