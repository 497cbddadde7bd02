"""Multi-rank tile sharding on CPU (gloo, world size 2).

Tiles are independent, so ranks share nothing on the data path: each rank
reconstructs its own tiles and the only collectives are the barrier and the
max/sum of timings that bench.py reports. This runs those exact helpers in two
processes and checks that every rank sees the same reductions and that the
per-rank tile seeds never collide.
"""

from __future__ import annotations

import os
import socket

import pytest

torch = pytest.importorskip("torch")
import torch.multiprocessing as mp  # noqa: E402

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, queue):
    import sys

    sys.path.insert(0, ROOT)
    os.environ.update(RANK=str(rank), WORLD_SIZE=str(world), LOCAL_RANK=str(rank), MASTER_ADDR="127.0.0.1",
                      MASTER_PORT=str(port))
    import bench

    dist = bench.Dist()
    dist.barrier()
    sizes = bench.tile_sizes(64, 3)
    seed_base = 1_000_000 * dist.rank + 10_000
    seeds = [seed_base + i for i in range(len(sizes))]
    step_ms = 100.0 + 10.0 * rank
    result = dict(rank=rank, max=dist.max(step_ms), sum=dist.sum(len(sizes)), sizes=sizes, seeds=seeds)
    dist.barrier()
    queue.put(result)
    import torch.distributed as td

    td.destroy_process_group()


def test_two_rank_sharding_reductions():
    ctx = mp.get_context("spawn")
    queue = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, queue)) for r in range(2)]
    for p in procs:
        p.start()
    results = [queue.get(timeout=120) for _ in procs]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    results.sort(key=lambda r: r["rank"])
    assert all(r["max"] == 110.0 for r in results)
    assert all(r["sum"] == 128.0 for r in results)
    assert results[0]["sizes"] == results[1]["sizes"]
    assert not set(results[0]["seeds"]) & set(results[1]["seeds"])
