"""Multi-rank tile sharding on CPU (gloo, world size 2).

Tiles are independent, so ranks share nothing on the data path: each rank
reconstructs its own tiles and the only collectives are the barrier and the
max/sum of timings that bench.py reports. These tests run those exact
helpers in two processes: every rank sees the same reductions, the per-rank
tile seeds never collide, and each rank reconstructs its own tiles (the
FP64 oracle standing in for the device) with results identical to a single
process reconstructing the same tiles.
"""

from __future__ import annotations

import hashlib
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


def _tile_digests(fpm, seed_base: int, sizes) -> list:
    """SHA-256 of each tile's reconstructed object: the oracle's forward
    stack of the tile's seeded object, then two AP iterations."""
    import helpers
    import oracle
    import workloads as W

    out = []
    for i, n in enumerate(sizes):
        model, omodel = helpers.planar_model(fpm, 3, n)
        truth = W.smooth_random_object(model.reconstruction_shape, seed_base + i)
        intensity = oracle.forward_stack(oracle.Problem(omodel, None), oracle.object_spectrum(truth), workers=1)
        result = oracle.run(oracle.Problem(omodel, intensity), "ap", iterations=2)
        out.append(hashlib.sha256(result["object"].tobytes()).hexdigest())
    return out


def _reconstruct_worker(rank, world, port, queue):
    import sys

    for path in (ROOT, os.path.join(ROOT, "tests"), os.path.join(ROOT, "oracle"), os.path.join(ROOT, "fpm-rs_gb300")):
        sys.path.insert(0, path)
    os.environ.update(RANK=str(rank), WORLD_SIZE=str(world), LOCAL_RANK=str(rank), MASTER_ADDR="127.0.0.1",
                      MASTER_PORT=str(port))
    import bench
    import fpm_rs

    dist = bench.Dist()
    sizes = [32, 32, 32]
    digests = _tile_digests(fpm_rs, bench.rank_seed_base(dist.rank), sizes)
    gathered = dist.gather(digests)
    total = dist.sum(len(sizes))
    dist.barrier()
    queue.put(dict(rank=rank, digests=digests, gathered=gathered, total=total))
    import torch.distributed as td

    td.destroy_process_group()


def test_two_ranks_reconstruct_their_own_tiles(native_library, oracle_module):
    import bench
    import fpm_rs

    ctx = mp.get_context("spawn")
    queue = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_reconstruct_worker, args=(r, 2, port, queue)) for r in range(2)]
    for p in procs:
        p.start()
    results = [queue.get(timeout=300) for _ in procs]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    results.sort(key=lambda r: r["rank"])
    # Every rank sees every rank's results, in rank order, and the tile total.
    assert results[0]["gathered"] == results[1]["gathered"] == [results[0]["digests"], results[1]["digests"]]
    assert all(r["total"] == 6.0 for r in results)
    # Disjoint tiles: no result appears on both ranks.
    assert not set(results[0]["digests"]) & set(results[1]["digests"])
    # Each rank's results are those of one process reconstructing its tiles.
    for r in results:
        assert r["digests"] == _tile_digests(fpm_rs, bench.rank_seed_base(r["rank"]), [32, 32, 32])
