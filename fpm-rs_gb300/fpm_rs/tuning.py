"""Autotuner of the frame-engine launch grids.

Each tile size's engine launch runs G thread-block clusters that walk the
launch's tiles (fpm_set_engine_grid); G = 0 gives every tile its own
cluster, and the hardware scheduler then shares the device between the tile
sizes of a batch as clusters finish. Smaller persistent grids instead fix
how many clusters of each size are resident at once. Launches of 256-point
tiles on the single-CTA engine run a number of CTAs (fpm_set_engine_ctas)
in the same way. `autotune` times a workload under a set of candidate
tables, keeps the fastest, and `save` writes the table that every new
context applies (tuning.json next to the package).
"""

from __future__ import annotations

import ctypes as C
import json
import os
import time

from . import _native as N

TABLE_PATH = os.path.join(N.PACKAGE_ROOT, "tuning.json")
SIZES = (32, 64, 128, 256)


def max_clusters(n: int) -> int:
    """Clusters of an n x n tile's frame engine that fit on the device at once."""
    ctx = N.context()
    out = C.c_int32()
    N.check(N.library().fpm_engine_max_clusters(ctx.handle, int(n), C.byref(out)), ctx.handle)
    return out.value


def set_engine_grid(n: int, clusters: int) -> None:
    ctx = N.context()
    N.check(N.library().fpm_set_engine_grid(ctx.handle, int(n), int(clusters)), ctx.handle)


CLUSTER, SINGLE_CTA, AUTO = 0, 1, 2  # FPM_ENGINE_CLUSTER, FPM_ENGINE_SINGLE_CTA, FPM_ENGINE_AUTO


def set_engine_shape(n: int, shape: int) -> None:
    """Selects the cluster engine (0), the single-CTA engine (1, 256-point
    tiles) or the choice by launch size (2, the default for 256) for size n."""
    ctx = N.context()
    N.check(N.library().fpm_set_engine_shape(ctx.handle, int(n), int(shape)), ctx.handle)


def set_engine_ctas(n: int, ctas: int) -> None:
    """CTAs of a single-CTA engine launch of size n (0: as many as fit at once)."""
    ctx = N.context()
    N.check(N.library().fpm_set_engine_ctas(ctx.handle, int(n), int(ctas)), ctx.handle)


def apply(grid: dict, shape: dict | None = None, ctas: dict | None = None) -> None:
    """Applies {tile size: engine shape}, {tile size: clusters} of cluster
    launches and {tile size: CTAs} of single-CTA launches (0: the default)
    to the context."""
    for n, sh in (shape or {}).items():
        set_engine_shape(int(n), int(sh))
    for n in SIZES:
        set_engine_grid(n, int(grid.get(str(n), grid.get(n, 0))))
    for n, c in (ctas or {}).items():
        set_engine_ctas(int(n), int(c))


def load(path: str = TABLE_PATH) -> dict | None:
    try:
        with open(path) as handle:
            return json.load(handle)
    except (OSError, ValueError):
        return None


def _limits(sizes):
    """Residency limits: clusters of each size's cluster engine, and CTAs of
    the single-CTA engine for 256-point tiles (whose shape stays AUTO)."""
    clusters, ctas = {}, {}
    for n in sizes:
        if n == 256:
            set_engine_shape(n, CLUSTER)
            clusters[n] = max_clusters(n)
            set_engine_shape(n, AUTO)
            ctas[n] = max_clusters(n)
        else:
            clusters[n] = max_clusters(n)
    return clusters, ctas


def candidates(sizes) -> list:
    """Launch tables to try, each {"grid": clusters per size of the cluster
    engine, "ctas": CTAs per single-CTA launch}: every size at its residency
    limit, and the largest size at its limit with the others at a quarter or
    a half of theirs (so that they run beside it rather than after it); with
    256-point tiles, each of these with the single-CTA launch at 1, 3/4 and
    1/2 of the CTAs that fit (one CTA holds a whole SM's registers, so the
    SMs it leaves run the other sizes from the start)."""
    clusters, ctas = _limits(sizes)
    largest = max(sizes)
    grids = [{str(n): clusters[n] for n in sizes}]
    for share in (0.25, 0.5):
        grid = {str(n): max(1, int(clusters[n] * share)) for n in sizes}
        grid[str(largest)] = clusters[largest]
        grids.append(grid)
    out = []
    for grid in grids:
        for frac in ((1.0, 0.75, 0.5) if ctas else (1.0,)):
            out.append({"grid": grid, "ctas": {str(n): max(1, int(c * frac)) for n, c in ctas.items()}})
    return out


def autotune(algorithm, problems, *, tables=None, repeats: int = 2) -> dict:
    """Times run_batch(algorithm, problems) (results left on the device)
    under each candidate launch table and returns the fastest, with every
    measurement."""
    from .reconstruction import last_run_stats, run_batch

    sizes = sorted({p.image_shape[0] for p in problems})
    tables = tables or candidates(sizes)
    measured = []
    for table in tables:
        apply(table["grid"], None, table.get("ctas"))
        run_batch(algorithm, problems, download=False)  # warm-up under this table
        times = []
        for _ in range(repeats):
            run_batch(algorithm, problems, download=False)
            times.append(last_run_stats()["run_ms"])
        measured.append({"grid": table["grid"], "ctas": table.get("ctas", {}), "run_ms": min(times)})
    best = min(measured, key=lambda m: m["run_ms"])
    apply(best["grid"], None, best["ctas"])
    return {"grid": best["grid"], "ctas": best["ctas"], "shape": {"256": AUTO}, "measured": measured,
            "tiles": len(problems), "algorithm": type(algorithm).__name__,
            "when": time.strftime("%Y-%m-%dT%H:%M:%SZ", time.gmtime())}


def save(table: dict, path: str = TABLE_PATH) -> None:
    with open(path, "w") as handle:
        json.dump(table, handle, indent=1)
        handle.write("\n")
