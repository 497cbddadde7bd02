"""The launch-table autotuner's host logic (fpm_rs.tuning), with the device
queries replaced by fixed residency limits: the candidate tables it times,
the order in which a table is applied, and the committed table's form."""

from __future__ import annotations

import json
import os

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CLUSTER_LIMITS = {32: 1064, 64: 304, 128: 74, 256: 14}
SINGLE_CTA_LIMIT = 152


@pytest.fixture()
def tuning(native_library, monkeypatch):
    import fpm_rs.tuning as T

    calls = []
    shapes = {}

    def set_shape(n, shape):
        shapes[n] = shape
        calls.append(("shape", n, shape))

    def max_clusters(n):
        return SINGLE_CTA_LIMIT if shapes.get(n, T.CLUSTER) != T.CLUSTER else CLUSTER_LIMITS[n]

    monkeypatch.setattr(T, "set_engine_shape", set_shape)
    monkeypatch.setattr(T, "max_clusters", max_clusters)
    monkeypatch.setattr(T, "set_engine_grid", lambda n, g: calls.append(("grid", n, g)))
    monkeypatch.setattr(T, "set_engine_ctas", lambda n, c: calls.append(("ctas", n, c)))
    T.calls = calls
    yield T
    del T.calls


def test_candidates_sweep_grids_and_single_cta_launch_sizes(tuning):
    tables = tuning.candidates([32, 64, 128, 256])
    # Three cluster-grid tables (all at the limit; the others at a quarter
    # or a half beside the largest at its limit), each with the single-CTA
    # launch at 1, 3/4 and 1/2 of the CTAs that fit.
    assert len(tables) == 9
    assert tables[0] == {"grid": {str(n): CLUSTER_LIMITS[n] for n in CLUSTER_LIMITS}, "ctas": {"256": 152}}
    assert sorted({t["ctas"]["256"] for t in tables}) == [76, 114, 152]
    assert all(t["grid"]["256"] == CLUSTER_LIMITS[256] for t in tables)
    quarters = [t for t in tables if t["grid"]["32"] == 266]
    assert len(quarters) == 3 and all(t["grid"]["128"] == 18 for t in quarters)


def test_candidates_without_256_point_tiles_have_no_single_cta_sweep(tuning):
    tables = tuning.candidates([32, 128])
    assert len(tables) == 3
    assert all(t["ctas"] == {} for t in tables)


def test_apply_sets_shapes_then_grids_then_ctas(tuning):
    tuning.calls.clear()
    tuning.apply({"32": 5, "256": 3}, {256: tuning.AUTO}, {256: 100})
    kinds = [c[0] for c in tuning.calls]
    assert kinds == ["shape"] + ["grid"] * 4 + ["ctas"]
    assert ("grid", 32, 5) in tuning.calls and ("grid", 64, 0) in tuning.calls
    assert tuning.calls[-1] == ("ctas", 256, 100)


def test_committed_table_names_every_size():
    with open(os.path.join(ROOT, "fpm-rs_gb300", "tuning.json")) as handle:
        table = json.load(handle)
    assert set(table["grid"]) == {"32", "64", "128", "256"}
    assert all(isinstance(v, int) and v >= 0 for v in table["grid"].values())
    assert set(table.get("shape", {})) <= {"256"} and set(table.get("ctas", {})) <= {"256"}
    # Every candidate the tuner measured is recorded with its time.
    assert table["measured"] and all(m["run_ms"] > 0 for m in table["measured"])
    best = min(table["measured"], key=lambda m: m["run_ms"])
    assert best["grid"] == table["grid"] and best.get("ctas", {}) == table.get("ctas", {})
