"""The serving loop (fpm_server_*, Python Server): requests that arrive
while others run are admitted and overlap them on the device, each result
is bit-identical to the same request run alone, admission follows the HBM
budget, and a full queue sheds requests."""

from __future__ import annotations

import numpy as np
import pytest

import helpers

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def fpm(native_library):
    import fpm_rs

    return fpm_rs


def _problem(fpm, side, n, seed):
    model, omodel, data, truth, gains = helpers.simulated(fpm, side, n, seed=seed, photons=1e4)
    return fpm.ReconstructionProblem(data, model)


def _same(a, b):
    assert np.array_equal(a.object, b.object)
    assert np.array_equal(a.object_spectrum, b.object_spectrum)
    assert np.array_equal(a.recovered_pupil, b.recovered_pupil)
    assert [t[1] for t in a.trace] == [t[1] for t in b.trace]


def test_requests_arriving_during_others_overlap_and_match_solo_runs(fpm):
    specs = [(fpm.Mpie(iterations=12), (15, 256, 31)), (fpm.Mpie(iterations=4), (5, 64, 32)),
             (fpm.AlternatingProjection(iterations=5), (3, 32, 33)), (fpm.Mpie(iterations=4), (5, 64, 34)),
             (fpm.GradientDescent(iterations=3), (5, 128, 35))]
    problems = [_problem(fpm, *spec) for _, spec in specs]
    solo = [fpm.run_batch(algo, [fpm.ReconstructionProblem(p.measurements, p.model)])[0]
            for (algo, _), p in zip(specs, problems)]
    with fpm.Server(hbm_budget_gb=150, max_batch=8, batch_window_ms=10.0) as server:
        first = server.submit(specs[0][0], problems[0])
        later = [server.submit(algo, p) for (algo, _), p in zip(specs[1:], problems[1:])]
        requests = [first] + later
        results = [r.wait() for r in requests]
        infos = [r.info() for r in requests]
        stats = server.stats()
    for got, want in zip(results, solo):
        _same(got, want)
    head = infos[0]
    for info in infos[1:]:
        assert info["submit_ms"] < head["done_ms"]  # arrived while the first request ran
        assert info["start_ms"] < head["done_ms"]   # and went on the device beside it
    for info in infos:
        assert info["submit_ms"] <= info["admit_ms"] <= info["start_ms"] <= info["done_ms"]
    assert stats["completed"] == len(specs) and stats["rejected"] == 0
    # The two equal-parameter 64-point requests share one batch.
    assert stats["batches"] == len(specs) - 1


def test_budget_admits_one_request_at_a_time(fpm):
    problems = [_problem(fpm, 5, 64, 41 + k) for k in range(3)]
    algo = fpm.Mpie(iterations=3)
    solo = [fpm.run_batch(algo, [fpm.ReconstructionProblem(p.measurements, p.model)])[0] for p in problems]
    with fpm.Server() as server:
        footprint = server.submit(algo, problems[0]).info()["footprint_bytes"]
    budget = 1.5 * footprint  # room for one of these requests at a time
    with fpm.Server(hbm_budget_gb=budget / 1e9, max_batch=8, batch_window_ms=0.0) as server:
        requests = [server.submit(algo, p) for p in problems]
        results = [r.wait() for r in requests]
        infos = sorted((r.info() for r in requests), key=lambda i: i["admit_ms"])
        peak = server.stats()["peak_bytes"]
    for got, want in zip(results, solo):
        _same(got, want)
    for prev, nxt in zip(infos, infos[1:]):
        assert nxt["admit_ms"] >= prev["done_ms"]
    assert footprint <= peak <= budget


def test_full_queue_sheds_and_oversized_requests_are_refused(fpm):
    p = _problem(fpm, 3, 32, 51)
    algo = fpm.AlternatingProjection(iterations=2)
    with fpm.Server(max_batch=4, batch_window_ms=300.0, max_queue=1) as server:
        first = server.submit(algo, p)
        with pytest.raises(fpm.ServerBusyError):
            server.submit(algo, p)
        assert first.wait().object.shape == p.reconstruction_shape
        assert server.stats()["rejected"] == 1
    with fpm.Server(hbm_budget_gb=1e-6) as server:
        with pytest.raises(fpm.InvalidParameterError):
            server.submit(algo, p)
