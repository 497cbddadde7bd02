"""Captured run plans (fpm_plan_create / _launch / _wait / _collect): a run
recorded once as a CUDA graph and replayed gives the same bits as
fpm_run_batch on the same problems, replay after replay, for the one-launch
engine path and for the per-batch launch loops of the GD regulariser and
illumination recovery; the plan holds its problems until it is closed."""

from __future__ import annotations

import numpy as np
import pytest

import helpers

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def fpm(native_library):
    import fpm_rs

    return fpm_rs


def _problems(fpm, specs):
    out = []
    for side, n, seed in specs:
        model, omodel, data, truth, gains = helpers.simulated(fpm, side, n, seed=seed, photons=1e4)
        out.append(fpm.ReconstructionProblem(data, model))
    return out


def _same(a, b):
    assert np.array_equal(a.object, b.object)
    assert np.array_equal(a.object_spectrum, b.object_spectrum)
    assert np.array_equal(a.recovered_pupil, b.recovered_pupil)
    assert [t[1] for t in a.trace] == [t[1] for t in b.trace]


@pytest.mark.parametrize("make", [
    lambda fpm: fpm.Mpie(iterations=3, momentum_interval=7),
    lambda fpm: fpm.AlternatingProjection(iterations=2),
    lambda fpm: fpm.Epry(iterations=2),
    lambda fpm: fpm.GradientDescent(iterations=2, batch_size=4, object_tv=1e-3),
    lambda fpm: fpm.GradientDescent(iterations=1, recover_illumination=True),
], ids=["mpie", "ap", "epry", "gd_tv", "gd_illumination"])
def test_replays_equal_run_batch(fpm, make):
    problems = _problems(fpm, [(5, 64, 11), (3, 32, 12), (5, 128, 13), (3, 32, 14)])
    algo = make(fpm)
    expected = fpm.run_batch(algo, problems)
    plan = fpm.capture_batch(algo, problems)
    try:
        for _ in range(2):
            plan.run()
            for a, b in zip(expected, plan.results()):
                _same(a, b)
        stats = fpm.last_run_stats()
        assert stats["engine_launches"] >= 1 and stats["run_ms"] > 0
    finally:
        plan.close()


def test_queued_replays_and_held_problems(fpm):
    problems = _problems(fpm, [(3, 32, 21), (5, 64, 22)])
    algo = fpm.Mpie(iterations=2)
    plan = fpm.capture_batch(algo, problems)
    try:
        for _ in range(3):
            plan.launch()
        plan.wait()
        first = plan.results()
        with pytest.raises(fpm.InvalidParameterError):
            fpm.run_batch(algo, problems)
        with pytest.raises(fpm.InvalidParameterError):
            problems[0].release()
    finally:
        plan.close()
    again = fpm.run_batch(algo, problems)
    for a, b in zip(first, again):
        _same(a, b)
