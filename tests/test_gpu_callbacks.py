"""Callbacks on the device path (src/callbacks/*.rs, src/reconstruction/runner.rs:76-285).

A run stopped by a callback returns the state an uninterrupted run of that
many iterations returns, bit for bit (the resumable device path restores the
complex64 state exactly; EPRY re-canonicalises a restored pair, within 1e-5
NRMSE). Image callbacks write what the result arrays quantise to, and the
residual images follow the oracle's forward model.
"""

from __future__ import annotations

import math

import numpy as np
import pytest

import helpers
import oracle

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def fpm(native_library):
    import fpm_rs

    return fpm_rs


def _plateau_stop(objectives, patience, minimum_improvement):
    """src/callbacks/early_stop.rs:53-67 restated."""
    best, stale = math.inf, 0
    for it, value in enumerate(objectives, start=1):
        if best - value > minimum_improvement:
            best, stale = value, 0
        else:
            stale += 1
        if stale >= patience:
            return it
    return None


@pytest.mark.parametrize("name,make", [
    ("ap", lambda fpm, k: fpm.AlternatingProjection(iterations=k)),
    ("mpie", lambda fpm, k: fpm.Mpie(iterations=k, momentum_interval=5)),
    ("gd", lambda fpm, k: fpm.GradientDescent(iterations=k, batch_size=4)),
])
def test_stop_on_plateau_returns_the_state_of_the_stopping_iteration(fpm, name, make):
    model, omodel, data, truth, gains = helpers.simulated(fpm, 5, 64, seed=71, photons=1e4)
    problem = fpm.ReconstructionProblem(data, model)
    total = 40
    straight = make(fpm, total).run(problem)
    objectives = [t[1] for t in straight.trace]
    # The smallest threshold from a ladder at which the run stops midway.
    patience, stop, threshold = 2, None, None
    for fraction in (1e-4, 3e-4, 1e-3, 3e-3, 1e-2, 3e-2, 1e-1):
        threshold = fraction * objectives[0]
        stop = _plateau_stop(objectives, patience, threshold)
        if stop is not None and 3 <= stop < total - 2:
            break
    assert stop is not None and 3 <= stop < total - 2, objectives
    stopped = make(fpm, total).run(problem, callbacks=[fpm.StopOnPlateau(patience, minimum_improvement=threshold)])
    assert stopped.runtime.stopped_early and stopped.runtime.completed_iterations == stop
    assert [t[1] for t in stopped.trace] == objectives[:stop]
    short = make(fpm, stop).run(problem)
    assert np.array_equal(stopped.object, short.object)
    assert np.array_equal(stopped.recovered_pupil, short.recovered_pupil)


def test_iteration_callback_stops_and_sees_each_iteration(fpm):
    model, omodel, data, truth, gains = helpers.simulated(fpm, 5, 32, seed=72, photons=1e4)
    problem = fpm.ReconstructionProblem(data, model, name="tile-7")
    seen = []

    def hook(values):
        seen.append(dict(values))
        return values["iteration"] < 9

    result = fpm.Mpie(iterations=30, momentum_interval=4).run(problem, callbacks=[fpm.IterationCallback(hook, every=3)])
    assert [v["iteration"] for v in seen] == [3, 6, 9]
    assert all(v["problem_name"] == "tile-7" for v in seen)
    assert result.runtime.completed_iterations == 9 and result.runtime.stopped_early
    straight = fpm.Mpie(iterations=9, momentum_interval=4).run(problem)
    assert np.array_equal(result.object, straight.object)
    assert [v["objective"] for v in seen] == [straight.trace[k - 1][1] for k in (3, 6, 9)]


def test_progress_and_csv_follow_the_trace(fpm, tmp_path, capsys):
    from fpm_rs.callbacks import scientific, shortest_float

    model, omodel, data, truth, gains = helpers.simulated(fpm, 3, 32, seed=73)
    problem = fpm.ReconstructionProblem(data, model)
    path = tmp_path / "history.csv"
    result = fpm.Epry(iterations=6).run(problem, callbacks=[fpm.ProgressLogger(every=2), fpm.CsvLogger(path)])
    # Objective-only hooks do not split the device run.
    plain = fpm.Epry(iterations=6).run(problem)
    assert np.array_equal(result.object, plain.object)
    rows = [line.split(",") for line in path.read_text().splitlines()]
    assert rows[0] == ["iteration", "objective", "elapsed_seconds"]
    assert [r[:2] for r in rows[1:]] == [[str(it), shortest_float(obj)] for it, obj, _ in result.trace]
    elapsed = [float(r[2]) for r in rows[1:]]
    assert elapsed == sorted(elapsed) and elapsed[-1] <= result.runtime.elapsed_seconds + 1e-9
    err = capsys.readouterr().err.splitlines()
    assert err == [f"iteration {it:>5}: objective {scientific(result.trace[it - 1][1])}" for it in (2, 4, 6)]


def test_image_callbacks_write_the_state_of_their_iteration(fpm, tmp_path):
    from fpm_rs.callbacks import grayscale_pixels, read_png

    model, omodel, data, truth, gains = helpers.simulated(fpm, 3, 32, seed=74, pupil_seed=5)
    problem = fpm.ReconstructionProblem(data, model)
    callbacks = [fpm.SaveImageEvery(2, tmp_path / "img"), fpm.SavePupilEvery(4, tmp_path / "pupil"),
                 fpm.SaveResidualsEvery(4, tmp_path / "res")]
    result = fpm.Mpie(iterations=4, momentum_interval=3).run(problem, callbacks=callbacks)
    two = fpm.Mpie(iterations=2, momentum_interval=3).run(problem)
    for it, state in ((2, two), (4, result)):
        amp = np.abs(state.object)
        assert np.array_equal(read_png(tmp_path / "img" / f"amplitude_{it:05d}.png"),
                              grayscale_pixels(amp, (amp.min(), amp.max())))
        assert np.array_equal(read_png(tmp_path / "img" / f"phase_{it:05d}.png"),
                              grayscale_pixels(np.angle(state.object), (-math.pi, math.pi)))
    pupil = result.recovered_pupil
    assert np.array_equal(read_png(tmp_path / "pupil" / "pupil_amplitude_00004.png"),
                          grayscale_pixels(np.abs(pupil), (np.abs(pupil).min(), np.abs(pupil).max())))
    assert sorted(p.name for p in (tmp_path / "pupil").iterdir()) == ["pupil_amplitude_00004.png",
                                                                       "pupil_phase_00004.png"]
    # Residuals against the oracle's FP64 forward model of the returned state.
    sim = dict(omodel)
    sim["pupil"] = pupil
    predicted = oracle.forward_stack(oracle.Problem(sim, None), oracle.object_spectrum(result.object))
    residual = predicted - data
    names = sorted(p.name for p in (tmp_path / "res").iterdir())
    assert names == [f"residual_00004_frame_{f:05d}.png" for f in range(model.frame_count)]
    for f in range(model.frame_count):
        extent = max(np.abs(residual[f]).max(), np.finfo(np.float64).eps)
        expected = grayscale_pixels(residual[f], (-extent, extent)).astype(int)
        got = read_png(tmp_path / "res" / f"residual_00004_frame_{f:05d}.png").astype(int)
        # The device forward model is FP32: a pixel may land one level over.
        assert np.abs(got - expected).max() <= 1
        assert np.mean(got != expected) < 0.02


def test_checkpoint_every_with_stop(fpm, tmp_path):
    """CheckpointEvery and StopOnPlateau together: checkpoints stop with the run."""
    model, omodel, data, truth, gains = helpers.simulated(fpm, 5, 32, seed=75, photons=1e4)
    problem = fpm.ReconstructionProblem(data, model)
    straight = fpm.AlternatingProjection(iterations=30).run(problem)
    objectives = [t[1] for t in straight.trace]
    stop = _plateau_stop(objectives, 1, 0.0)
    result = fpm.AlternatingProjection(iterations=30).run(problem, callbacks=[
        fpm.CheckpointEvery(4, tmp_path), fpm.StopOnPlateau(1)])
    expected_stop = stop if stop is not None else 30
    assert result.runtime.completed_iterations == expected_stop
    saved = sorted(p.name for p in tmp_path.iterdir())
    assert saved == [f"checkpoint_{k:05d}.json" for k in range(4, expected_stop + 1, 4)]
