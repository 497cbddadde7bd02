"""Host logic of the reconstruction callbacks (src/callbacks/*.rs).

No GPU: the formatters, the PNG writer, StopOnPlateau's counter, the segment
planner, and the segmented runner driven by a fake device entry point that
records which iteration ranges were run and returns a scripted objective
sequence.
"""

from __future__ import annotations

import ctypes as C
import math

import numpy as np
import pytest

import fpm_rs as fpm
from fpm_rs import _native as N
from fpm_rs import callbacks as cbs
from fpm_rs import reconstruction as R


def _plateau_reference(objectives, patience, minimum_improvement, prior=()):
    """src/callbacks/early_stop.rs:40-67 restated: the 1-based iteration the
    run stops after, or None."""
    patience = max(patience, 1)
    minimum_improvement = max(minimum_improvement, 0.0)
    best, stale = math.inf, 0
    for value in prior:
        if best - value > minimum_improvement:
            best, stale = value, 0
        else:
            stale += 1
    for it, value in enumerate(objectives, start=len(prior) + 1):
        if best - value > minimum_improvement:
            best, stale = value, 0
        else:
            stale += 1
        if stale >= patience:
            return it
    return None


def test_rust_number_formats():
    # ryu's shortest form, as the csv crate writes f64 fields.
    cases = {0.1: "0.1", 1.0: "1.0", 100.0: "100.0", 1e16: "1e16", 1.5e20: "1.5e20", 1e-5: "0.00001",
             1.234e-5: "0.00001234", 2.5e-7: "2.5e-7", -0.0: "-0.0", 12.5: "12.5", float("nan"): "NaN",
             float("inf"): "inf", 123456789012345.6: "123456789012345.6", 0.000123: "0.000123"}
    for value, text in cases.items():
        assert cbs.shortest_float(value) == text, value
    # Rust's {:.6e}.
    assert cbs.scientific(0.001234) == "1.234000e-3"
    assert cbs.scientific(2.0) == "2.000000e0"
    assert cbs.scientific(-1.5e20) == "-1.500000e20"
    assert cbs.scientific(float("nan")) == "NaN"


def test_grayscale_png_round_trip(tmp_path):
    values = np.linspace(-1.0, 3.0, 48).reshape(6, 8)
    pixels = cbs.grayscale_pixels(values, (values.min(), values.max()))
    assert pixels[0, 0] == 0 and pixels[-1, -1] == 255
    # Rounding is half away from zero: 0.5/255 of the range maps to 1.
    assert cbs.grayscale_pixels(np.array([0.5 / 255.0]), (0.0, 1.0))[0] == 1
    assert cbs.grayscale_pixels(np.array([0.49 / 255.0, 2.0, -1.0]), (0.0, 1.0)).tolist() == [0, 255, 0]
    cbs.save_grayscale(values, tmp_path / "a.png", False)
    assert np.array_equal(cbs.read_png(tmp_path / "a.png"), pixels)
    phase = np.array([[-math.pi, 0.0, math.pi]])
    cbs.save_grayscale(phase, tmp_path / "p.png", True)
    assert cbs.read_png(tmp_path / "p.png").tolist() == [[0, 128, 255]]
    cbs.save_signed_grayscale(np.array([[-2.0, 0.0, 1.0]]), tmp_path / "s.png")
    assert cbs.read_png(tmp_path / "s.png").tolist() == [[0, 128, 191]]
    cbs.save_signed_grayscale(np.zeros((2, 2)), tmp_path / "z.png")
    assert cbs.read_png(tmp_path / "z.png").tolist() == [[128, 128], [128, 128]]


def test_constructor_rules(tmp_path):
    # python/src/reconstruction.rs:822-911: zero intervals become one.
    assert fpm.ProgressLogger(every=0).every == 1
    assert fpm.SaveImageEvery(0, tmp_path).every == 1
    assert fpm.StopOnPlateau(0).patience == 1
    assert fpm.StopOnPlateau(2, minimum_improvement=-1.0).minimum_improvement == 0.0
    with pytest.raises(OverflowError):
        fpm.ProgressLogger(every=-1)
    with pytest.raises(TypeError):
        fpm.IterationCallback(3)


@pytest.mark.parametrize("patience,minimum", [(1, 0.0), (2, 0.0), (3, 0.05), (5, 0.5)])
def test_stop_on_plateau_counter(patience, minimum):
    rng = np.random.default_rng(patience)
    objectives = list(np.cumsum(rng.normal(-0.1, 0.3, 40)) + 10.0)
    expected = _plateau_reference(objectives, patience, minimum)
    cb = fpm.StopOnPlateau(patience, minimum_improvement=minimum)
    cb.on_start(cbs.StepContext(0, None, [], None, "ap"))
    got = None
    for it, value in enumerate(objectives, start=1):
        if cb.on_iteration_end(cbs.StepContext(it, value, [], None, "ap")):
            got = it
            break
    assert got == expected
    # A resumed run rebuilds the counter from the checkpoint trace.
    prior = objectives[:7]
    cb.on_start(cbs.StepContext(7, None, [(i + 1, v, 0.0) for i, v in enumerate(prior)], None, "ap"))
    got = None
    for it, value in enumerate(objectives[7:], start=8):
        if cb.on_iteration_end(cbs.StepContext(it, value, [], None, "ap")):
            got = it
            break
    assert got == _plateau_reference(objectives[7:], patience, minimum, prior)


def test_segment_planner(tmp_path):
    plan = cbs.plan_segment
    assert plan([], 0, 50, 16) == 50
    assert plan([fpm.ProgressLogger(), fpm.CsvLogger(tmp_path / "x.csv")], 0, 50, 16) == 50
    assert plan([fpm.CheckpointEvery(7, tmp_path)], 0, 50, 16) == 7
    assert plan([fpm.CheckpointEvery(7, tmp_path)], 49, 50, 16) == 50
    assert plan([fpm.SaveImageEvery(4, tmp_path), fpm.CheckpointEvery(6, tmp_path)], 4, 50, 16) == 6
    # A stop is possible from iteration 3 on: speculate 16 iterations.
    assert plan([fpm.StopOnPlateau(3)], 0, 50, 16) == 16
    # No stop can come before iteration 40: run exactly there.
    assert plan([fpm.StopOnPlateau(40)], 0, 50, 16) == 40
    assert plan([fpm.IterationCallback(print, every=20)], 0, 50, 16) == 20
    assert plan([fpm.IterationCallback(print, every=1), fpm.CheckpointEvery(5, tmp_path)], 0, 50, 16) == 5
    assert plan([fpm.StopOnPlateau(3)], 45, 50, 16) == 50
    assert plan([fpm.StopOnPlateau(3)], 50, 50, 16) == 50


class _FakeDevice:
    """Stands in for fpm_run_batch_resumable: objective k (1-based) is
    script[k-1]; the object's first element records the iteration the
    returned state belongs to."""

    def __init__(self, script):
        self.script = script
        self.calls = []

    def fpm_run_batch_resumable(self, ctx, count, handles, params, resume, results, capture):
        p = params._obj
        start = resume[0].completed_iterations if resume is not None else 0
        end = p.iterations
        self.calls.append((start, end))
        for desc in (capture[0], results[0]):
            for k in range(end):
                desc.objectives[k] = self.script[k]
        capture[0].completed_iterations = end
        results[0].object[0] = float(end)
        capture[0].object_spectrum[0] = float(end)
        results[0].completed_iterations = end
        return 0


class _FakeProblem:
    reconstruction_shape = (4, 4)
    image_shape = (2, 2)
    name = "tile"

    class model:
        source_count = 1
        pupil_support = np.ones((2, 2), bool)
        frame_gains = None
        _background = None

    def device_handle(self):
        return C.c_void_p(1)


@pytest.fixture
def fake_device(monkeypatch):
    def install(script):
        device = _FakeDevice(script)
        monkeypatch.setattr(N, "library", lambda: device)
        monkeypatch.setattr(N, "context", lambda: type("Ctx", (), {"handle": None})())
        monkeypatch.setattr(R, "upload", lambda problems: None)
        return device
    return install


def test_runner_rolls_back_a_speculative_segment(fake_device):
    script = [10.0, 9.0, 8.5, 8.4, 8.4, 8.4, 8.4, 8.3] + [8.3] * 40
    device = fake_device(script)
    algo = fpm.AlternatingProjection(iterations=40)
    stop = _plateau_reference(script[:40], 2, 0.05)
    assert stop == 6
    result = R.run_batch(algo, [_FakeProblem()], callbacks=[fpm.StopOnPlateau(2, minimum_improvement=0.05)])[0]
    # One speculative segment of 16 iterations, then the re-run to the stop.
    assert device.calls == [(0, 16), (0, stop)]
    assert result.runtime.stopped_early and result.runtime.completed_iterations == stop
    assert [t[0] for t in result.trace] == list(range(1, stop + 1))
    assert [t[1] for t in result.trace] == script[:stop]
    assert result.object[0, 0] == stop


def test_runner_hooks_order_and_state_boundaries(fake_device, tmp_path):
    script = [float(20 - k) for k in range(12)]
    device = fake_device(script)
    seen = []
    states = []

    class Probe(cbs.Callback):
        def _next_state(self, current):
            return cbs._next_multiple(current, 4)

        def on_start(self, context):
            seen.append(("start", context.iteration))

        def on_iteration_end(self, context):
            seen.append(("end", context.iteration, context.objective))
            if context.iteration % 4 == 0:
                states.append(context.object[0, 0].real)
            return False

        def on_finish(self, result):
            seen.append(("finish", result.runtime.completed_iterations))

    csv = tmp_path / "history.csv"
    calls = []
    result = R.run_batch(fpm.AlternatingProjection(iterations=10), [_FakeProblem()], callbacks=[
        Probe(), fpm.CsvLogger(csv), fpm.IterationCallback(lambda m: calls.append(dict(m)), every=3)])[0]
    assert device.calls == [(0, 4), (4, 8), (8, 10)]
    assert states == [4.0, 8.0]
    assert seen[0] == ("start", 0) and seen[-1] == ("finish", 10)
    assert [s[1] for s in seen[1:-1]] == list(range(1, 11))
    assert [c["iteration"] for c in calls] == [3, 6, 9]
    assert set(calls[0]) == {"iteration", "objective", "algorithm_metrics", "problem_name",
                             "physical_illumination_calibration"}
    assert calls[0]["problem_name"] == "tile" and calls[0]["objective"] == script[2]
    lines = csv.read_text().splitlines()
    assert lines[0] == "iteration,objective,elapsed_seconds"
    assert [line.split(",")[:2] for line in lines[1:]] == [[str(k), cbs.shortest_float(script[k - 1])]
                                                           for k in range(1, 11)]
    assert not result.runtime.stopped_early and result.runtime.completed_iterations == 10


def test_iteration_callback_stop_semantics(fake_device):
    script = [5.0] * 30
    # None and truthy values continue; False (or another falsy value) stops.
    for response, stop in ((None, None), (1, None), (False, 6), (0, 6), ("", 6)):
        device = fake_device(script)
        cb = fpm.IterationCallback(lambda m, r=response: r if m["iteration"] >= 6 else None, every=3)
        result = R.run_batch(fpm.AlternatingProjection(iterations=12), [_FakeProblem()], callbacks=[cb])[0]
        # A stop is possible at every third iteration: the runner speculates
        # past it and re-runs to the stop when one comes.
        if stop is None:
            assert device.calls == [(0, 12)]
            assert result.runtime.completed_iterations == 12
        else:
            assert device.calls == [(0, 12), (0, 6)]
            assert result.runtime.completed_iterations == stop and result.runtime.stopped_early


def test_progress_logger_lines(fake_device, capsys):
    fake_device([0.5, 0.25, 0.125, 0.0625])
    R.run_batch(fpm.AlternatingProjection(iterations=4), [_FakeProblem()], callbacks=[fpm.ProgressLogger(every=2)])
    err = capsys.readouterr().err.splitlines()
    assert err == ["iteration     2: objective 2.500000e-1", "iteration     4: objective 6.250000e-2"]


def test_checkpoint_every_with_a_resumed_trace(fake_device, tmp_path):
    device = fake_device([3.0, 2.0, 1.0, 1.0, 1.0, 1.0])
    R.run_batch(fpm.AlternatingProjection(iterations=6), [_FakeProblem()],
                callbacks=[fpm.CheckpointEvery(2, tmp_path / "cp")])
    assert device.calls == [(0, 2), (2, 4), (4, 6)]
    saved = sorted(p.name for p in (tmp_path / "cp").iterdir())
    assert saved == ["checkpoint_00002.json", "checkpoint_00004.json", "checkpoint_00006.json"]
    cp = fpm.ReconstructionCheckpoint.load(tmp_path / "cp" / "checkpoint_00004.json")
    assert cp.completed_iterations == 4 and cp.objectives == [3.0, 2.0, 1.0, 1.0]
    assert cp.object_spectrum[0, 0] == 4.0
