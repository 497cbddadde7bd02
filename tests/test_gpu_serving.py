"""Serving entry points: submitted jobs (fpm_run_batch_submit,
fpm_spectral_run_batch_submit, fpm_job_poll / fpm_job_wait) give the same
bits as the blocking batch calls, run side by side, and keep their problems
reserved until they finish."""

from __future__ import annotations

import time

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


def test_submitted_batch_equals_blocking_batch(fpm):
    problems = _problems(fpm, [(3, 32, 1), (5, 64, 2), (3, 32, 3)])
    algo = fpm.Mpie(iterations=4, momentum_interval=5)
    blocking = fpm.run_batch(algo, problems)
    job = fpm.submit_batch(algo, problems)
    got = job.wait()
    assert job.done()
    for a, b in zip(blocking, got):
        np.testing.assert_array_equal(a.object_spectrum, b.object_spectrum)
        np.testing.assert_array_equal(a.object, b.object)
        np.testing.assert_array_equal([t[1] for t in a.trace], [t[1] for t in b.trace])
    stats = job.stats()
    assert stats["engine_launches"] == 2 and stats["kernel_launches"] > 2


def test_jobs_in_flight_side_by_side_and_reserved(fpm):
    first = _problems(fpm, [(5, 64, 4), (3, 32, 5)])
    second = _problems(fpm, [(3, 128, 6), (3, 32, 7)])
    algo = fpm.GradientDescent(iterations=5)
    expect_first = fpm.run_batch(algo, first)
    expect_second = fpm.run_batch(algo, second)
    j1 = fpm.submit_batch(algo, first)
    j2 = fpm.submit_batch(algo, second)
    with pytest.raises(fpm.FpmError, match="in use by a submitted job"):
        fpm.run_batch(algo, [first[0]])
    with pytest.raises(fpm.FpmError, match="in use by a submitted job"):
        second[1].release()
    deadline = time.time() + 60
    while not (j1.done() and j2.done()):
        assert time.time() < deadline
        time.sleep(0.001)
    for expect, got in ((expect_first, j1.wait()), (expect_second, j2.wait())):
        for a, b in zip(expect, got):
            np.testing.assert_array_equal(a.object_spectrum, b.object_spectrum)
    # Finished jobs release their problems.
    again = fpm.run_batch(algo, [first[0]])
    np.testing.assert_array_equal(again[0].object_spectrum, expect_first[0].object_spectrum)


def test_submitted_spectral_batch_equals_run_many(fpm):
    import test_gpu_spectral as ts

    cases = [ts._case(fpm, 32, mixed=True), ts._case(fpm, 64, mixed=True, shared=True, background=0.2)]
    problems = [fpm.SpectralReconstructionProblem(measurements=c[3], model=c[0]) for c in cases]
    solver = fpm.SpectralAlternatingProjection(iterations=3)
    blocking = solver.run_many(problems=problems)
    job = solver.submit_many(problems=problems)
    other = fpm.submit_batch(fpm.AlternatingProjection(iterations=3), _problems(fpm, [(3, 32, 8)]))
    got = job.wait()
    other.wait()
    for a, b in zip(blocking, got):
        np.testing.assert_array_equal(a.object_spectrum, b.object_spectrum)
        np.testing.assert_array_equal([t[1] for t in a.trace], [t[1] for t in b.trace])
