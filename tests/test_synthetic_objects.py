"""SyntheticObject (src/simulation/synthetic_object.rs; python/src/simulation.rs:25-180):
the deterministic targets, validation, and the seeded generators' contract.
Host-only: no GPU."""

from __future__ import annotations

import math

import numpy as np
import pytest

from test_oracle_kat import _mixed_test_pattern


@pytest.fixture(scope="module")
def fpm(native_library):
    import fpm_rs

    return fpm_rs


def test_mixed_test_pattern(fpm):
    # tests/simulation_tests.rs:613-616 and the restatement the oracle tests use.
    for shape in [(16, 16), (32, 24)]:
        field = fpm.SyntheticObject.mixed_test_pattern(shape).field
        assert field.shape == shape
        assert np.abs(field - _mixed_test_pattern(shape)).max() <= 1e-15
    field = fpm.SyntheticObject.mixed_test_pattern((32, 32)).field
    assert np.any(np.abs(field) < 0.9) and np.any(np.abs(np.angle(field)) > 0.1)


def test_deterministic_targets(fpm):
    disk = fpm.SyntheticObject.phase_disk((16, 16), 4.0, 0.7).field
    assert np.allclose(np.abs(disk), 1.0, atol=1e-15)
    centre = (7.5, 7.5)
    for r in range(16):
        for c in range(16):
            inside = math.hypot(r - centre[0], c - centre[1]) <= 4.0
            assert disk[r, c] == complex(math.cos(0.7 if inside else 0.0), math.sin(0.7 if inside else 0.0))
    star = fpm.SyntheticObject.siemens_star((33, 33), 8).field
    assert set(np.unique(star.real)) == {0.25, 1.0} and np.all(star.imag == 0.0)
    assert star[0, 0] == 1.0 and star[16, 16] == 0.25  # corners lie outside 0.46 of the side
    target = fpm.SyntheticObject.resolution_target((20, 12)).field
    assert set(np.unique(target.real)) == {0.2, 1.0}
    # Group 0 (rows 0-3): vertical bars of period 2; group 1 (rows 4-7): horizontal bars of period 3.
    assert np.array_equal(target[0].real, [0.2, 0.2, 1, 1] * 3)
    assert np.array_equal(target[4:8, 0].real, [0.2, 0.2, 0.2, 1.0])
    constant = fpm.SyntheticObject.constant((16, 16), 10.0, 0.0)
    assert constant.shape == (16, 16) and np.all(constant.field == 10.0) and constant.label is None


def test_array_constructors_and_validation(fpm):
    rng = np.random.default_rng(3)
    amplitude, phase = rng.uniform(0.1, 1.0, (5, 6)), rng.uniform(-3.0, 3.0, (5, 6))
    both = fpm.SyntheticObject.from_amplitude_phase(amplitude, phase).field
    assert np.array_equal(both.real, amplitude * np.vectorize(math.cos)(phase))
    assert np.array_equal(both.imag, amplitude * np.vectorize(math.sin)(phase))
    assert np.array_equal(fpm.SyntheticObject.amplitude_only(amplitude).field, amplitude + 0j)
    assert np.allclose(np.abs(fpm.SyntheticObject.phase_only(phase).field), 1.0, atol=1e-15)
    assert np.array_equal(fpm.SyntheticObject(both).field, both)
    for bad, error in [(lambda: fpm.SyntheticObject(np.full((2, 2), np.nan + 0j)), fpm.InvalidParameterError),
                       (lambda: fpm.SyntheticObject.amplitude_only(-amplitude), fpm.InvalidParameterError),
                       (lambda: fpm.SyntheticObject.phase_only(np.full((2, 2), np.inf)), fpm.InvalidParameterError),
                       (lambda: fpm.SyntheticObject.from_amplitude_phase(amplitude, phase[:4]), fpm.InvalidShapeError),
                       (lambda: fpm.SyntheticObject.constant((0, 4)), fpm.InvalidShapeError),
                       (lambda: fpm.SyntheticObject.constant((4, 4), -1.0), fpm.InvalidParameterError),
                       (lambda: fpm.SyntheticObject.phase_disk((4, 4), 0.0, 0.1), fpm.InvalidParameterError),
                       (lambda: fpm.SyntheticObject.siemens_star((4, 4), 1), fpm.InvalidParameterError),
                       (lambda: fpm.SyntheticObject.from_amplitude_image("a.png"), fpm.UnsupportedError)]:
        with pytest.raises(error):
            bad()


def test_seeded_generators(fpm):
    # tests/simulation_tests.rs:618-630: reproducible for a seed, finite,
    # amplitude at least 0.1, and empty shapes refused.
    first = fpm.SyntheticObject.biological_like((32, 32), 12, 99).field
    assert np.array_equal(first, fpm.SyntheticObject.biological_like((32, 32), 12, 99).field)
    assert np.all(np.isfinite(first)) and np.all(np.abs(first) >= 0.1 - 1e-15)
    assert not np.array_equal(first, fpm.SyntheticObject.biological_like((32, 32), 12, 100).field)
    with pytest.raises(fpm.InvalidShapeError):
        fpm.SyntheticObject.biological_like((0, 32), 4, 1)
    with pytest.raises(fpm.InvalidShapeError):
        fpm.SyntheticObject.particle_field((32, 0), 4, 1)
    particles = fpm.SyntheticObject.particle_field((16, 16), 5, 2).field
    assert set(np.unique(particles.real)) <= {0.1, 1.0} and 1 <= np.sum(particles.real == 0.1) <= 5
    assert np.array_equal(fpm.SyntheticObject.random_phase((4, 4), 0.0, 1).field, np.ones((4, 4)))
    noisy = fpm.SyntheticObject.random_phase((64, 64), 0.3, 7).field
    assert np.allclose(np.abs(noisy), 1.0) and abs(np.std(np.angle(noisy)) - 0.3) < 0.02
