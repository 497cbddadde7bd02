"""Host side of simulate's illumination acquisition errors
(src/simulation/simulator.rs:230-330; illumination_acquisition_errors.rs):
the true-model permutation, the seeded gain variation, missing frames, and
validation. The forward stack itself is covered by the GPU tests."""

from __future__ import annotations

import numpy as np
import pytest

import helpers


@pytest.fixture(scope="module")
def fpm(native_library):
    import fpm_rs

    return fpm_rs


@pytest.fixture(scope="module")
def model(fpm):
    m, _ = helpers.planar_model(fpm, 3, 32)
    rng = np.random.default_rng(4)
    return m._replace(frame_gains=rng.uniform(0.5, 2.0, m.frame_count),
                      background=rng.uniform(0.0, 1.0, m.frame_count * 32 * 32))


def test_source_permutation_reorders_every_per_source_array(fpm, model):
    from fpm_rs.simulation import _apply_acquisition_errors

    order = list(np.random.default_rng(1).permutation(model.frame_count))
    errors = fpm.IlluminationAcquisitionErrors(source_permutation=order)
    out = _apply_acquisition_errors(model, errors, seed=0)
    assert np.array_equal(out.k_vectors, model.k_vectors[order])
    assert np.array_equal(out.crop_origins, model.crop_origins[order])
    assert np.array_equal(out.subpixel_offsets, model.subpixel_offsets[order])
    assert np.array_equal(out.frame_gains, model.frame_gains[order])
    n = 32 * 32
    assert np.array_equal(out._background.reshape(-1, n), model._background.reshape(-1, n)[order])
    single = model._replace(background=np.arange(n, dtype=np.float64))
    assert np.array_equal(_apply_acquisition_errors(single, errors, 0)._background, single._background)


def test_frame_gain_variation_is_seeded_and_clamped(fpm, model):
    from fpm_rs.simulation import _apply_acquisition_errors

    errors = fpm.IlluminationAcquisitionErrors(frame_gain_relative_std=0.2)
    first = _apply_acquisition_errors(model, errors, seed=11).frame_gains
    assert np.array_equal(first, _apply_acquisition_errors(model, errors, seed=11).frame_gains)
    draws = np.random.default_rng(11).normal(1.0, 0.2, model.frame_count)
    assert np.array_equal(first, model.frame_gains * np.maximum(draws, 0.01))
    wild = _apply_acquisition_errors(model._replace(frame_gains=None),
                                     fpm.IlluminationAcquisitionErrors(frame_gain_relative_std=5.0), seed=2)
    assert np.all(wild.frame_gains >= 0.01)
    unchanged = _apply_acquisition_errors(model, fpm.IlluminationAcquisitionErrors(), seed=3)
    assert np.array_equal(unchanged.frame_gains, model.frame_gains)


def test_missing_frames_see_only_the_background(fpm, model):
    from fpm_rs.simulation import _frame_background

    assert np.array_equal(_frame_background(model, 5).ravel(), model._background[5 * 1024:6 * 1024])
    assert np.array_equal(_frame_background(model._replace(background=None), 5), np.zeros((32, 32)))
    flat = np.linspace(0.0, 1.0, 1024)
    assert np.array_equal(_frame_background(model._replace(background=flat), 7).ravel(), flat)


def test_acquisition_error_validation(fpm, model):
    from fpm_rs.simulation import _apply_acquisition_errors

    frames = model.frame_count
    for errors in (fpm.IlluminationAcquisitionErrors(missing_frames=[frames]),
                   fpm.IlluminationAcquisitionErrors(missing_frames=[1, 1]),
                   fpm.IlluminationAcquisitionErrors(source_permutation=[0] * frames),
                   fpm.IlluminationAcquisitionErrors(source_permutation=list(range(frames - 1)))):
        with pytest.raises(fpm.InvalidParameterError):
            _apply_acquisition_errors(model, errors, 0)
    with pytest.raises(ValueError):
        fpm.IlluminationAcquisitionErrors(frame_gain_relative_std=-0.1)
    with pytest.raises(OverflowError):
        fpm.IlluminationAcquisitionErrors(missing_frames=[-1])
    with pytest.raises(TypeError):
        fpm.simulate(model, np.ones(model.reconstruction_shape, np.complex128), illumination_errors={"missing": [1]})
