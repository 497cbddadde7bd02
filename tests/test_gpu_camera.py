"""GPU simulate: forward stack + CameraModel::measure_frame on the device
(src/simulation/simulator.rs:107-206, src/simulation/camera.rs:249-290).

The reference draws noise from ChaCha12, which is not reproducible here, so
noise is checked in distribution (mean and variance against the expected
electrons, several standard errors) and the deterministic response (gain,
offset, clamping, quantisation, bad pixels) exactly.
"""

from __future__ import annotations

import numpy as np
import pytest

import helpers
import workloads as W

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def fpm(native_library):
    import fpm_rs

    return fpm_rs


@pytest.fixture(scope="module")
def case(fpm):
    model, omodel = helpers.planar_model(fpm, 5, 64)
    obj = W.smooth_random_object(model.reconstruction_shape, 3)
    intensity = fpm.forward_intensities(model, obj)
    return model, obj, intensity


def test_noise_free_response_is_exact(fpm, case):
    model, obj, intensity = case
    cam = fpm.CameraModel(photons_per_pixel=2.5, gain_counts_per_electron=3.0, offset_counts=10.0,
                          dark_current_electrons=0.5, bit_depth=None, quantize=False)
    counts = fpm.simulate(model, obj, camera=cam, seed=1).measurements._data
    expected = (np.maximum(intensity, 0.0) * 2.5 + 0.5) * 3.0 + 10.0
    assert np.abs(counts - expected).max() <= 1e-12 * np.abs(expected).max()


@pytest.mark.parametrize("photons", [0.3, 4.0, 40.0, 1e4])
def test_shot_noise_mean_and_variance(fpm, case, photons):
    """Poisson counts (inversion below a mean of 10, PTRS above): mean and
    variance match the expected electrons."""
    model, obj, intensity = case
    cam = fpm.CameraModel(photons_per_pixel=photons, shot_noise=True, bit_depth=None, quantize=False)
    counts = fpm.simulate(model, obj, camera=cam, seed=7).measurements._data
    lam = np.maximum(intensity, 0.0) * photons
    assert np.all(counts == np.round(counts)) and counts.min() >= 0.0
    total = lam.sum()
    assert abs(counts.sum() - total) <= 6.0 * np.sqrt(total)
    ratio = np.sum((counts - lam) ** 2) / total  # E = 1
    assert abs(ratio - 1.0) <= 0.05


def test_read_noise_and_reproducibility(fpm, case):
    model, obj, intensity = case
    cam = fpm.CameraModel(photons_per_pixel=100.0, read_noise_electrons=5.0, offset_counts=1000.0, bit_depth=None,
                          quantize=False)
    a = fpm.simulate(model, obj, camera=cam, seed=11).measurements._data
    b = fpm.simulate(model, obj, camera=cam, seed=11).measurements._data
    c = fpm.simulate(model, obj, camera=cam, seed=12).measurements._data
    assert np.array_equal(a, b)
    assert not np.array_equal(a, c)
    residual = a - (np.maximum(intensity, 0.0) * 100.0 + 1000.0)
    assert abs(residual.mean()) <= 6.0 * 5.0 / np.sqrt(residual.size)
    assert abs(residual.std() / 5.0 - 1.0) <= 0.03


def test_clamping_quantisation_and_bad_pixels(fpm, case):
    model, obj, intensity = case
    cam = fpm.CameraModel(photons_per_pixel=3e3, shot_noise=True, bit_depth=8, quantize=True, bad_pixels=(0, 5, 77),
                          bad_pixel_value_counts=1e9)
    counts = fpm.simulate(model, obj, camera=cam, seed=3).measurements._data
    assert counts.max() <= 255.0 and counts.min() >= 0.0
    assert np.all(counts == np.round(counts))
    flat = counts.reshape(counts.shape[0], -1)
    assert np.all(flat[:, [0, 5, 77]] == 255.0)
    bright = np.maximum(intensity, 0.0) * 3e3 > 400.0
    assert np.all(counts[bright] == 255.0)


def test_camera_validation(fpm, case):
    model, obj, intensity = case
    with pytest.raises(fpm.InvalidParameterError):
        fpm.simulate(model, obj, camera=fpm.CameraModel(photons_per_pixel=-1.0), seed=1)
    with pytest.raises(fpm.InvalidParameterError):
        fpm.simulate(model, obj, camera=fpm.CameraModel(bad_pixels=(10**9,)), seed=1)
