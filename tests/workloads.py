"""Seeded synthetic FPM workloads shared by the test suite and bench.py.

The reference publishes no dataset for these shapes, so seeded synthetic
inputs stand in: objects with uniform random amplitude in [0.5, 1] and phase
in [-pi/2, pi/2], each Gaussian-smoothed with sigma = 2 px (periodic
boundary, smoothing after drawing), rescaled back onto their stated ranges;
Poisson noise at a stated photon count at the bright-field peak. Geometry is
the reference README quickstart: 532 nm, NA 0.10, 4x, 6.5 um pixels, a planar
LED array with 4 mm pitch at z = -90 mm, centred on the middle LED.
"""

from __future__ import annotations

import math

import numpy as np

OPTICS = dict(wavelength_vacuum_m=532e-9, objective_na=0.10, magnification=4.0,
              camera_pixel_size=6.5e-6)
PITCH = 4e-3
Z = -90e-3


def _smooth_periodic(field: np.ndarray, sigma: float) -> np.ndarray:
    """Gaussian filter with periodic boundaries, applied in Fourier space."""
    h, w = field.shape
    fy = np.fft.fftfreq(h)[:, None]
    fx = np.fft.fftfreq(w)[None, :]
    kernel = np.exp(-2.0 * (math.pi * sigma) ** 2 * (fx * fx + fy * fy))
    return np.real(np.fft.ifft2(np.fft.fft2(field) * kernel))


def _rescale(values: np.ndarray, lo: float, hi: float) -> np.ndarray:
    vmin, vmax = values.min(), values.max()
    if vmax - vmin <= 0:
        return np.full_like(values, 0.5 * (lo + hi))
    return lo + (hi - lo) * (values - vmin) / (vmax - vmin)


def smooth_random_object(shape, seed: int, sigma: float = 2.0) -> np.ndarray:
    rng = np.random.default_rng(seed)
    amplitude = rng.uniform(0.5, 1.0, size=shape)
    phase = rng.uniform(-math.pi / 2, math.pi / 2, size=shape)
    amplitude = _rescale(_smooth_periodic(amplitude, sigma), 0.5, 1.0)
    phase = _rescale(_smooth_periodic(phase, sigma), -math.pi / 2, math.pi / 2)
    return (amplitude * np.exp(1j * phase)).astype(np.complex128)


def led_grid(side: int):
    """(shape, reference_index (col,row)) for a square LED grid centred on its middle LED."""
    centre = (side - 1) / 2.0
    return (side, side), (centre, centre)


def zernike_pupil(support: np.ndarray, seed: int, sigma_rad: float = 0.5) -> np.ndarray:
    """Support x exp(i * sum of defocus, two astigmatisms and two comas), N(0, sigma) coefficients."""
    h, w = support.shape
    rng = np.random.default_rng(seed)
    coeff = rng.normal(0.0, sigma_rad, size=5)
    rows, cols = np.indices((h, w))
    y = rows - h // 2
    x = cols - w // 2
    radius = max(np.sqrt((x * x + y * y)[support != 0]).max(), 1.0)
    rho = np.sqrt(x * x + y * y) / radius
    theta = np.arctan2(y, x)
    phase = (coeff[0] * (2 * rho**2 - 1)
             + coeff[1] * rho**2 * np.cos(2 * theta)
             + coeff[2] * rho**2 * np.sin(2 * theta)
             + coeff[3] * (3 * rho**3 - 2 * rho) * np.cos(theta)
             + coeff[4] * (3 * rho**3 - 2 * rho) * np.sin(theta))
    return np.where(support != 0, np.exp(1j * phase), 0.0).astype(np.complex128)


def poisson_counts(intensity: np.ndarray, photons_at_peak: float, seed: int):
    """Poisson photon counts with ``photons_at_peak`` expected at the bright-field peak.

    Returns (counts, photons_per_unit_intensity): the reconstruction model's
    frame gains are the latter, as the reference's
    CameraModel.compile_reconstruction_model does (src/simulation/camera.rs:296-318).
    """
    peak = float(intensity.max())
    scale = photons_at_peak / peak
    rng = np.random.default_rng(seed)
    counts = rng.poisson(np.maximum(intensity, 0.0) * scale).astype(np.float64)
    return counts, scale
