"""Narrowband spectral test cases shared by the oracle and GPU parity tests.

The channel set follows the reference's spectral fixtures
(tests/spectral_tests.rs:307-427, python/tests/test_spectral.py:8-63): three
wavelengths (450, 532, 630 nm) at NA 0.12, 4x, 6.5 um pixels and 1 um
defocus, one shared direction-cosine geometry resolved per wavelength, and
the smooth union grid of every channel's crops. Source calibration is
expressed as per-source frame gains.
"""

from __future__ import annotations

import math

import numpy as np

import oracle

WAVELENGTHS = (450e-9, 532e-9, 630e-9)
CHANNEL_IDS = ("blue", "green", "red")
DIRECTIONS = ((0.0, 0.0), (0.08, 0.03), (-0.05, 0.07))


def optics(wavelength: float, defocus=1e-6) -> dict:
    return dict(wavelength_vacuum_m=wavelength, objective_na=0.12, magnification=4.0, camera_pixel_size=6.5e-6,
                defocus_distance=defocus)


def kvectors(wavelength: float, directions, refractive_index=1.0) -> np.ndarray:
    """DirectionList::resolve (src/experiment/illumination.rs:240-254): k * (ux, uy)."""
    k = 2.0 * math.pi * refractive_index / wavelength
    d = np.asarray(directions, dtype=np.float64)
    return np.stack([k * d[:, 0], k * d[:, 1]], axis=1)


def compile_channels(count=3, directions=DIRECTIONS, image_shape=(8, 12), policy="smooth", frame_gains=None,
                     defocus=1e-6) -> list:
    """Oracle-compiled channel kernels on the union grid of all channels
    (SpectralImagePlaneModel::from_experiment, src/model/spectral.rs:128-200)."""
    opts = [optics(w, defocus) for w in WAVELENGTHS[:count]]
    ks = [kvectors(w, directions) for w in WAVELENGTHS[:count]]
    union = np.concatenate(ks)
    first = oracle.compile_model(opts[0], union[:, 0], union[:, 1], image_shape, policy)
    shape = (first["mh"], first["mw"])
    channels = []
    for o, k in zip(opts, ks):
        m = oracle.compile_model(o, k[:, 0], k[:, 1], image_shape, shape)
        m["frame_gains"] = np.ones(len(k)) if frame_gains is None else np.asarray(frame_gains, np.float64)
        channels.append(m)
    return channels


def separate_frames(counts) -> list:
    """SpectralAcquisitionPlan::separate (src/experiment/spectral.rs:91-116)."""
    return [(1.0, 0.0, [(c, l, 1.0)]) for c, n in enumerate(counts) for l in range(n)]


def mixed_frames(local_frames=2, weights=(0.4, 0.8, 1.1), gain=1.7, background=0.2, count=3) -> list:
    return [(gain, background, [(c, l, weights[c]) for c in range(count)]) for l in range(local_frames)]


def truth_objects(shape, count) -> np.ndarray:
    rows, cols = np.indices(shape)
    return np.ascontiguousarray([
        (0.8 + 0.1 * np.sin(rows + cols + c)) * np.exp(1j * 0.1 * np.cos(rows * 0.4 + cols * 0.7 + c))
        for c in range(count)], dtype=np.complex128)


def spectra_of(objects) -> np.ndarray:
    return np.stack([oracle.object_spectrum(o) for o in objects])
