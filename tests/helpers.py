"""Problem builders shared by the parity tests and bench.py.

Each builder returns the product model (fpm_rs), the oracle's compiled model
dict (bit-identical crops and offsets, checked in test_host.py) and the
measurement stack generated by the FP64 oracle forward model, optionally with
Poisson noise. GPU and oracle always see identical float64 measurements.
"""

from __future__ import annotations

import numpy as np

import oracle
import workloads as W


def planar_model(fpm, side: int, n: int, shape_policy="smooth"):
    optics = fpm.Optics(**W.OPTICS)
    grid, ref = W.led_grid(side)
    geometry = fpm.PlanarLEDArray(grid, W.PITCH, ref, fpm.ArrayPose.from_translation((0.0, 0.0, W.Z)))
    model = fpm.compile_model(optics, fpm.Illumination(geometry), (n, n), shape_policy)
    omodel = oracle.compile_model(W.OPTICS, model.k_vectors[:, 0], model.k_vectors[:, 1], (n, n), shape_policy)
    return model, omodel


def simulated(fpm, side: int, n: int, seed: int, photons: float | None = None, pupil_seed: int | None = None,
              workers: int = 8):
    """(model, oracle model, measurements, truth) for a planar LED tile.

    ``photons``: Poisson counts with that many photons at the bright-field
    peak; the frame gains of both models become photons per unit intensity.
    ``pupil_seed``: true pupil with random Zernike aberrations (defocus, two
    astigmatisms, two comas, N(0, 0.5 rad)) used for the simulation; the
    reconstruction models keep the compiled circular pupil.
    """
    model, omodel = planar_model(fpm, side, n)
    truth = W.smooth_random_object(model.reconstruction_shape, seed)
    sim = dict(omodel)
    if pupil_seed is not None:
        sim["pupil"] = W.zernike_pupil(omodel["support"], pupil_seed)
    spectrum = oracle.object_spectrum(truth)
    intensity = oracle.forward_stack(oracle.Problem(sim, None), spectrum, workers=workers)
    gains = None
    if photons is not None:
        counts, scale = W.poisson_counts(intensity, photons, seed + 1)
        intensity = counts
        gains = np.full(model.frame_count, scale)
        model = model._replace(frame_gains=gains)
    return model, omodel, intensity, truth, gains
