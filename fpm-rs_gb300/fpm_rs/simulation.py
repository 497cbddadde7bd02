"""Measurement stacks and acquisition simulation (src/simulation/simulator.rs:107-226).

The forward stack (object FFT, crop, pupil, IFFT, |psi|^2 * gain + background)
runs on the GPU; the camera's noise draws run on the host in frame order.
"""

from __future__ import annotations

import ctypes as C

import numpy as np

from . import _native as N
from .errors import InvalidMeasurementsError, InvalidShapeError, UnsupportedError
from .experiment import CameraModel
from .model import ImagePlaneModel, compile_camera_model


class MeasurementStack:
    """Resident float64 intensity stack shaped (frames, height, width)."""

    def __init__(self, measurements, *, frame_weights=None, masks=None):
        data = np.array(measurements, dtype=np.float64, order="C", copy=True)
        if data.ndim != 3 or 0 in data.shape:
            raise InvalidMeasurementsError("measurements must have non-empty shape (frames, height, width)")
        if not np.all(np.isfinite(data)):
            raise InvalidMeasurementsError("measurements contain non-finite values")
        self._data = data
        frames = data.shape[0]
        if frame_weights is None:
            self._weights = np.ones(frames)
        else:
            w = np.array(frame_weights, dtype=np.float64)
            if w.shape != (frames,):
                raise InvalidMeasurementsError(f"{w.size} frame weights for {frames} frames")
            if np.any(~np.isfinite(w)) or np.any(w < 0):
                bad = int(np.flatnonzero(~np.isfinite(w) | (w < 0))[0])
                raise InvalidMeasurementsError(f"frame {bad} has invalid weight {w[bad]}")
            self._weights = w
        if masks is None:
            self._masks = None
        else:
            m = np.array(masks, dtype=np.uint8, order="C", copy=True)
            if m.shape == data.shape[1:]:
                m = np.broadcast_to(m, data.shape).copy()
            if m.shape != data.shape:
                raise InvalidMeasurementsError("masks dimensions do not match the measurement stack")
            self._masks = m

    @property
    def shape(self):
        return self._data.shape

    @property
    def frame_count(self) -> int:
        return self._data.shape[0]

    def __len__(self) -> int:
        """The frame count (python/src/measurements.rs:118-120)."""
        return self._data.shape[0]

    @property
    def image_shape(self):
        return self._data.shape[1:]

    @property
    def array(self) -> np.ndarray:
        return self._data.copy()

    @property
    def frame_weights(self) -> np.ndarray:
        return self._weights.copy()

    @property
    def masks(self):
        return None if self._masks is None else self._masks.copy()


class SimulationResult:
    def __init__(self, measurements, ground_truth_object, true_model, reconstruction_model, ideal, seed):
        self.measurements = measurements
        self.ground_truth_object = ground_truth_object
        self.true_model = true_model
        self.reconstruction_model = reconstruction_model
        self.ideal = ideal
        self.missing_frames = []
        self.random_seed = seed


def forward_intensities(model: ImagePlaneModel, object_field) -> np.ndarray:
    """ForwardModel::forward_intensity_stack of a complex object on the GPU."""
    obj = N.c128(object_field)
    if obj.shape != model.reconstruction_shape:
        raise InvalidShapeError(
            f"object shape {obj.shape} differs from reconstruction shape {model.reconstruction_shape}")
    desc, keep = model._descriptor()
    out = np.zeros((model.frame_count, *model.image_shape))
    ctx = N.context()
    N.check(N.library().fpm_forward_stack(ctx.handle, C.byref(desc), N.ptr(obj, C.c_double),
                                          N.ptr(out, C.c_double)), ctx.handle)
    del keep
    return out


def simulate(true_model: ImagePlaneModel, object, *, reconstruction_model=None, camera: CameraModel | None = None,
             illumination_errors=None, seed: int = 0) -> SimulationResult:
    """Simulate an image-plane FPM acquisition (Simulator::simulate)."""
    if illumination_errors is not None:
        raise UnsupportedError("illumination acquisition errors are not supported on the GB300 device path")
    field = getattr(object, "field", object)
    field = N.c128(field)
    recon = reconstruction_model if reconstruction_model is not None else true_model
    if (recon.image_shape != true_model.image_shape or recon.reconstruction_shape != true_model.reconstruction_shape
            or recon.frame_count != true_model.frame_count):
        raise InvalidShapeError("true and reconstruction models must have matching image, object, and frame dimensions")
    if camera is None:
        data = forward_intensities(true_model, field)
    else:
        recon = compile_camera_model(recon, camera)
        data = _simulate_counts(true_model, field, camera, seed)
    return SimulationResult(MeasurementStack(data), field.copy(), true_model, recon, camera is None, seed)


def _simulate_counts(model: ImagePlaneModel, field: np.ndarray, camera: CameraModel, seed: int) -> np.ndarray:
    """Forward stack and detector in one device call (fpm_simulate_stack)."""
    if field.shape != model.reconstruction_shape:
        raise InvalidShapeError(
            f"object shape {field.shape} differs from reconstruction shape {model.reconstruction_shape}")
    h, w = model.image_shape
    desc, keep = model._descriptor()
    cam, cam_keep = camera._descriptor(h * w)
    out = np.empty((model.frame_count, h, w), np.float64)
    ctx = N.context()
    N.check(N.library().fpm_simulate_stack(ctx.handle, C.byref(desc), N.ptr(field, C.c_double), C.byref(cam),
                                           C.c_uint64(int(seed) & (2**64 - 1)), N.ptr(out, C.c_double)), ctx.handle)
    return out
