"""Measurement stacks, synthetic objects and acquisition simulation
(src/simulation/simulator.rs:107-226, src/simulation/synthetic_object.rs).

The forward stack (object FFT, crop, pupil, IFFT, |psi|^2 * gain + background)
and the camera model with its noise draws run in one device call.
"""

from __future__ import annotations

import ctypes as C
import math

import numpy as np

from . import _native as N
from .errors import InvalidMeasurementsError, InvalidParameterError, InvalidShapeError, UnsupportedError
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


def _polar(r: float, theta: float) -> complex:
    """Complex64::from_polar: (r cos theta, r sin theta), libm cos and sin
    (NaN for a non-finite angle, as in Rust)."""
    if not math.isfinite(theta):
        return complex(math.nan, math.nan)
    return complex(r * math.cos(theta), r * math.sin(theta))


def _object_shape(shape) -> tuple:
    h, w = int(shape[0]), int(shape[1])
    if h <= 0 or w <= 0:
        raise InvalidShapeError(f"synthetic object dimensions must be non-zero, got ({h}, {w})")
    return h, w


def _real_2d(values, name: str) -> np.ndarray:
    a = np.array(values, dtype=np.float64, order="C")
    if a.ndim != 2:
        raise TypeError(f"{name} must be a 2-D float64 array")
    return a


class SyntheticObject:
    """High-resolution complex sample field used as simulation ground truth
    (src/simulation/synthetic_object.rs:36-376; python/src/simulation.rs:25-180).

    The deterministic targets follow the reference's arithmetic term by term
    (libm hypot, atan2, sin, cos, exp), so their values match it bit for bit.
    `random_phase`, `particle_field` and `biological_like` draw from NumPy's
    PCG64 seeded with `seed`: the same distributions as the reference's
    ChaCha12 stream, not the same values. Image files are not decoded here:
    load the image as an array and use `amplitude_only` or
    `from_amplitude_phase`."""

    def __init__(self, field):
        f = np.array(field, dtype=np.complex128, order="C")
        if f.ndim != 2:
            raise TypeError("field must be a 2-D complex128 array")
        _object_shape(f.shape)
        if not (np.all(np.isfinite(f.real)) and np.all(np.isfinite(f.imag))):
            raise InvalidParameterError("field: values must have finite real and imaginary components")
        self._field = f

    @staticmethod
    def _of(values: np.ndarray) -> "SyntheticObject":
        obj = SyntheticObject.__new__(SyntheticObject)
        obj._field = values
        return obj

    @staticmethod
    def _build(shape, value) -> "SyntheticObject":
        h, w = shape
        out = np.empty((h, w), np.complex128)
        for row in range(h):
            for column in range(w):
                out[row, column] = value(row, column)
        return SyntheticObject._of(out)

    @property
    def field(self) -> np.ndarray:
        return self._field.copy()

    @property
    def shape(self) -> tuple:
        return tuple(self._field.shape)

    @property
    def label(self):
        return None

    @staticmethod
    def constant(shape, amplitude: float = 1.0, phase: float = 0.0) -> "SyntheticObject":
        shape = _object_shape(shape)
        amplitude, phase = float(amplitude), float(phase)
        if not math.isfinite(amplitude) or amplitude < 0.0:
            raise InvalidParameterError("amplitude: must be finite and non-negative")
        return SyntheticObject._of(np.full(shape, _polar(amplitude, phase), np.complex128))

    @staticmethod
    def amplitude_only(amplitude) -> "SyntheticObject":
        a = _real_2d(amplitude, "amplitude")
        _object_shape(a.shape)
        if not np.all(np.isfinite(a)) or np.any(a < 0.0):
            raise InvalidParameterError("amplitude: values must be finite and non-negative")
        return SyntheticObject._of(a.astype(np.complex128))

    @staticmethod
    def phase_only(phase) -> "SyntheticObject":
        p = _real_2d(phase, "phase")
        _object_shape(p.shape)
        if not np.all(np.isfinite(p)):
            raise InvalidParameterError("phase: values must be finite")
        return SyntheticObject._build(p.shape, lambda r, c: _polar(1.0, float(p[r, c])))

    @staticmethod
    def from_amplitude_phase(amplitude, phase) -> "SyntheticObject":
        a, p = _real_2d(amplitude, "amplitude"), _real_2d(phase, "phase")
        if a.shape != p.shape:
            raise InvalidShapeError(f"amplitude {a.shape} and phase {p.shape} differ")
        _object_shape(a.shape)
        return SyntheticObject(SyntheticObject._build(a.shape, lambda r, c: _polar(float(a[r, c]), float(p[r, c])))._field)

    @staticmethod
    def from_amplitude_image(path) -> "SyntheticObject":
        raise UnsupportedError("image decoding is not available here: load the image as an array and use "
                               "SyntheticObject.amplitude_only")

    @staticmethod
    def from_amplitude_phase_images(amplitude_path, phase_path, phase_extent) -> "SyntheticObject":
        raise UnsupportedError("image decoding is not available here: load the images as arrays and use "
                               "SyntheticObject.from_amplitude_phase")

    @staticmethod
    def phase_disk(shape, radius_pixels: float, phase_shift: float) -> "SyntheticObject":
        """Unit amplitude; phase `phase_shift` within `radius_pixels` of the centre (:156-180)."""
        shape = _object_shape(shape)
        radius_pixels, phase_shift = float(radius_pixels), float(phase_shift)
        if not math.isfinite(radius_pixels) or radius_pixels <= 0.0 or not math.isfinite(phase_shift):
            raise InvalidParameterError("phase disk: radius must be positive and phase must be finite")
        c0, c1 = (shape[0] - 1) / 2.0, (shape[1] - 1) / 2.0
        return SyntheticObject._build(shape, lambda r, c: _polar(
            1.0, phase_shift if float(np.hypot(r - c0, c - c1)) <= radius_pixels else 0.0))

    @staticmethod
    def siemens_star(shape, spokes: int) -> "SyntheticObject":
        """Binary amplitude (0.25 / 1) star of `spokes` spokes inside 0.46 of the smaller side (:183-209)."""
        shape = _object_shape(shape)
        spokes = int(spokes)
        if spokes < 2:
            raise InvalidParameterError("spokes: must be at least 2")
        c0, c1 = (shape[0] - 1) / 2.0, (shape[1] - 1) / 2.0
        maximum_radius = float(min(shape)) * 0.46

        def value(r, c):
            y, x = r - c0, c - c1
            dark = float(np.hypot(x, y)) <= maximum_radius and math.sin(math.atan2(x, y) * float(spokes)) >= 0.0
            return complex(0.25 if dark else 1.0, 0.0)

        return SyntheticObject._build(shape, value)

    @staticmethod
    def resolution_target(shape) -> "SyntheticObject":
        """Horizontal and vertical bar groups of periods 2, 3, 4, 6, 8 at amplitude 0.2 (:212-233)."""
        h, w = _object_shape(shape)
        out = np.ones((h, w), np.complex128)
        groups = (2, 3, 4, 6, 8)
        for group, period in enumerate(groups):
            top, bottom = group * h // len(groups), (group + 1) * h // len(groups)
            for row in range(top, bottom):
                for column in range(w):
                    dark = (column // period) % 2 == 0 if group % 2 == 0 else ((row - top) // period) % 2 == 0
                    if dark:
                        out[row, column] = 0.2
        return SyntheticObject._of(out)

    @staticmethod
    def mixed_test_pattern(shape) -> "SyntheticObject":
        """Amplitude bar and disk at 0.45 with a Gaussian plus sinusoidal phase (:275-299)."""
        shape = _object_shape(shape)
        c0, c1 = (shape[0] - 1) / 2.0, (shape[1] - 1) / 2.0
        scale = float(min(shape))

        def value(r, c):
            y, x = r - c0, c - c1
            radius = float(np.hypot(x, y))
            inside = (abs(x) < 0.12 * scale and abs(y) < 0.35 * scale) or radius < 0.12 * scale
            phase = 0.8 * math.exp(-radius * radius / (0.08 * scale * scale)) + 0.25 * math.sin(math.tau * x / scale)
            return _polar(0.45 if inside else 1.0, phase)

        return SyntheticObject._build(shape, value)

    @staticmethod
    def random_phase(shape, standard_deviation: float, seed: int) -> "SyntheticObject":
        shape = _object_shape(shape)
        sd = float(standard_deviation)
        if not math.isfinite(sd) or sd < 0.0:
            raise InvalidParameterError("standard_deviation: must be finite and non-negative")
        if sd == 0.0:
            return SyntheticObject._of(np.ones(shape, np.complex128))
        phase = np.random.default_rng(int(seed)).normal(0.0, sd, shape)
        return SyntheticObject._of(np.cos(phase) + 1j * np.sin(phase))

    @staticmethod
    def particle_field(shape, particles: int, seed: int) -> "SyntheticObject":
        shape = _object_shape(shape)
        out = np.ones(shape, np.complex128)
        rng = np.random.default_rng(int(seed))
        for _ in range(int(particles)):
            out[rng.integers(0, shape[0]), rng.integers(0, shape[1])] = 0.1
        return SyntheticObject._of(out)

    @staticmethod
    def biological_like(shape, features: int, seed: int) -> "SyntheticObject":
        shape = _object_shape(shape)
        if int(features) == 0:
            raise InvalidParameterError("features: must be greater than zero")
        rng = np.random.default_rng(int(seed))
        minimum_size = float(min(shape))
        lower = max(0.02 * minimum_size, 1.0)
        upper = max(0.12 * minimum_size, lower + 0.1)
        rows, cols = np.meshgrid(np.arange(shape[0], dtype=np.float64), np.arange(shape[1], dtype=np.float64),
                                 indexing="ij")
        phase = np.zeros(shape)
        absorption = np.zeros(shape)
        for _ in range(int(features)):
            cr, cc = rng.uniform(0.0, shape[0]), rng.uniform(0.0, shape[1])
            sigma, strength, absorb = rng.uniform(lower, upper), rng.uniform(-0.4, 1.0), rng.uniform(0.0, 0.25)
            profile = np.exp(-((rows - cr) ** 2 + (cols - cc) ** 2) / (2.0 * sigma * sigma))
            phase += strength * profile
            absorption += absorb * profile
        amplitude = np.maximum(1.0 - absorption, 0.1)
        return SyntheticObject._of(amplitude * np.cos(phase) + 1j * amplitude * np.sin(phase))


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


class IlluminationAcquisitionErrors:
    """Acquisition faults applied to the true model before simulation
    (src/simulation/illumination_acquisition_errors.rs:8-50;
    python/src/config.rs:1229-1258): relative Gaussian frame-gain variation,
    frames whose illumination fails, and a source permutation."""

    def __init__(self, *, frame_gain_relative_std: float = 0.0, missing_frames=(), source_permutation=None):
        std = float(frame_gain_relative_std)
        if not math.isfinite(std) or std < 0.0:
            raise ValueError("frame_gain_relative_std must be finite and non-negative")
        indices = [int(i) for i in missing_frames]
        permutation = None if source_permutation is None else [int(i) for i in source_permutation]
        if any(i < 0 for i in indices + (permutation or [])):
            raise OverflowError("frame and source indices must be non-negative")
        self.frame_gain_relative_std = std
        self.missing_frames = indices
        self.source_permutation = permutation


def _apply_acquisition_errors(model: ImagePlaneModel, errors: IlluminationAcquisitionErrors,
                              seed: int) -> ImagePlaneModel:
    """apply_illumination_acquisition_errors (src/simulation/simulator.rs:230-330):
    validation, then the source permutation of k-vectors, crops, offsets,
    gains and per-frame backgrounds, then each frame gain times
    max(N(1, std), 0.01). The draws come from NumPy's PCG64 seeded with
    `seed`: the reference's distribution, not its ChaCha12 values."""
    frames = model.frame_count
    missing = sorted(errors.missing_frames)
    if any(f >= frames for f in missing) or any(a == b for a, b in zip(missing, missing[1:])):
        raise InvalidParameterError(f"missing_frames: must contain unique frame indices below {frames}")
    permutation = errors.source_permutation
    if permutation is not None and sorted(permutation) != list(range(model.source_count)):
        raise InvalidParameterError(f"source_permutation: must be a permutation of 0..{model.source_count}")
    changes = {}
    gains = None if model._gains is None else model._gains.copy()
    if permutation is not None:
        order = np.asarray(permutation, dtype=np.int64)
        changes.update(k_vectors=model._k[order], start_row=model._start_row[order], start_col=model._start_col[order],
                       offset_row=model._offset_row[order], offset_col=model._offset_col[order])
        if gains is not None:
            gains = gains[order]
        n = model.image_shape[0] * model.image_shape[1]
        if model._background is not None and model._background.size == n * frames:
            changes["background"] = model._background.reshape(frames, n)[order].ravel()
    if errors.frame_gain_relative_std > 0.0:
        if gains is None:
            gains = np.ones(frames)
        draws = np.random.default_rng(int(seed) & (2**64 - 1)).normal(1.0, errors.frame_gain_relative_std, frames)
        gains = gains * np.maximum(draws, 0.01)
    if gains is not None:
        changes["frame_gains"] = gains
    return model._replace(**changes) if changes else model


def _frame_background(model: ImagePlaneModel, frame: int) -> np.ndarray:
    """The background a frame's camera sees without illumination (zero when none)."""
    h, w = model.image_shape
    if model._background is None:
        return np.zeros((h, w))
    bg = model._background.ravel()
    return (bg if bg.size == h * w else bg[frame * h * w:(frame + 1) * h * w]).reshape(h, w).copy()


def simulate(true_model: ImagePlaneModel, object, *, reconstruction_model=None, camera: CameraModel | None = None,
             illumination_errors=None, seed: int = 0) -> SimulationResult:
    """Simulate an image-plane FPM acquisition (Simulator::simulate)."""
    field = getattr(object, "field", object)
    field = N.c128(field)
    recon = reconstruction_model if reconstruction_model is not None else true_model
    if (recon.image_shape != true_model.image_shape or recon.reconstruction_shape != true_model.reconstruction_shape
            or recon.frame_count != true_model.frame_count):
        raise InvalidShapeError("true and reconstruction models must have matching image, object, and frame dimensions")
    missing = []
    if illumination_errors is not None:
        if not isinstance(illumination_errors, IlluminationAcquisitionErrors):
            raise TypeError("illumination_errors must be an IlluminationAcquisitionErrors object")
        true_model = _apply_acquisition_errors(true_model, illumination_errors, seed)
        missing = list(illumination_errors.missing_frames)
    if camera is None:
        data = forward_intensities(true_model, field)
        for f in missing:
            data[f] = _frame_background(true_model, f)
    else:
        recon = compile_camera_model(recon, camera)
        data = _simulate_counts(true_model, field, camera, seed)
        if missing:
            # A failed source leaves only the background for the camera
            # (src/simulation/simulator.rs:168-180). A zero object gives
            # gain * 0 + background on every frame, and the camera's streams
            # are keyed by (seed, frame, pixel), so the same seed draws each
            # missing frame's noise as it would have in place.
            dark = _simulate_counts(true_model, np.zeros_like(field), camera, seed)
            data[missing] = dark[missing]
    if missing:
        weights = np.ones(true_model.frame_count)
        weights[missing] = 0.0
        stack = MeasurementStack(data, frame_weights=weights)
    else:
        stack = MeasurementStack(data)
    result = SimulationResult(stack, field.copy(), true_model, recon, camera is None, seed)
    result.missing_frames = missing
    return result


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
