"""Narrowband spectral reconstruction on the GB300 device backend.

Mirrors the reference's spectral Python surface (python/src/spectral.rs:34-823):
SpectralChannel, SpectralGeometry, SpectralFrame, SpectralAcquisitionPlan,
compile_spectral_model, SpectralImagePlaneModel, SpectralReconstructionProblem,
SpectralAlternatingProjection and SpectralReconstructionResult, with the
checkpoint format of src/reconstruction/spectral_checkpoint.rs:25-135. The
passes run in libfpm_gpu (fpm_spectral_run): every exposure's coherent modes
are evaluated from the pre-exposure objects, one amplitude ratio from their
weighted intensity sum is applied to all of them, and each mode's
local-denominator correction goes into its channel's object or the one
shared object.
"""

from __future__ import annotations

import ctypes as C
import hashlib
import json
import math
import os
import tempfile
import time
from dataclasses import dataclass, field
from pathlib import Path

import numpy as np

from . import _native as N
from .errors import InvalidMeasurementsError, InvalidParameterError, InvalidShapeError, UnsupportedError, json_file_errors
from .experiment import KVectorList, Optics
from .model import ImagePlaneModel, compile_model, suggest_reconstruction_shape
from .simulation import MeasurementStack

_COUPLINGS = {"independent": 0, "shared_complex": 1}
_LOSSES = {"amplitude_mse": 0, "intensity_mse": 1, "poisson_nll": 2, "huber_amplitude": 3}
FORMAT_VERSION = 1


def _coupling(value: str) -> int:
    if value not in _COUPLINGS:
        raise InvalidParameterError("object_coupling must be 'independent' or 'shared_complex'")
    return _COUPLINGS[value]


class SpectralChannel:
    """Fixed narrowband optics and the channel's local acquisition
    (src/experiment/spectral.rs:11-26). Source calibration and local
    multiplexing are expressed through the compiled channel's frame gains;
    the GB300 device path accepts only unit calibration and the all-sources plan here."""

    def __init__(self, *, channel_id, optics: Optics, calibration=None, acquisition=None):
        if calibration is not None or acquisition is not None:
            raise UnsupportedError(
                "source calibration and local acquisition plans are not supported on the GB300 device path; "
                "set frame gains on compiled channels with SpectralImagePlaneModel.from_compiled_channels")
        self._channel_id = str(channel_id)
        self.optics = optics

    @property
    def channel_id(self) -> str:
        return self._channel_id

    @property
    def wavelength_vacuum_m(self) -> float:
        return self.optics.wavelength_vacuum_m


class SpectralGeometry:
    """Physical source geometry shared across channels (resolved per
    wavelength) or given per channel (src/experiment/spectral.rs:28-37)."""

    def __init__(self, shared, geometries):
        self._shared = shared
        self._geometries = geometries

    @staticmethod
    def shared(*, geometry) -> "SpectralGeometry":
        return SpectralGeometry(True, [geometry])

    @staticmethod
    def per_channel(*, geometries) -> "SpectralGeometry":
        return SpectralGeometry(False, list(geometries))

    def _for_channels(self, count: int) -> list:
        if self._shared:
            if isinstance(self._geometries[0], KVectorList):
                raise InvalidParameterError("wavelength-specific KVectorList cannot be shared physical geometry")
            return self._geometries * count
        if len(self._geometries) != count:
            raise InvalidParameterError("spectral_geometry requires one geometry per channel")
        return self._geometries


class SpectralFrame:
    """One detector exposure: (channel, local_frame, spectral_weight)
    contributions, detector gain and uniform background
    (src/experiment/spectral.rs:51-60)."""

    def __init__(self, *, contributions, gain=1.0, background=0.0):
        self._contributions = [(int(c), int(l), float(w)) for c, l, w in contributions]
        self._gain = float(gain)
        self._background = float(background)

    @property
    def contributions(self) -> list:
        return list(self._contributions)

    @property
    def gain(self) -> float:
        return self._gain

    @property
    def background(self) -> float:
        return self._background


class SpectralAcquisitionPlan:
    """Canonical sparse detector plan (src/experiment/spectral.rs:62-170):
    duplicate (channel, local_frame) pairs summed, zero weights removed,
    pairs sorted, global row order kept."""

    def __init__(self, frames):
        self._frames = frames

    @staticmethod
    def separate(*, frame_counts) -> "SpectralAcquisitionPlan":
        counts = [int(c) for c in frame_counts]
        if not counts or any(c <= 0 for c in counts):
            raise InvalidParameterError("frame_counts: every channel must have at least one local frame")
        return SpectralAcquisitionPlan.multiplexed(
            frames=[SpectralFrame(contributions=[(c, l, 1.0)]) for c, n in enumerate(counts) for l in range(n)])

    @staticmethod
    def multiplexed(*, frames) -> "SpectralAcquisitionPlan":
        frames = list(frames)
        if not frames:
            raise InvalidParameterError("spectral_acquisition: at least one detector frame is required")
        canonical = []
        for frame in frames:
            if not math.isfinite(frame.gain) or frame.gain <= 0.0:
                raise InvalidParameterError("spectral_frame_gain must be finite and positive")
            if not math.isfinite(frame.background) or frame.background < 0.0:
                raise InvalidParameterError("spectral_frame_background must be finite and non-negative")
            pairs = {}
            for c, l, w in frame.contributions:
                if not math.isfinite(w) or w < 0.0:
                    raise InvalidParameterError("spectral_weight must be finite and non-negative")
                pairs[(c, l)] = pairs.get((c, l), 0.0) + w
            if any(not math.isfinite(w) for w in pairs.values()):
                raise InvalidParameterError("spectral_weight: summed duplicate weights must be finite")
            kept = [(c, l, w) for (c, l), w in sorted(pairs.items()) if w > 0.0]
            if not kept:
                raise InvalidParameterError("spectral_acquisition: each detector frame must have a positive contribution")
            canonical.append(SpectralFrame(contributions=kept, gain=frame.gain, background=frame.background))
        return SpectralAcquisitionPlan(canonical)

    @property
    def frame_count(self) -> int:
        return len(self._frames)

    @property
    def frames(self) -> list:
        return list(self._frames)


@dataclass
class SpectralMixingDiagnostics:
    """Linear exposure/channel weight diagnostics (src/model/mixing.rs:5-25)."""

    channel_ids: list
    matrix: np.ndarray
    singular_values: list
    rank: int
    relative_tolerance: float
    absolute_tolerance: float
    condition_number: float | None


class SpectralImagePlaneModel:
    """Channel kernels on one common grid and the detector plan
    (src/model/spectral.rs:46-398)."""

    def __init__(self, channel_ids, models, acquisition: SpectralAcquisitionPlan, object_coupling="independent"):
        self._ids = [str(i) for i in channel_ids]
        self._models = list(models)
        self._acquisition = acquisition
        self._coupling = object_coupling
        _coupling(object_coupling)
        self._validate()

    @staticmethod
    def from_compiled_channels(*, channel_ids, models, acquisition, object_coupling="independent"):
        if len(channel_ids) != len(models):
            raise InvalidParameterError("one channel ID is needed per compiled model")
        return SpectralImagePlaneModel(channel_ids, models, acquisition, object_coupling)

    def _validate(self) -> None:
        if not self._models:
            raise InvalidParameterError("spectral_channels: at least one channel is required")
        first = self._models[0]
        seen, wavelengths = set(), []
        for cid, m in zip(self._ids, self._models):
            if not cid.strip() or cid in seen:
                raise InvalidParameterError("channel_id: channel IDs must be non-empty and unique")
            seen.add(cid)
            w = m._wavelength
            if w is None:
                raise InvalidParameterError("wavelength_vacuum_m: every channel must retain wavelength metadata")
            if not math.isfinite(w) or w <= 0.0 or w in wavelengths:
                raise InvalidParameterError("wavelength_vacuum_m: wavelengths must be finite, positive, and distinct")
            wavelengths.append(w)
            pa, pb = m._low_res_pixel_size, first._low_res_pixel_size
            same_pitch = pa is None or pb is None or abs(pa - pb) <= 1e-12 * max(abs(pa), abs(pb))
            if m.image_shape != first.image_shape or m.reconstruction_shape != first.reconstruction_shape or not same_pitch:
                raise InvalidParameterError(
                    "spectral_sampling: all channel kernels must share detector shape, reconstruction grid, and "
                    "object-plane pixel pitch")
            if m._background is not None:
                raise InvalidParameterError("spectral_background: background belongs to physical detector rows, not channel kernels")
        covered = [np.zeros(m.frame_count, bool) for m in self._models]
        for frame in self._acquisition.frames:
            total = 0.0
            for c, l, w in frame.contributions:
                if c >= len(self._models) or l >= self._models[c].frame_count:
                    raise InvalidParameterError("spectral_acquisition: channel/local_frame reference is out of range")
                covered[c][l] = True
                total += w * self._frame_gain(c, l)
            if not math.isfinite(total) or total <= 0.0 or not math.isfinite(frame.gain * total) or frame.gain * total <= 0:
                raise InvalidParameterError("spectral_weight: effective source-mode weight sum must be finite and positive")
        if not all(np.all(c) for c in covered):
            raise InvalidParameterError(
                "spectral_acquisition: every channel and local frame must participate in the detector plan")

    def _frame_gain(self, c: int, l: int) -> float:
        g = self._models[c]._gains
        return 1.0 if g is None else float(g[l])

    @property
    def channel_ids(self) -> list:
        return list(self._ids)

    @property
    def wavelengths_vacuum_m(self) -> list:
        return [m._wavelength for m in self._models]

    @property
    def image_shape(self):
        return self._models[0].image_shape

    @property
    def reconstruction_shape(self):
        return self._models[0].reconstruction_shape

    @property
    def frame_count(self) -> int:
        return self._acquisition.frame_count

    @property
    def object_coupling(self) -> str:
        return self._coupling

    @property
    def object_count(self) -> int:
        return 1 if self._coupling == "shared_complex" else len(self._models)

    @property
    def channel_models(self) -> list:
        return list(self._models)

    @property
    def acquisition(self) -> SpectralAcquisitionPlan:
        return self._acquisition

    def _descriptor(self):
        keep = []
        descs = (N.ModelDesc * len(self._models))()
        for i, m in enumerate(self._models):
            d, k = m._descriptor()
            descs[i] = d
            keep.append(k)
        offsets = [0]
        chan, local, weight = [], [], []
        for frame in self._acquisition.frames:
            for c, l, w in frame.contributions:
                chan.append(c)
                local.append(l)
                weight.append(w)
            offsets.append(len(chan))
        arrays = dict(offsets=np.array(offsets, np.int32), chan=np.array(chan, np.int32),
                      local=np.array(local, np.int32), weight=np.array(weight, np.float64),
                      gain=np.array([f.gain for f in self._acquisition.frames], np.float64),
                      background=np.array([f.background for f in self._acquisition.frames], np.float64))
        keep.append((descs, arrays))
        sd = N.SpectralModelDesc()
        sd.channels = len(self._models)
        sd.channel_models = C.cast(descs, C.POINTER(N.ModelDesc))
        sd.object_coupling = _COUPLINGS[self._coupling]
        sd.exposures = self.frame_count
        sd.contribution_offsets = N.ptr(arrays["offsets"], C.c_int32)
        sd.contribution_channel = N.ptr(arrays["chan"], C.c_int32)
        sd.contribution_local_frame = N.ptr(arrays["local"], C.c_int32)
        sd.contribution_weight = N.ptr(arrays["weight"], C.c_double)
        sd.exposure_gain = N.ptr(arrays["gain"], C.c_double)
        sd.exposure_background = N.ptr(arrays["background"], C.c_double)
        return sd, keep

    def _check_spectra(self, values, name: str) -> np.ndarray:
        if not isinstance(values, np.ndarray) or values.dtype != np.complex128 or not values.flags.c_contiguous:
            raise InvalidParameterError(f"{name} must be a C-contiguous complex128 array")
        if values.shape != (self.object_count, *self.reconstruction_shape):
            raise InvalidShapeError(f"{name} must have shape {(self.object_count, *self.reconstruction_shape)}")
        if not np.all(np.isfinite(values)):
            raise InvalidParameterError(f"{name}: complex values must be finite")
        return values

    def forward_intensities(self, *, object_spectra) -> np.ndarray:
        """Predicted detector stack (frames, h, w) from centred spectra, on the device
        (SpectralImagePlaneModel::forward_intensity, src/model/spectral.rs:400-446)."""
        spectra = self._check_spectra(object_spectra, "object_spectra")
        h, w = self.image_shape
        out = np.zeros((self.frame_count, h, w))
        sd, keep = self._descriptor()
        ctx = N.context()
        N.check(N.library().fpm_spectral_forward(ctx.handle, C.byref(sd), N.ptr(spectra, C.c_double),
                                                 N.ptr(out, C.c_double)), ctx.handle)
        return out

    def mixing_diagnostics(self, *, relative_tolerance=None) -> SpectralMixingDiagnostics:
        """Exposure/channel mode-weight matrix and its singular values
        (src/model/spectral.rs:218-253, src/model/mixing.rs:27-72); host FP64."""
        matrix = np.zeros((self.frame_count, len(self._models)))
        for r, frame in enumerate(self._acquisition.frames):
            for c, l, w in frame.contributions:
                matrix[r, c] += frame.gain * w * self._frame_gain(c, l)
        tol = max(matrix.shape) * np.finfo(np.float64).eps if relative_tolerance is None else float(relative_tolerance)
        if not math.isfinite(tol) or tol < 0.0:
            raise InvalidParameterError("mixing_tolerance: matrix and nonnegative relative tolerance must be finite")
        values = sorted((float(v) for v in np.linalg.svd(matrix, compute_uv=False)), reverse=True)
        largest = values[0] if values else 0.0
        absolute = largest * tol
        rank = sum(1 for v in values if v > absolute)
        condition = None
        if rank == matrix.shape[1] and values and values[-1] > 0.0 and math.isfinite(largest / values[-1]):
            condition = largest / values[-1]
        return SpectralMixingDiagnostics(list(self._ids), matrix, values, rank, tol, absolute, condition)


def compile_spectral_model(*, channels, geometry: SpectralGeometry, acquisition: SpectralAcquisitionPlan, image_shape,
                           reconstruction_shape="smooth", object_coupling="independent") -> SpectralImagePlaneModel:
    """SpectralImagePlaneModel::from_experiment (src/model/spectral.rs:128-200).

    All channels share the detector pitch, so their crop grids share the
    frequency step; the union of the channels' crop bounds is then the bounds
    of their concatenated k-vectors, from which the common grid is resolved
    once. Each channel is compiled on that exact grid."""
    channels = list(channels)
    if not channels:
        raise InvalidParameterError("spectral_channels: at least one channel is required")
    _coupling(object_coupling)
    geometries = geometry._for_channels(len(channels))
    pitch = channels[0].optics.object_pixel_size
    ks = []
    for ch, g in zip(channels, geometries):
        ch.optics._validate()
        p = ch.optics.object_pixel_size
        if abs(p - pitch) > 1e-12 * max(abs(p), abs(pitch)):
            raise InvalidParameterError(
                "object_plane_pixel_pitch_m: spectral channels require the same detector sampling; resampling is not implemented")
        ks.append(g.resolve(ch.optics).k_vectors)
    union = KVectorList(np.concatenate(ks))
    shape = suggest_reconstruction_shape(channels[0].optics, union, image_shape, reconstruction_shape)
    models = [compile_model(ch.optics, KVectorList(k), image_shape, tuple(shape)) for ch, k in zip(channels, ks)]
    return SpectralImagePlaneModel([ch.channel_id for ch in channels], models, acquisition, object_coupling)


class SpectralReconstructionProblem:
    """Detector measurements with a compiled spectral model
    (python/src/spectral.rs:442-497, src/reconstruction/spectral.rs:44-92)."""

    def __init__(self, *, measurements, model: SpectralImagePlaneModel, frame_weights=None, masks=None):
        if not isinstance(measurements, MeasurementStack):
            measurements = MeasurementStack(measurements, frame_weights=frame_weights, masks=masks)
        self.measurements = measurements
        self.model = model
        if measurements.frame_count != model.frame_count or tuple(measurements.image_shape) != tuple(model.image_shape):
            raise InvalidMeasurementsError("spectral detector frame count and shape must match the compiled model")
        weights = measurements._weights
        masks_a = measurements._masks
        covered = [np.zeros(m.frame_count, bool) for m in model.channel_models]
        for f, frame in enumerate(model.acquisition.frames):
            if weights[f] == 0.0:
                continue
            if masks_a is not None and not np.any(masks_a[f]):
                raise InvalidMeasurementsError(f"positive-weight frame {f} has no unmasked pixels")
            for c, l, _ in frame.contributions:
                covered[c][l] = True
        if not all(np.all(c) for c in covered):
            raise InvalidMeasurementsError(
                "every spectral channel and local frame must participate in a positive-weight detector frame")

    @property
    def frame_count(self) -> int:
        return self.model.frame_count

    @property
    def image_shape(self):
        return self.model.image_shape

    @property
    def reconstruction_shape(self):
        return self.model.reconstruction_shape

    def _fingerprints(self):
        m = hashlib.sha256()
        for model in self.model.channel_models:
            for a in (model._start_row, model._start_col, model._offset_row, model._offset_col, model._pupil,
                      model._gains if model._gains is not None else np.ones(model.frame_count)):
                m.update(np.ascontiguousarray(a).tobytes())
        for frame in self.model.acquisition.frames:
            m.update(repr((frame.contributions, frame.gain, frame.background)).encode())
        m.update(self.model.object_coupling.encode())
        d = hashlib.sha256()
        d.update(self.measurements._data.tobytes())
        d.update(self.measurements._weights.tobytes())
        if self.measurements._masks is not None:
            d.update(self.measurements._masks.tobytes())
        return m.hexdigest(), d.hexdigest()


def _encode(a: np.ndarray):
    a = np.ascontiguousarray(a, np.complex128)
    return {"shape": list(a.shape), "re": a.real.ravel().tolist(), "im": a.imag.ravel().tolist()}


def _decode(v) -> np.ndarray:
    shape = tuple(int(x) for x in v["shape"])
    re = np.asarray(v["re"], np.float64)
    im = np.asarray(v["im"], np.float64)
    if re.size != int(np.prod(shape)) or im.size != re.size:
        raise InvalidParameterError("checkpoint array does not match its shape")
    return (re + 1j * im).reshape(shape)


@dataclass
class SpectralReconstructionCheckpoint:
    """Spectral AP state after complete passes: the stored objects' centred
    spectra, the trace, the stepping options and the schedule, plus SHA-256
    fingerprints of the compiled model and of the measurements
    (src/reconstruction/spectral_checkpoint.rs:83-135)."""

    completed_iterations: int
    elapsed_seconds: float
    spectra: np.ndarray
    trace: list
    configuration: dict
    schedule: list | None
    model_fingerprint: str
    measurement_fingerprint: str
    kind: str = "spectral_alternating_projection"
    format_version: int = FORMAT_VERSION

    def save(self, path) -> None:
        """Atomic JSON write: a temporary file in the same directory, then a rename."""
        with json_file_errors(path):
            self._save(path)

    def _save(self, path) -> None:
        path = Path(path)
        doc = dict(kind=self.kind, format_version=self.format_version, completed_iterations=self.completed_iterations,
                   elapsed_seconds=self.elapsed_seconds, spectra=[_encode(s) for s in self.spectra],
                   trace=[list(r) for r in self.trace], configuration=self.configuration, schedule=self.schedule,
                   model_fingerprint=self.model_fingerprint, measurement_fingerprint=self.measurement_fingerprint)
        fd, tmp = tempfile.mkstemp(dir=path.parent, prefix=".spectral-checkpoint-", suffix=".tmp")
        try:
            with os.fdopen(fd, "w") as f:
                json.dump(doc, f)
            os.replace(tmp, path)
        except BaseException:
            if os.path.exists(tmp):
                os.unlink(tmp)
            raise

    @staticmethod
    def load(path) -> "SpectralReconstructionCheckpoint":
        with json_file_errors(path):
            return SpectralReconstructionCheckpoint._load(path)

    @staticmethod
    def _load(path) -> "SpectralReconstructionCheckpoint":
        with open(path) as f:
            doc = json.load(f)
        if doc.get("kind") != "spectral_alternating_projection" or int(doc.get("format_version", -1)) != FORMAT_VERSION:
            raise InvalidParameterError("not a spectral alternating projection checkpoint of a supported format")
        cp = SpectralReconstructionCheckpoint(
            completed_iterations=int(doc["completed_iterations"]), elapsed_seconds=float(doc["elapsed_seconds"]),
            spectra=np.stack([_decode(s) for s in doc["spectra"]]), trace=[tuple(r) for r in doc["trace"]],
            configuration=dict(doc["configuration"]), schedule=doc["schedule"],
            model_fingerprint=doc["model_fingerprint"], measurement_fingerprint=doc["measurement_fingerprint"])
        if len(cp.trace) != cp.completed_iterations:
            raise InvalidParameterError("checkpoint trace length differs from its completed iterations")
        return cp


@dataclass
class SpectralReconstructionResult:
    """Channel-ordered fields, fixed pupils and the pass trace
    (python/src/spectral.rs:499-665). Shared coupling repeats the one object
    for every channel."""

    channel_ids: list
    wavelengths_vacuum_m: list
    object_coupling: str
    _objects: np.ndarray
    _spectra: np.ndarray
    _pupils: np.ndarray
    trace: list
    completed_iterations: int
    checkpoint: SpectralReconstructionCheckpoint | None = None
    runtime: dict = field(default_factory=dict)

    @property
    def object(self) -> np.ndarray:
        return self._objects.copy()

    @property
    def object_spectrum(self) -> np.ndarray:
        return self._spectra.copy()

    @property
    def amplitude(self) -> np.ndarray:
        return np.abs(self._objects)

    @property
    def phase(self) -> np.ndarray:
        return np.angle(self._objects)

    @property
    def pupils(self) -> np.ndarray:
        return self._pupils.copy()


class SpectralAlternatingProjection:
    """Object-only alternating projection for separate or multiplexed
    narrowband exposures (src/algorithms/spectral.rs:86-271); pupils, source
    powers and detector calibration stay fixed."""

    def __init__(self, *, iterations=50, object_step=1.0, batch_size=1, epsilon=1e-10, loss_type="amplitude_mse"):
        if loss_type not in _LOSSES:
            raise ValueError("loss_type must be amplitude_mse, intensity_mse, poisson_nll, or huber_amplitude")
        self.iterations, self.object_step, self.batch_size = iterations, object_step, batch_size
        self.epsilon, self.loss_type = epsilon, loss_type

    def _params(self) -> N.SpectralParams:
        for name in ("object_step", "epsilon"):
            v = float(getattr(self, name))
            if not math.isfinite(v) or v <= 0.0:
                raise InvalidParameterError(f"{name} must be finite and positive")
        if int(self.iterations) <= 0:
            raise InvalidParameterError("iterations must be positive")
        if int(self.batch_size) <= 0:
            raise InvalidParameterError("batch_size must be positive")
        return N.SpectralParams(int(self.iterations), int(self.batch_size), _LOSSES[self.loss_type],
                                float(self.object_step), float(self.epsilon))

    def _configuration(self) -> dict:
        return dict(object_step=float(self.object_step), batch_size=int(self.batch_size), epsilon=float(self.epsilon),
                    loss_type=self.loss_type)

    def _batch(self, problems):
        """Descriptors, result arrays and their keep-alive list for a batch call."""
        params = self._params()
        keep = []
        models = (N.SpectralModelDesc * len(problems))()
        meas = (N.MeasurementDesc * len(problems))()
        outs = (N.SpectralResultDesc * len(problems))()
        arrays = []
        for i, p in enumerate(problems):
            sd, k = p.model._descriptor()
            keep.append(k)
            models[i] = sd
            m = meas[i]
            m.frames = p.measurements.frame_count
            m.measurements = N.ptr(p.measurements._data, C.c_double)
            m.frame_weights = N.ptr(p.measurements._weights, C.c_double)
            m.masks = N.ptr(p.measurements._masks, C.c_uint8)
            shape = (p.model.object_count, *p.model.reconstruction_shape)
            a = dict(objects=np.zeros(shape, np.complex128), spectra=np.zeros(shape, np.complex128),
                     objectives=np.zeros(int(self.iterations)))
            outs[i].objects = N.ptr(a["objects"], C.c_double)
            outs[i].object_spectra = N.ptr(a["spectra"], C.c_double)
            outs[i].objectives = N.ptr(a["objectives"], C.c_double)
            arrays.append(a)
        return params, models, meas, outs, arrays, keep

    def _results(self, problems, arrays, elapsed) -> list:
        results = []
        for p, a in zip(problems, arrays):
            model = p.model
            index = [0 if model.object_coupling == "shared_complex" else c for c in range(len(model.channel_ids))]
            results.append(SpectralReconstructionResult(
                channel_ids=model.channel_ids, wavelengths_vacuum_m=model.wavelengths_vacuum_m,
                object_coupling=model.object_coupling, _objects=a["objects"][index], _spectra=a["spectra"][index],
                _pupils=np.stack([m.pupil for m in model.channel_models]),
                trace=[(it + 1, float(a["objectives"][it]), elapsed) for it in range(int(self.iterations))],
                completed_iterations=int(self.iterations),
                runtime=dict(elapsed_seconds=elapsed, algorithm="SpectralAlternatingProjection")))
        return results

    def run_many(self, *, problems) -> list:
        """Independent problems in one device call (fpm_spectral_run_batch):
        one engine launch per tile size, one thread-block cluster per problem,
        acquisition order and measured-amplitude initialisation. Each result
        equals the problem's own run()."""
        problems = list(problems)
        if not problems:
            return []
        params, models, meas, outs, arrays, keep = self._batch(problems)
        ctx = N.context()
        started = time.perf_counter()
        N.check(N.library().fpm_spectral_run_batch(ctx.handle, len(problems), models, meas, C.byref(params), outs),
                ctx.handle)
        return self._results(problems, arrays, time.perf_counter() - started)

    def submit_many(self, *, problems) -> "SpectralJob":
        """run_many without the wait (fpm_spectral_run_batch_submit): the
        uploads are queued and the call returns; SpectralJob.done() polls and
        SpectralJob.wait() returns the results."""
        problems = list(problems)
        if not problems:
            raise InvalidParameterError("submit_many needs at least one problem")
        params, models, meas, outs, arrays, keep = self._batch(problems)
        ctx = N.context()
        handle = C.c_void_p()
        started = time.perf_counter()
        N.check(N.library().fpm_spectral_run_batch_submit(ctx.handle, len(problems), models, meas, C.byref(params),
                                                          outs, C.byref(handle)), ctx.handle)
        return SpectralJob(handle, self, problems, arrays, outs, started)

    def run(self, *, problem: SpectralReconstructionProblem, initial_objects=None, frame_order=None, seed=None,
            resume=None, checkpoint_directory=None, checkpoint_every=1) -> SpectralReconstructionResult:
        """Runs the passes on the device and returns owned channel records
        (python/src/spectral.rs:764-822, SpectralRunner::run
        src/reconstruction/spectral.rs:494-642)."""
        if frame_order is not None and seed is not None:
            raise ValueError("frame_order and seed are mutually exclusive")
        if seed is not None:
            raise UnsupportedError(
                "the random spectral schedule depends on the reference's ChaCha12 stream and is not supported on the GB300 device path")
        params = self._params()
        if int(checkpoint_every) <= 0 or (checkpoint_directory is not None and not str(checkpoint_directory)):
            raise InvalidParameterError("checkpoint_options: interval must be positive and directory nonempty")
        model = problem.model
        k = model.object_count
        mh, mw = model.reconstruction_shape
        order = None
        if frame_order is not None:
            order = np.ascontiguousarray(frame_order, dtype=np.int32)
            if sorted(order.tolist()) != list(range(model.frame_count)):
                raise InvalidParameterError("explicit order must be a permutation of all detector frames")
        start, trace, elapsed0, resume_spectra = 0, [], 0.0, None
        fingerprints = problem._fingerprints()
        if resume is not None:
            if initial_objects is not None:
                raise InvalidParameterError("initial_objects cannot be combined with a checkpoint")
            if (resume.model_fingerprint, resume.measurement_fingerprint) != fingerprints:
                raise InvalidParameterError("resume_from: the checkpoint belongs to another model or measurement set")
            if resume.configuration != self._configuration():
                raise InvalidParameterError("resume_from: solver stepping options or schedule changed")
            saved = None if resume.schedule is None else list(resume.schedule)
            if frame_order is not None and saved != order.tolist():
                raise InvalidParameterError("resume_from: solver stepping options or schedule changed")
            if saved is not None:
                order = np.ascontiguousarray(saved, dtype=np.int32)
            if int(self.iterations) < resume.completed_iterations:
                raise InvalidParameterError("iterations: total target cannot precede checkpoint iterations")
            start = resume.completed_iterations
            trace = list(resume.trace)
            elapsed0 = resume.elapsed_seconds
            resume_spectra = model._check_spectra(np.ascontiguousarray(resume.spectra, np.complex128), "checkpoint spectra")
        init = None
        if initial_objects is not None:
            init = model._check_spectra(initial_objects, "initial_objects")
        total = int(self.iterations)
        ends = sorted({e for e in range(start + 1, total) if checkpoint_directory is not None and e % int(checkpoint_every) == 0}
                      | {total})
        sd, keep = model._descriptor()
        ms = N.MeasurementDesc()
        ms.frames = problem.measurements.frame_count
        ms.measurements = N.ptr(problem.measurements._data, C.c_double)
        ms.frame_weights = N.ptr(problem.measurements._weights, C.c_double)
        ms.masks = N.ptr(problem.measurements._masks, C.c_uint8)
        ctx = N.context()
        objects = np.zeros((k, mh, mw), np.complex128)
        spectra = np.zeros((k, mh, mw), np.complex128)
        started = time.perf_counter()
        done = start
        checkpoint = None
        for end in ends:
            params.iterations = end
            objectives = np.zeros(max(end - done, 1))
            N.check(N.library().fpm_spectral_run(
                ctx.handle, C.byref(sd), C.byref(ms), C.byref(params), N.ptr(order, C.c_int32),
                N.ptr(init if resume_spectra is None else None, C.c_double),
                N.ptr(resume_spectra, C.c_double), done,
                N.ptr(objects, C.c_double), N.ptr(spectra, C.c_double), N.ptr(objectives, C.c_double)), ctx.handle)
            elapsed = elapsed0 + time.perf_counter() - started
            trace.extend((it + 1, float(objectives[it - done]), elapsed) for it in range(done, end))
            done = end
            resume_spectra = spectra.copy()
            checkpoint = SpectralReconstructionCheckpoint(
                completed_iterations=end, elapsed_seconds=elapsed, spectra=resume_spectra, trace=list(trace),
                configuration=self._configuration(), schedule=None if order is None else order.tolist(),
                model_fingerprint=fingerprints[0], measurement_fingerprint=fingerprints[1])
            if checkpoint_directory is not None and (end % int(checkpoint_every) == 0 or end == total):
                directory = Path(checkpoint_directory)
                directory.mkdir(parents=True, exist_ok=True)
                checkpoint.save(directory / f"spectral_checkpoint_{end:05d}.json")
        index = [0 if model.object_coupling == "shared_complex" else c for c in range(len(model.channel_ids))]
        pupils = np.stack([m.pupil for m in model.channel_models])
        return SpectralReconstructionResult(
            channel_ids=model.channel_ids, wavelengths_vacuum_m=model.wavelengths_vacuum_m,
            object_coupling=model.object_coupling, _objects=objects[index], _spectra=spectra[index], _pupils=pupils,
            trace=trace, completed_iterations=total, checkpoint=checkpoint,
            runtime=dict(elapsed_seconds=elapsed0 + time.perf_counter() - started, algorithm="SpectralAlternatingProjection"))


class SpectralJob:
    """Spectral requests queued by SpectralAlternatingProjection.submit_many."""

    def __init__(self, handle, solver, problems, arrays, outs, submitted):
        self._handle = handle
        self._solver = solver
        self._problems = problems
        self._arrays = arrays
        self._outs = outs  # the result descriptors the device writes through
        self._submitted = submitted
        self._finished_at = None
        self._out = None
        N.own(self)

    _release_order = 0

    def _release_native(self) -> None:
        handle = getattr(self, "_handle", None)
        if handle:
            N.library().fpm_job_wait(handle)
            N.library().fpm_job_destroy(handle)
            self._handle = None

    def done(self) -> bool:
        if self._out is not None:
            return True
        flag = C.c_int32(0)
        N.check(N.library().fpm_job_poll(self._handle, C.byref(flag)), N.context().handle)
        if flag.value:
            self._collect()
        return bool(flag.value)

    def wait(self) -> list:
        if self._out is None:
            N.check(N.library().fpm_job_wait(self._handle), N.context().handle)
            self._collect()
        return self._out

    @property
    def finished_at(self):
        """time.perf_counter() when done() or wait() first saw the job finished."""
        return self._finished_at

    def _collect(self) -> None:
        self._finished_at = time.perf_counter()
        self._out = self._solver._results(self._problems, self._arrays, self._finished_at - self._submitted)

    def __del__(self):
        handle = getattr(self, "_handle", None)
        if handle and not N.closed():
            N.library().fpm_job_destroy(handle)
        self._handle = None
