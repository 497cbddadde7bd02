"""fpm_rs: GB300-native drop-in for fpm-rs's image-plane forward model and
reconstruction inner loop.

The public names follow the reference's Python bindings (python/fpm_rs);
the numerical work runs in libfpm_gpu.so, hand-written CUDA for sm_103a,
reached through the C ABI declared in include/fpm_gpu.h.
"""

from __future__ import annotations

import ctypes as _C

import numpy as _np

from . import _native, tuning
from .errors import (DatasetError, DeviceError, FpmError, FpmIoError, FrameOutOfRangeError, InvalidMeasurementsError,
                     InvalidModelError, InvalidParameterError, InvalidShapeError, LengthMismatchError, NumericalError,
                     SerializationError, ServerBusyError, UnsupportedError)
from .experiment import (ArrayPose, CameraModel, DirectionList, Illumination, KVectorList, Optics, PlanarLEDArray,
                         PupilAberration, ResolvedFrame, ResolvedIllumination, ResolvedSources, SourceContribution,
                         SourcePositionList)
from .model import ImagePlaneModel, compile_camera_model, compile_model, suggest_reconstruction_shape
from .objective import intensity_loss
from .callbacks import (Callback, CsvLogger, IterationCallback, ProgressLogger, SaveImageEvery, SavePupilEvery,
                        SaveResidualsEvery, StepContext, StopOnPlateau)
from .checkpoint import CheckpointEvery, ReconstructionCheckpoint
from .reconstruction import (AdaptiveAlternatingProjection, AlternatingProjection, Epry, Fpie, GradientDescent, Mpie,
                             ReconstructionProblem,
                             ReconstructionResult, Request, RunPlan, RuntimeInfo, Job, Server, capture_batch, last_run_stats, run_batch,
                             submit_batch)
from .simulation import (IlluminationAcquisitionErrors, MeasurementStack, SimulationResult, SyntheticObject,
                         forward_intensities, simulate)
from .spectral import (SpectralAcquisitionPlan, SpectralAlternatingProjection, SpectralChannel, SpectralFrame,
                       SpectralGeometry, SpectralImagePlaneModel, SpectralMixingDiagnostics,
                       SpectralJob, SpectralReconstructionCheckpoint, SpectralReconstructionProblem,
                       SpectralReconstructionResult, compile_spectral_model)


def fft2(values, *, inverse: bool = False):
    """Backend::fft2 (src/backend/traits.rs:123-131) on the GPU in FP64.

    Forward transforms are scaled by 1/(height*width); inverse transforms are
    not. Returns a new complex128 array.
    """
    out = _np.array(values, dtype=_np.complex128, order="C", copy=True)
    if out.ndim != 2:
        raise InvalidShapeError("fft2 expects a 2-D array")
    ctx = _native.context()
    _native.check(_native.library().fpm_fft2(ctx.handle, _native.ptr(out, _C.c_double), out.shape[0],
                                             out.shape[1], int(bool(inverse))), ctx.handle)
    return out


__all__ = [
    "AdaptiveAlternatingProjection", "AlternatingProjection", "ArrayPose", "CameraModel", "CheckpointEvery", "DeviceError",
    "DirectionList", "SpectralAcquisitionPlan", "SpectralAlternatingProjection", "SpectralChannel", "SpectralFrame",
    "SpectralGeometry", "SpectralImagePlaneModel", "SpectralMixingDiagnostics", "SpectralReconstructionCheckpoint",
    "SpectralReconstructionProblem", "SpectralReconstructionResult", "compile_spectral_model", "Epry", "Fpie", "FpmError",
    "FrameOutOfRangeError", "GradientDescent", "Illumination", "ImagePlaneModel", "InvalidMeasurementsError",
    "InvalidModelError", "InvalidParameterError", "InvalidShapeError", "KVectorList", "LengthMismatchError",
    "MeasurementStack", "Mpie", "NumericalError", "Optics", "PlanarLEDArray", "PupilAberration",
    "ReconstructionCheckpoint", "ReconstructionProblem", "ReconstructionResult", "ResolvedSources", "RuntimeInfo",
    "SimulationResult",
    "UnsupportedError", "compile_camera_model", "compile_model", "fft2", "forward_intensities", "last_run_stats",
    "run_batch", "simulate", "suggest_reconstruction_shape", "Job", "submit_batch", "SpectralJob", "RunPlan",
    "capture_batch", "Server", "Request", "ServerBusyError", "Callback", "CsvLogger", "IterationCallback",
    "ProgressLogger", "SaveImageEvery", "SavePupilEvery", "SaveResidualsEvery", "StepContext", "StopOnPlateau",
    "intensity_loss", "ResolvedFrame", "ResolvedIllumination", "SourceContribution", "SourcePositionList",
    "SyntheticObject", "IlluminationAcquisitionErrors", "DatasetError", "FpmIoError", "SerializationError",
]
