"""ctypes binding of libfpm_gpu.so (include/fpm_gpu.h).

The library is built in-tree by fpm-rs_gb300/build.py. Loading never falls
back to another implementation: a missing library raises ImportError with
the build command, and device entry points raise FpmError when no Blackwell
GPU is available.
"""

from __future__ import annotations

import atexit
import ctypes as C
import os
import threading
import weakref

import numpy as np

from . import errors

PACKAGE_ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
LIB_PATH = os.environ.get("FPM_GPU_LIBRARY", os.path.join(PACKAGE_ROOT, "libfpm_gpu.so"))

EXPORTED = (
    "fpm_create", "fpm_destroy", "fpm_last_error", "fpm_global_last_error",
    "fpm_planar_led_kvectors", "fpm_suggest_shape", "fpm_compile_model", "fpm_intensity_loss",
    "fpm_fft2", "fpm_forward_stack", "fpm_simulate_stack", "fpm_problem_create", "fpm_problem_create_batch", "fpm_problem_destroy",
    "fpm_run", "fpm_run_batch", "fpm_run_batch_host", "fpm_run_batch_resumable", "fpm_last_run_stats",
    "fpm_spectral_run", "fpm_spectral_run_batch", "fpm_spectral_forward",
    "fpm_run_batch_submit", "fpm_spectral_run_batch_submit", "fpm_job_poll", "fpm_job_wait", "fpm_job_stats", "fpm_job_destroy",
    "fpm_plan_create", "fpm_plan_launch", "fpm_plan_wait", "fpm_plan_collect", "fpm_plan_destroy",
    "fpm_server_create", "fpm_server_submit", "fpm_server_poll", "fpm_server_wait", "fpm_server_stats_get",
    "fpm_server_destroy", "fpm_set_engine_grid", "fpm_engine_max_clusters", "fpm_set_engine_shape",
    "fpm_set_engine_ctas",
)


class Optics(C.Structure):
    _fields_ = [
        ("wavelength_vacuum_m", C.c_double), ("objective_na", C.c_double),
        ("magnification", C.c_double), ("camera_pixel_size", C.c_double),
        ("illumination_refractive_index", C.c_double),
        ("objective_medium_refractive_index", C.c_double),
        ("has_defocus", C.c_int32), ("defocus_distance", C.c_double),
        ("has_aberration", C.c_int32), ("astigmatism", C.c_double), ("coma", C.c_double),
        ("spherical", C.c_double), ("edge_apodization", C.c_double),
    ]


class ModelDesc(C.Structure):
    _fields_ = [
        ("image_height", C.c_int32), ("image_width", C.c_int32),
        ("recon_height", C.c_int32), ("recon_width", C.c_int32),
        ("sources", C.c_int32),
        ("crop_start_row", C.POINTER(C.c_int64)), ("crop_start_col", C.POINTER(C.c_int64)),
        ("offset_row", C.POINTER(C.c_double)), ("offset_col", C.POINTER(C.c_double)),
        ("pupil", C.POINTER(C.c_double)), ("support", C.POINTER(C.c_uint8)),
        ("frame_gains", C.POINTER(C.c_double)), ("background", C.POINTER(C.c_double)),
        ("background_len", C.c_int64),
        ("kx", C.POINTER(C.c_double)), ("ky", C.POINTER(C.c_double)),
    ]


class MeasurementDesc(C.Structure):
    _fields_ = [
        ("frames", C.c_int32), ("measurements", C.POINTER(C.c_double)),
        ("frame_weights", C.POINTER(C.c_double)), ("masks", C.POINTER(C.c_uint8)),
    ]


class AlgorithmParams(C.Structure):
    _fields_ = [
        ("algorithm", C.c_int32), ("iterations", C.c_int32), ("batch_size", C.c_int32),
        ("loss_type", C.c_int32), ("schedule", C.c_int32),
        ("object_step", C.c_double), ("epsilon", C.c_double), ("stability", C.c_double),
        ("momentum_interval", C.c_int32), ("momentum_friction", C.c_double),
        ("momentum_feedback", C.c_double),
        ("recover_pupil", C.c_int32), ("constrain_pupil_support", C.c_int32),
        ("pupil_step", C.c_double),
        ("recover_frame_gains", C.c_int32), ("recover_background", C.c_int32),
        ("poisson_truncation", C.c_int32), ("poisson_truncation_threshold", C.c_double),
        ("progress_threshold", C.c_double), ("reduction_factor", C.c_double), ("minimum_object_step", C.c_double),
        ("object_tv_weight", C.c_double), ("object_tv_epsilon", C.c_double), ("pupil_smoothing_weight", C.c_double),
        ("recover_illumination", C.c_int32), ("illumination_step", C.c_double),
        ("illumination_finite_difference", C.c_double), ("maximum_illumination_correction", C.c_double),
        ("compensated_accumulation", C.c_int32),
        ("gain_step", C.c_double), ("gain_min", C.c_double), ("gain_max", C.c_double),
        ("background_step", C.c_double), ("background_min", C.c_double), ("background_max", C.c_double),
    ]


class CameraDesc(C.Structure):
    _fields_ = [
        ("photons_per_pixel", C.c_double), ("gain_counts_per_electron", C.c_double), ("offset_counts", C.c_double),
        ("read_noise_electrons", C.c_double), ("dark_current_electrons", C.c_double),
        ("shot_noise", C.c_int32), ("quantize", C.c_int32), ("maximum_count", C.c_double),
        ("pixel_sensitivity", C.POINTER(C.c_double)), ("bad_pixels", C.POINTER(C.c_int64)),
        ("bad_pixel_count", C.c_int64), ("bad_pixel_value", C.c_double),
    ]


class StateDesc(C.Structure):
    _fields_ = [
        ("completed_iterations", C.c_int32), ("momentum_counter", C.c_int32),
        ("object_spectrum", C.POINTER(C.c_double)), ("pupil", C.POINTER(C.c_double)),
        ("velocity", C.POINTER(C.c_double)), ("anchor", C.POINTER(C.c_double)),
        ("objectives", C.POINTER(C.c_double)),
        ("illumination_corrections", C.POINTER(C.c_double)),
    ]


class SpectralModelDesc(C.Structure):
    _fields_ = [
        ("channels", C.c_int32), ("channel_models", C.POINTER(ModelDesc)), ("object_coupling", C.c_int32),
        ("exposures", C.c_int32), ("contribution_offsets", C.POINTER(C.c_int32)),
        ("contribution_channel", C.POINTER(C.c_int32)), ("contribution_local_frame", C.POINTER(C.c_int32)),
        ("contribution_weight", C.POINTER(C.c_double)), ("exposure_gain", C.POINTER(C.c_double)),
        ("exposure_background", C.POINTER(C.c_double)),
    ]


class SpectralParams(C.Structure):
    _fields_ = [("iterations", C.c_int32), ("batch_size", C.c_int32), ("loss_type", C.c_int32),
                ("object_step", C.c_double), ("epsilon", C.c_double)]


class SpectralResultDesc(C.Structure):
    _fields_ = [("objects", C.POINTER(C.c_double)), ("object_spectra", C.POINTER(C.c_double)),
                ("objectives", C.POINTER(C.c_double))]


class ResultDesc(C.Structure):
    _fields_ = [
        ("object", C.POINTER(C.c_double)), ("object_spectrum", C.POINTER(C.c_double)),
        ("pupil", C.POINTER(C.c_double)), ("objectives", C.POINTER(C.c_double)),
        ("completed_iterations", C.c_int32),
        ("illumination_corrections", C.POINTER(C.c_double)),
        ("frame_gains", C.POINTER(C.c_double)), ("background", C.POINTER(C.c_double)),
    ]


class RunStats(C.Structure):
    _fields_ = [
        ("kernel_launches", C.c_int32), ("engine_launches", C.c_int32), ("run_ms", C.c_double),
        ("engine_ms_sum", C.c_double), ("engine_span_ms", C.c_double), ("engine_bytes", C.c_double),
        ("buckets", C.c_int32), ("bucket_size", C.c_int32 * 8), ("bucket_tiles", C.c_int32 * 8),
        ("bucket_end_ms", C.c_double * 8),
        ("host_first_launch_ms", C.c_double), ("host_scan_ms", C.c_double), ("host_upload_ms", C.c_double),
        ("host_call_ms", C.c_double),
        ("host_chunks", C.c_int32), ("host_done_tiles", C.c_int32 * 16), ("host_done_ms", C.c_double * 16),
    ]


class ServerConfig(C.Structure):
    _fields_ = [("hbm_budget_bytes", C.c_int64), ("max_batch", C.c_int32), ("batch_window_ms", C.c_double),
                ("max_queue", C.c_int64)]


class RequestInfo(C.Structure):
    _fields_ = [("submit_ms", C.c_double), ("admit_ms", C.c_double), ("start_ms", C.c_double),
                ("done_ms", C.c_double), ("footprint_bytes", C.c_int64), ("status", C.c_int32),
                ("message", C.c_char * 256)]


class ServerStats(C.Structure):
    _fields_ = [("submitted", C.c_int64), ("admitted", C.c_int64), ("completed", C.c_int64),
                ("rejected", C.c_int64), ("batches", C.c_int64), ("in_use_bytes", C.c_int64),
                ("peak_bytes", C.c_int64), ("waiting", C.c_int64), ("in_flight_batches", C.c_int64)]


_lib = None
_lock = threading.RLock()


def library() -> C.CDLL:
    """Loads libfpm_gpu.so, raising ImportError when it has not been built."""
    global _lib
    if _lib is None:
        with _lock:
            if _lib is None:
                if not os.path.exists(LIB_PATH):
                    raise ImportError(
                        f"{LIB_PATH} is missing; build it with `python fpm-rs_gb300/build.py` "
                        "(there is no CPU implementation of this path)")
                lib = C.CDLL(LIB_PATH)
                lib.fpm_global_last_error.restype = C.c_char_p
                for name in EXPORTED:
                    getattr(lib, name)
                _lib = lib
    return _lib


def ptr(array, ctype):
    if array is None:
        return C.POINTER(ctype)()
    return array.ctypes.data_as(C.POINTER(ctype))


def check(status: int, context=None) -> None:
    if status == 0:
        return
    lib = library()
    if context is not None:
        buf = C.create_string_buffer(2048)
        lib.fpm_last_error(context, buf, len(buf))
        message = buf.value.decode(errors="replace")
    else:
        message = lib.fpm_global_last_error().decode(errors="replace")
    raise errors.from_status(status, message)


class Context:
    """A device context of libfpm_gpu (one per process and device)."""

    def __init__(self, device: int = 0):
        self._lib = library()
        handle = C.c_void_p()
        check(self._lib.fpm_create(C.byref(handle), int(device)))
        self.handle = handle
        self.device = device

    def close(self) -> None:
        if self.handle:
            self._lib.fpm_destroy(self.handle)
            self.handle = C.c_void_p()

    def __del__(self):
        try:
            if not _closed:
                self.close()
        except Exception:
            pass


_context: Context | None = None

# Objects that hold device handles of the process context (problems, submitted
# jobs). At interpreter exit they are released before the context is
# destroyed: jobs first (each waits for its device work), then problems, and
# handles released after that are left alone.
_owners: "weakref.WeakSet" = weakref.WeakSet()
_closed = False


def own(obj) -> None:
    _owners.add(obj)


def closed() -> bool:
    return _closed


def _shutdown() -> None:
    global _closed
    for obj in sorted(list(_owners), key=lambda o: getattr(o, "_release_order", 1)):
        try:
            obj._release_native()
        except Exception:
            pass
    if _context is not None:
        _context.close()
    _closed = True


atexit.register(_shutdown)


def context() -> Context:
    global _context
    if _context is None:
        with _lock:
            if _context is None:
                ctx = Context(int(os.environ.get("FPM_DEVICE", "0")))
                _apply_tuning(ctx)
                _context = ctx
    return _context


def _apply_tuning(ctx: "Context") -> None:
    """The committed frame-engine shapes and launch grids (tuning.json), if any."""
    import json

    try:
        with open(os.path.join(PACKAGE_ROOT, "tuning.json")) as handle:
            table = json.load(handle)
    except (OSError, ValueError):
        return
    grid = table.get("grid", {})
    for n, shape in table.get("shape", {}).items():
        check(ctx._lib.fpm_set_engine_shape(ctx.handle, int(n), int(shape)), ctx.handle)
    for n, ctas in table.get("ctas", {}).items():
        check(ctx._lib.fpm_set_engine_ctas(ctx.handle, int(n), int(ctas)), ctx.handle)
    for n in (32, 64, 128, 256):
        clusters = int(grid.get(str(n), 0))
        if clusters:
            check(ctx._lib.fpm_set_engine_grid(ctx.handle, n, clusters), ctx.handle)


def c128(a) -> np.ndarray:
    return np.ascontiguousarray(a, dtype=np.complex128)


def f64(a) -> np.ndarray:
    return np.ascontiguousarray(a, dtype=np.float64)
