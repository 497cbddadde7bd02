"""Reconstruction problems, algorithms and results on the GB300 device backend.

Mirrors python/src/reconstruction.rs (ReconstructionProblem 88-153,
run_algorithm 1107-1141, AlternatingProjection 2238-2286, Mpie 2500-2560,
Epry 2612-2680, GradientDescent 2831-2908) and python/fpm_rs/__init__.pyi
(ReconstructionResult 2959-3000, _Algorithm.run 3312-3340). Every
reconstruction runs to completion in libfpm_gpu; the Python layer only
validates arguments, uploads arrays and wraps results.
"""

from __future__ import annotations

import ctypes as C
import math
import time
from dataclasses import dataclass, field

import numpy as np

from . import _native as N
from .callbacks import Callback, StepContext, plan_segment
from .checkpoint import ReconstructionCheckpoint
from .errors import (InvalidMeasurementsError, InvalidModelError, InvalidParameterError, InvalidShapeError,
                     UnsupportedError)
from .model import ImagePlaneModel
from .simulation import MeasurementStack

_LOSSES = {"amplitude_mse": 0, "intensity_mse": 1, "poisson_nll": 2, "huber_amplitude": 3}
_SCHEDULES = {"sequential": 0, "brightfield_first": 1, "spiral_out": 2, "snr_weighted": 3}
_ALG = {"ap": 0, "fpie": 1, "mpie": 2, "epry": 3, "gd": 4, "adaptive_ap": 5}


def _loss(value: str) -> int:
    if value not in _LOSSES:
        raise ValueError("loss_type must be amplitude_mse, intensity_mse, poisson_nll, or huber_amplitude")
    return _LOSSES[value]


class ReconstructionProblem:
    """Validated pairing of measurements and a compiled image-plane model.

    The measurement stack is uploaded to the device on first use and stays
    resident for later runs of the same problem.
    """

    def __init__(self, measurements, model: ImagePlaneModel, *, frame_weights=None, masks=None, name=None):
        if not isinstance(measurements, MeasurementStack):
            measurements = MeasurementStack(measurements, frame_weights=frame_weights, masks=masks)
        self.measurements = measurements
        self.model = model
        self.name = name
        self._handle = None
        self._keep = None
        if measurements.frame_count != model.frame_count:
            raise InvalidModelError(
                f"{measurements.frame_count} measurement frames but {model.frame_count} model frames")
        if tuple(measurements.image_shape) != tuple(model.image_shape):
            raise InvalidShapeError(
                f"measurement shape {tuple(measurements.image_shape)} differs from model image shape {model.image_shape}")
        weights = measurements._weights
        if not np.any(weights > 0):
            raise InvalidMeasurementsError("at least one frame must have positive weight")
        if measurements._masks is not None:
            empty = np.flatnonzero((weights > 0) & ~measurements._masks.reshape(len(weights), -1).any(axis=1))
            if empty.size:
                raise InvalidMeasurementsError(f"positive-weight frame {int(empty[0])} has no unmasked pixels")

    @property
    def frame_count(self) -> int:
        return self.measurements.frame_count

    @property
    def image_shape(self):
        return self.model.image_shape

    @property
    def reconstruction_shape(self):
        return self.model.reconstruction_shape

    def _descriptors(self):
        desc, keep = self.model._descriptor()
        m = N.MeasurementDesc()
        m.frames = self.measurements.frame_count
        m.measurements = N.ptr(self.measurements._data, C.c_double)
        m.frame_weights = N.ptr(self.measurements._weights, C.c_double)
        m.masks = N.ptr(self.measurements._masks, C.c_uint8)
        return desc, m, keep

    def device_handle(self):
        """Uploads the problem (once) and returns its opaque device handle."""
        if self._handle is None:
            ctx = N.context()
            desc, m, keep = self._descriptors()
            handle = C.c_void_p()
            N.check(N.library().fpm_problem_create(ctx.handle, C.byref(desc), C.byref(m), C.byref(handle)),
                    ctx.handle)
            self._handle = handle
            self._ctx = ctx
            N.own(self)
        return self._handle

    def release(self) -> None:
        """Frees the problem's device buffers (refused while a submitted job uses them)."""
        if self._handle is not None and not N.closed():
            N.check(N.library().fpm_problem_destroy(self._handle), N.context().handle)
        self._handle = None

    _release_order = 1

    def _release_native(self) -> None:
        self.release()

    def __del__(self):
        try:
            self.release()
        except Exception:
            pass


@dataclass
class RuntimeInfo:
    elapsed_seconds: float
    completed_iterations: int
    stopped_early: bool
    algorithm: str


@dataclass
class ReconstructionResult:
    """Owned reconstruction products (python/fpm_rs/__init__.pyi:2959-3000)."""

    object: np.ndarray
    object_spectrum: np.ndarray
    recovered_pupil: np.ndarray
    pupil_support: np.ndarray
    trace: list
    runtime: RuntimeInfo
    recovered_frame_gains: np.ndarray | None = None
    recovered_background: np.ndarray | None = None
    calibrated_illumination: np.ndarray | None = None
    physical_illumination_calibration: object = None
    calibrated_model: object = None
    algorithm_metrics: list = field(default_factory=list)
    metadata: dict = field(default_factory=dict)

    @property
    def amplitude(self) -> np.ndarray:
        return np.abs(self.object)

    @property
    def phase(self) -> np.ndarray:
        return np.angle(self.object)

    @property
    def final_objective(self):
        return self.trace[-1][1] if self.trace else None

    @property
    def scalar_diagnostics(self) -> dict:
        return {} if not self.trace else {"final_objective": self.trace[-1][1]}


class _Algorithm:
    _name = ""
    _code = 0

    def _params(self, schedule: str) -> N.AlgorithmParams:
        raise NotImplementedError

    def _schedule(self, schedule: str) -> int:
        if schedule == "random":
            raise UnsupportedError(
                "the random schedule depends on the reference's ChaCha12 stream and is not supported on the GB300 device path")
        if schedule not in _SCHEDULES:
            raise ValueError("schedule must be sequential, brightfield_first, spiral_out, random, or snr_weighted")
        return _SCHEDULES[schedule]

    _compensated = False

    def compensated(self, enabled: bool = True):
        """Accumulates the per-frame updates into the complex64 object (or the
        mini-batch gradient) with compensated (Kahan) summation; returns self."""
        self._compensated = bool(enabled)
        return self

    def run(self, problem: ReconstructionProblem, *, callbacks=None, resume_from=None, schedule="sequential",
            schedule_seed=0) -> ReconstructionResult:
        """Run the reconstruction on the GPU and return host results."""
        return run_batch(self, [problem], callbacks=callbacks, resume_from=resume_from, schedule=schedule)[0]


def _base_params(alg: _Algorithm, schedule: str, iterations, object_step, batch_size, epsilon, loss_type):
    p = N.AlgorithmParams()
    p.algorithm = alg._code
    p.iterations = int(iterations)
    p.batch_size = int(batch_size)
    p.loss_type = _loss(loss_type)
    p.schedule = alg._schedule(schedule)
    p.object_step = float(object_step)
    p.epsilon = float(epsilon)
    p.constrain_pupil_support = 1
    p.compensated_accumulation = int(alg._compensated)
    return p


class AlternatingProjection(_Algorithm):
    _name = "AlternatingProjection"
    _code = _ALG["ap"]

    def __init__(self, *, iterations=50, object_step=1.0, batch_size=1, epsilon=1e-10, loss_type="amplitude_mse"):
        _loss(loss_type)
        self.iterations, self.object_step, self.batch_size = iterations, object_step, batch_size
        self.epsilon, self.loss_type = epsilon, loss_type

    def _params(self, schedule):
        return _base_params(self, schedule, self.iterations, self.object_step, self.batch_size, self.epsilon,
                            self.loss_type)


class AdaptiveAlternatingProjection(_Algorithm):
    """AP with the adaptive step rule of Zuo et al.
    (src/algorithms/adaptive_alternating_projection.rs:96-126): after two
    passes, a pass whose relative objective progress is at most
    progress_threshold multiplies the step by reduction_factor, not below
    minimum_object_step. The objective is always amplitude MSE."""

    _name = "AdaptiveAlternatingProjection"
    _code = _ALG["adaptive_ap"]

    def __init__(self, *, iterations=50, initial_object_step=1.0, progress_threshold=0.01, reduction_factor=0.5,
                 minimum_object_step=0.001, batch_size=1, epsilon=1e-10):
        self.iterations, self.initial_object_step = iterations, initial_object_step
        self.progress_threshold, self.reduction_factor = progress_threshold, reduction_factor
        self.minimum_object_step, self.batch_size, self.epsilon = minimum_object_step, batch_size, epsilon

    def _params(self, schedule):
        p = _base_params(self, schedule, self.iterations, self.initial_object_step, self.batch_size, self.epsilon,
                         "amplitude_mse")
        p.progress_threshold = float(self.progress_threshold)
        p.reduction_factor = float(self.reduction_factor)
        p.minimum_object_step = float(self.minimum_object_step)
        return p


class Fpie(_Algorithm):
    _name = "Fpie"
    _code = _ALG["fpie"]

    def __init__(self, *, iterations=50, object_step=0.8, stability=0.1, batch_size=1, epsilon=1e-10,
                 loss_type="amplitude_mse"):
        _loss(loss_type)
        self.iterations, self.object_step, self.stability = iterations, object_step, stability
        self.batch_size, self.epsilon, self.loss_type = batch_size, epsilon, loss_type

    def _params(self, schedule):
        p = _base_params(self, schedule, self.iterations, self.object_step, self.batch_size, self.epsilon,
                         self.loss_type)
        p.stability = float(self.stability)
        return p


class Mpie(_Algorithm):
    _name = "Mpie"
    _code = _ALG["mpie"]

    def __init__(self, *, iterations=50, object_step=0.2, stability=0.05, momentum_interval=30,
                 momentum_friction=0.9, momentum_feedback=0.9, batch_size=1, epsilon=1e-10,
                 loss_type="amplitude_mse"):
        _loss(loss_type)
        self.iterations, self.object_step, self.stability = iterations, object_step, stability
        self.momentum_interval, self.momentum_friction = momentum_interval, momentum_friction
        self.momentum_feedback, self.batch_size = momentum_feedback, batch_size
        self.epsilon, self.loss_type = epsilon, loss_type

    def _params(self, schedule):
        p = _base_params(self, schedule, self.iterations, self.object_step, self.batch_size, self.epsilon,
                         self.loss_type)
        p.stability = float(self.stability)
        p.momentum_interval = int(self.momentum_interval)
        p.momentum_friction = float(self.momentum_friction)
        p.momentum_feedback = float(self.momentum_feedback)
        return p


class Epry(_Algorithm):
    _name = "Epry"
    _code = _ALG["epry"]

    def __init__(self, *, iterations=100, object_step=0.8, pupil_step=0.1, batch_size=1, recover_pupil=True,
                 constrain_pupil_support=True, recover_frame_gains=False, gain_step=0.2, gain_bounds=(1e-6, 1e6),
                 recover_background=False, background_step=0.2, background_bounds=(0.0, 1e12), epsilon=1e-10,
                 loss_type="amplitude_mse"):
        _loss(loss_type)
        self.iterations, self.object_step, self.pupil_step = iterations, object_step, pupil_step
        self.batch_size, self.recover_pupil = batch_size, recover_pupil
        self.constrain_pupil_support = constrain_pupil_support
        self.recover_frame_gains, self.gain_step, self.gain_bounds = recover_frame_gains, gain_step, gain_bounds
        self.recover_background, self.background_step = recover_background, background_step
        self.background_bounds, self.epsilon, self.loss_type = background_bounds, epsilon, loss_type

    def _params(self, schedule):
        p = _base_params(self, schedule, self.iterations, self.object_step, self.batch_size, self.epsilon,
                         self.loss_type)
        p.pupil_step = float(self.pupil_step)
        p.recover_pupil = int(bool(self.recover_pupil))
        p.constrain_pupil_support = int(bool(self.constrain_pupil_support))
        p.recover_frame_gains = int(bool(self.recover_frame_gains))
        p.recover_background = int(bool(self.recover_background))
        p.gain_step = float(self.gain_step)
        p.gain_min, p.gain_max = (float(v) for v in self.gain_bounds)
        p.background_step = float(self.background_step)
        p.background_min, p.background_max = (float(v) for v in self.background_bounds)
        return p


class GradientDescent(_Algorithm):
    _name = "GradientDescent"
    _code = _ALG["gd"]

    def __init__(self, *, iterations=100, object_step=0.5, batch_size=1, epsilon=1e-10, loss_type="amplitude_mse",
                 poisson_truncation_threshold=None, recover_illumination=False, illumination_step=0.1,
                 illumination_finite_difference=0.05, illumination_bounds=1.0, recover_pupil=False, pupil_step=0.05,
                 constrain_pupil_support=True, object_tv=0.0, object_tv_epsilon=1e-6, pupil_smoothing=0.0,
                 parallel_workers=0):
        _loss(loss_type)
        self.iterations, self.object_step, self.batch_size = iterations, object_step, batch_size
        self.epsilon, self.loss_type = epsilon, loss_type
        self.poisson_truncation_threshold = poisson_truncation_threshold
        self.recover_illumination, self.recover_pupil = recover_illumination, recover_pupil
        self.pupil_step, self.constrain_pupil_support = pupil_step, constrain_pupil_support
        self.object_tv, self.pupil_smoothing = object_tv, pupil_smoothing
        self.parallel_workers = parallel_workers
        self.object_tv_epsilon = object_tv_epsilon
        self.illumination_step = illumination_step
        self.illumination_finite_difference = illumination_finite_difference
        self.illumination_bounds = illumination_bounds
        # GradientDescent::validate (src/algorithms/gradient_descent.rs:333-355).
        for name in ("illumination_step", "illumination_finite_difference", "illumination_bounds"):
            value = getattr(self, name)
            if not (isinstance(value, (int, float)) and math.isfinite(value) and value > 0):
                raise InvalidParameterError(f"{name} must be finite and positive")
        if recover_illumination and (recover_pupil or poisson_truncation_threshold is not None):
            raise UnsupportedError("illumination recovery with pupil recovery or Poisson truncation is not "
                                   "implemented on the GB300 device path")

    def _params(self, schedule):
        p = _base_params(self, schedule, self.iterations, self.object_step, self.batch_size, self.epsilon,
                         self.loss_type)
        p.poisson_truncation = int(self.poisson_truncation_threshold is not None)
        if self.poisson_truncation_threshold is not None:
            p.poisson_truncation_threshold = float(self.poisson_truncation_threshold)
        p.recover_pupil = int(bool(self.recover_pupil))
        p.pupil_step = float(self.pupil_step)
        p.constrain_pupil_support = int(bool(self.constrain_pupil_support))
        p.object_tv_weight = float(self.object_tv)
        p.object_tv_epsilon = float(self.object_tv_epsilon)
        p.pupil_smoothing_weight = float(self.pupil_smoothing)
        p.recover_illumination = int(bool(self.recover_illumination))
        p.illumination_step = float(self.illumination_step)
        p.illumination_finite_difference = float(self.illumination_finite_difference)
        p.maximum_illumination_correction = float(self.illumination_bounds)
        return p


def upload(problems) -> None:
    """Uploads every problem that has no device handle yet in one batched call
    (one parallel validation pass over all frames, one synchronisation)."""
    pending = []
    seen = set()
    for p in problems:
        if p._handle is None and id(p) not in seen:
            seen.add(id(p))
            pending.append(p)
    if not pending:
        return
    if len(pending) == 1:
        pending[0].device_handle()
        return
    ctx = N.context()
    descs = [p._descriptors() for p in pending]
    models = (N.ModelDesc * len(pending))(*[d[0] for d in descs])
    meas = (N.MeasurementDesc * len(pending))(*[d[1] for d in descs])
    handles = (C.c_void_p * len(pending))()
    N.check(N.library().fpm_problem_create_batch(ctx.handle, len(pending), models, meas, handles), ctx.handle)
    for p, h in zip(pending, handles):
        p._handle = C.c_void_p(h)
        p._ctx = ctx


def _result_arrays(problem, params, desc) -> dict:
    """Host arrays of one problem's results, bound into its ResultDesc."""
    mh, mw = problem.reconstruction_shape
    h, w = problem.image_shape
    frames = problem.model.source_count
    # EPRY frame-gain / background recovery returns the recovered state.
    recovering = params.algorithm == _ALG["epry"] and (params.recover_frame_gains or params.recover_background)
    a = dict(object=np.zeros((mh, mw), np.complex128), object_spectrum=np.zeros((mh, mw), np.complex128),
             pupil=np.zeros((h, w), np.complex128), objectives=np.zeros(max(params.iterations, 1)),
             illumination=np.zeros((frames, 2)) if params.recover_illumination else None,
             gains=np.zeros(frames) if recovering else None,
             background=np.zeros((frames, h, w)) if recovering else None)
    desc.object = N.ptr(a["object"], C.c_double)
    desc.object_spectrum = N.ptr(a["object_spectrum"], C.c_double)
    desc.pupil = N.ptr(a["pupil"], C.c_double)
    desc.objectives = N.ptr(a["objectives"], C.c_double)
    if a["illumination"] is not None:
        desc.illumination_corrections = N.ptr(a["illumination"], C.c_double)
    if a["gains"] is not None:
        desc.frame_gains = N.ptr(a["gains"], C.c_double)
        desc.background = N.ptr(a["background"], C.c_double)
    return a


def _recovered_gains(problem, arrays):
    """Frame gains of a result: the recovered ones, else the model's."""
    return arrays["gains"] if arrays.get("gains") is not None else problem.model.frame_gains


def _recovered_background(problem, arrays):
    """Background of a result: the recovered [frames, h, w] stack, else the model's."""
    return arrays["background"] if arrays.get("background") is not None else problem.model._background


def run_batch(algorithm: _Algorithm, problems, *, callbacks=None, resume_from=None, schedule="sequential",
              download=True):
    """Runs one algorithm over many independent problems in shared device launches.

    Tiles of one image size share one frame-engine launch (one thread-block
    cluster per tile); different sizes run concurrently. Each tile follows
    the exact frame order a single run would. With ``download=False`` the
    results stay on the device and ``None`` is returned per problem.
    """
    callbacks = list(callbacks or [])
    for cb in callbacks:
        if not isinstance(cb, Callback):
            raise TypeError("unsupported callback object")
    problems = list(problems)
    if callbacks or resume_from is not None:
        return _run_resumable(algorithm, problems, callbacks, resume_from, schedule, download)
    params = algorithm._params(schedule)
    # Problems that are all still on the host take the overlapped path:
    # uploads and downloads run beside the reconstructions.
    host_path = len(problems) > 1 and len({id(p) for p in problems}) == len(problems) and all(
        p._handle is None for p in problems)
    if not host_path:
        upload(problems)
    handles = None if host_path else (C.c_void_p * len(problems))(*[p.device_handle() for p in problems])
    ctx = N.context()
    results = (N.ResultDesc * len(problems))()
    arrays = []
    if download:
        arrays = [_result_arrays(p, params, results[i]) for i, p in enumerate(problems)]
    start = time.perf_counter()
    if host_path:
        descs = [p._descriptors() for p in problems]
        models = (N.ModelDesc * len(problems))(*[d[0] for d in descs])
        meas = (N.MeasurementDesc * len(problems))(*[d[1] for d in descs])
        made = (C.c_void_p * len(problems))()
        N.check(N.library().fpm_run_batch_host(ctx.handle, len(problems), models, meas, C.byref(params),
                                               results if download else None, made), ctx.handle)
        for p, h in zip(problems, made):
            p._handle = C.c_void_p(h)
            p._ctx = ctx
    else:
        N.check(N.library().fpm_run_batch(ctx.handle, len(problems), handles, C.byref(params),
                                          results if download else None), ctx.handle)
    elapsed = time.perf_counter() - start
    if not download:
        return [None] * len(problems)
    out = []
    for p, a in zip(problems, arrays):
        trace = [(it + 1, float(a["objectives"][it]), elapsed) for it in range(params.iterations)]
        result = ReconstructionResult(
            object=a["object"], object_spectrum=a["object_spectrum"], recovered_pupil=a["pupil"],
            pupil_support=p.model.pupil_support, trace=trace,
            runtime=RuntimeInfo(elapsed, params.iterations, False, algorithm._name),
            recovered_frame_gains=_recovered_gains(p, a), recovered_background=_recovered_background(p, a),
            calibrated_illumination=a["illumination"])
        if p.name is not None:
            result.metadata["problem_name"] = p.name
        out.append(result)
    return out


class Job:
    """A batch queued on the device by submit_batch; its problems stay
    reserved until the job has finished (fpm_run_batch_submit, fpm_job_poll,
    fpm_job_wait)."""

    def __init__(self, handle, algorithm, problems, params, arrays, results, submitted):
        self._handle = handle
        self._algorithm = algorithm
        self._problems = problems
        self._params = params
        self._arrays = arrays
        self._results = results  # the result descriptors the device writes through
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
        """True once the device work and the result copies have finished."""
        if self._out is not None:
            return True
        flag = C.c_int32(0)
        N.check(N.library().fpm_job_poll(self._handle, C.byref(flag)), N.context().handle)
        if flag.value:
            self._collect()
        return bool(flag.value)

    def wait(self) -> list:
        """Blocks until the job has finished and returns one ReconstructionResult per problem."""
        if self._out is None:
            N.check(N.library().fpm_job_wait(self._handle), N.context().handle)
            self._collect()
        return self._out

    @property
    def finished_at(self):
        """time.perf_counter() when done() or wait() first saw the job finished."""
        return self._finished_at

    def stats(self) -> dict:
        """Device statistics of the finished job (as last_run_stats)."""
        self.wait()
        st = N.RunStats()
        N.check(N.library().fpm_job_stats(self._handle, C.byref(st)), N.context().handle)
        out = {name: getattr(st, name) for name, _ in N.RunStats._fields_[:6]}
        out["buckets"] = [(st.bucket_size[k], st.bucket_tiles[k], st.bucket_end_ms[k]) for k in range(st.buckets)]
        return out

    def _collect(self) -> None:
        self._finished_at = time.perf_counter()
        elapsed = self._finished_at - self._submitted
        out = []
        for p, a in zip(self._problems, self._arrays):
            trace = [(it + 1, float(a["objectives"][it]), elapsed) for it in range(self._params.iterations)]
            result = ReconstructionResult(
                object=a["object"], object_spectrum=a["object_spectrum"], recovered_pupil=a["pupil"],
                pupil_support=p.model.pupil_support, trace=trace,
                runtime=RuntimeInfo(elapsed, self._params.iterations, False, self._algorithm._name),
                recovered_frame_gains=_recovered_gains(p, a), recovered_background=_recovered_background(p, a),
                calibrated_illumination=a["illumination"])
            if p.name is not None:
                result.metadata["problem_name"] = p.name
            out.append(result)
        self._out = out

    def __del__(self):
        handle = getattr(self, "_handle", None)
        if handle and not N.closed():
            N.library().fpm_job_destroy(handle)
        self._handle = None


def submit_batch(algorithm: _Algorithm, problems, *, schedule="sequential") -> Job:
    """Queues run_batch on the device and returns at once; Job.done() polls
    and Job.wait() returns the results. For serving loops: several jobs of
    one context run side by side."""
    problems = list(problems)
    params = algorithm._params(schedule)
    upload(problems)
    handles = (C.c_void_p * len(problems))(*[p.device_handle() for p in problems])
    results = (N.ResultDesc * len(problems))()
    arrays = []
    arrays = [_result_arrays(p, params, results[i]) for i, p in enumerate(problems)]
    ctx = N.context()
    handle = C.c_void_p()
    submitted = time.perf_counter()
    N.check(N.library().fpm_run_batch_submit(ctx.handle, len(problems), handles, C.byref(params), results,
                                             C.byref(handle)), ctx.handle)
    return Job(handle, algorithm, problems, params, arrays, results, submitted)


class RunPlan:
    """run_batch over fixed problems, captured once as a CUDA graph
    (fpm_plan_create) and replayed as a single launch per run. Each replay
    starts from the problems' initial state, as a fresh run does; the
    problems stay held by the plan until close()."""

    _release_order = 0

    def __init__(self, handle, algorithm, problems, params):
        self._handle = handle
        self._algorithm = algorithm
        self._problems = problems
        self._params = params
        N.own(self)

    def launch(self) -> None:
        """Queues one replay and returns."""
        N.check(N.library().fpm_plan_launch(self._handle), N.context().handle)

    def wait(self) -> None:
        """Waits for the queued replays; last_run_stats() then describes the last one."""
        N.check(N.library().fpm_plan_wait(self._handle), N.context().handle)

    def run(self) -> None:
        self.launch()
        self.wait()

    def results(self) -> list:
        """The last replay's results, one ReconstructionResult per problem."""
        results = (N.ResultDesc * len(self._problems))()
        arrays = [_result_arrays(p, self._params, results[i]) for i, p in enumerate(self._problems)]
        start = time.perf_counter()
        N.check(N.library().fpm_plan_collect(self._handle, results), N.context().handle)
        elapsed = time.perf_counter() - start
        out = []
        for p, a in zip(self._problems, arrays):
            trace = [(it + 1, float(a["objectives"][it]), elapsed) for it in range(self._params.iterations)]
            result = ReconstructionResult(
                object=a["object"], object_spectrum=a["object_spectrum"], recovered_pupil=a["pupil"],
                pupil_support=p.model.pupil_support, trace=trace,
                runtime=RuntimeInfo(elapsed, self._params.iterations, False, self._algorithm._name),
                recovered_frame_gains=_recovered_gains(p, a), recovered_background=_recovered_background(p, a),
                calibrated_illumination=a["illumination"])
            if p.name is not None:
                result.metadata["problem_name"] = p.name
            out.append(result)
        return out

    def _release_native(self) -> None:
        handle = getattr(self, "_handle", None)
        if handle:
            N.library().fpm_plan_destroy(handle)
            self._handle = None

    def close(self) -> None:
        """Frees the graph; the problems are free for other runs again."""
        if getattr(self, "_handle", None) and not N.closed():
            N.check(N.library().fpm_plan_destroy(self._handle), N.context().handle)
        self._handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def capture_batch(algorithm: _Algorithm, problems, *, schedule="sequential") -> RunPlan:
    """Captures run_batch(algorithm, problems) as a CUDA graph for repeated
    replays (RunPlan.launch / wait / results)."""
    problems = list(problems)
    params = algorithm._params(schedule)
    upload(problems)
    handles = (C.c_void_p * len(problems))(*[p.device_handle() for p in problems])
    ctx = N.context()
    handle = C.c_void_p()
    N.check(N.library().fpm_plan_create(ctx.handle, len(problems), handles, C.byref(params), C.byref(handle)),
            ctx.handle)
    return RunPlan(handle, algorithm, problems, params)


class Request:
    """One request of a Server: done() polls, wait() returns its
    ReconstructionResult; info() gives its timeline (ms since the server
    started: submitted, admitted, started on the device, done)."""

    def __init__(self, server, rid, problem, algorithm, params, arrays, desc, keep):
        self._server = server
        self._id = rid
        self._problem = problem
        self._algorithm = algorithm
        self._params = params
        self._arrays = arrays
        self._desc = desc
        self._keep = keep  # host inputs the device reads until the request finishes
        self._result = None
        self._info = None

    def done(self) -> bool:
        if self._result is not None:
            return True
        flag = C.c_int32(0)
        N.check(N.library().fpm_server_poll(self._server._handle, C.c_uint64(self._id), C.byref(flag)),
                N.context().handle)
        return bool(flag.value)

    def wait(self):
        if self._result is None:
            info = N.RequestInfo()
            status = N.library().fpm_server_wait(self._server._handle, C.c_uint64(self._id), C.byref(info))
            self._info = info
            self._keep = None
            N.check(status, N.context().handle)
            a, p = self._arrays, self._problem
            elapsed = (info.done_ms - info.submit_ms) / 1e3
            trace = [(it + 1, float(a["objectives"][it]), elapsed) for it in range(self._params.iterations)]
            self._result = ReconstructionResult(
                object=a["object"], object_spectrum=a["object_spectrum"], recovered_pupil=a["pupil"],
                pupil_support=p.model.pupil_support, trace=trace,
                runtime=RuntimeInfo(elapsed, self._params.iterations, False, self._algorithm._name),
                recovered_frame_gains=_recovered_gains(p, a), recovered_background=_recovered_background(p, a),
                calibrated_illumination=a["illumination"])
            if p.name is not None:
                self._result.metadata["problem_name"] = p.name
        return self._result

    def info(self) -> dict:
        """Timeline of a finished request (wait() first)."""
        self.wait()
        i = self._info
        return {"submit_ms": i.submit_ms, "admit_ms": i.admit_ms, "start_ms": i.start_ms, "done_ms": i.done_ms,
                "latency_ms": i.done_ms - i.submit_ms, "footprint_bytes": i.footprint_bytes}


class Server:
    """The serving loop of libfpm_gpu (fpm_server_*): requests submitted from
    any thread are admitted by device footprint against an HBM budget as
    earlier work finishes, batched with others of the same algorithm that
    arrive within the batching window, and run while other batches are on
    the GPU. Each result equals a run of that request alone."""

    def __init__(self, *, hbm_budget_gb: float = 150.0, max_batch: int = 16, batch_window_ms: float = 2.0,
                 max_queue: int = 0):
        cfg = N.ServerConfig()
        cfg.hbm_budget_bytes = int(hbm_budget_gb * 1e9)
        cfg.max_batch = int(max_batch)
        cfg.batch_window_ms = float(batch_window_ms)
        cfg.max_queue = int(max_queue)
        ctx = N.context()
        handle = C.c_void_p()
        N.check(N.library().fpm_server_create(ctx.handle, C.byref(cfg), C.byref(handle)), ctx.handle)
        self._handle = handle
        N.own(self)

    def submit(self, algorithm: _Algorithm, problem: ReconstructionProblem, *, schedule="sequential") -> Request:
        """Queues `algorithm.run(problem)` and returns at once."""
        params = algorithm._params(schedule)
        desc, meas, keep = problem._descriptors()
        result = N.ResultDesc()
        arrays = _result_arrays(problem, params, result)
        rid = C.c_uint64()
        N.check(N.library().fpm_server_submit(self._handle, C.byref(desc), C.byref(meas), C.byref(params),
                                              C.byref(result), C.byref(rid)), N.context().handle)
        return Request(self, rid.value, problem, algorithm, params, arrays, (desc, meas, result),
                       (keep, problem.measurements))

    def stats(self) -> dict:
        st = N.ServerStats()
        N.check(N.library().fpm_server_stats_get(self._handle, C.byref(st)), N.context().handle)
        return {name: getattr(st, name) for name, _ in N.ServerStats._fields_}

    _release_order = 0

    def _release_native(self) -> None:
        handle = getattr(self, "_handle", None)
        if handle:
            N.library().fpm_server_destroy(handle)
            self._handle = None

    def close(self) -> None:
        """Finishes every queued and running request, then stops the loop."""
        if getattr(self, "_handle", None) and not N.closed():
            N.library().fpm_server_destroy(self._handle)
        self._handle = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def _recovers_illumination(algorithm) -> bool:
    return isinstance(algorithm, GradientDescent) and bool(algorithm.recover_illumination)


def _state_arrays(problem, algorithm, iterations):
    mh, mw = problem.reconstruction_shape
    h, w = problem.image_shape
    mpie = isinstance(algorithm, Mpie)
    return dict(object_spectrum=np.zeros((mh, mw), np.complex128), pupil=np.zeros((h, w), np.complex128),
                velocity=np.zeros((mh, mw), np.complex128) if mpie else None,
                anchor=np.zeros((mh, mw), np.complex128) if mpie else None,
                objectives=np.zeros(max(int(iterations), 1)),
                illumination=np.zeros((problem.model.source_count, 2)) if _recovers_illumination(algorithm)
                else None)


def _state_desc(arrays, completed, counter):
    d = N.StateDesc()
    d.completed_iterations = int(completed)
    d.momentum_counter = int(counter)
    for name in ("object_spectrum", "pupil", "velocity", "anchor", "objectives"):
        setattr(d, name, N.ptr(arrays[name], C.c_double))
    if arrays.get("illumination") is not None:
        d.illumination_corrections = N.ptr(arrays["illumination"], C.c_double)
    return d


def _checkpoint_arrays(cp: ReconstructionCheckpoint, problem, algorithm):
    """Host arrays of a checkpoint, validated against the problem and algorithm."""
    if cp.algorithm != algorithm._name:
        raise InvalidParameterError(f"checkpoint of {cp.algorithm} cannot resume {algorithm._name}")
    mh, mw = problem.reconstruction_shape
    h, w = problem.image_shape
    if cp.object_spectrum.shape != (mh, mw) or cp.pupil.shape != (h, w):
        raise InvalidShapeError("checkpoint arrays do not match the problem's shapes")
    mpie = isinstance(algorithm, Mpie)
    if mpie and (cp.velocity is None or cp.anchor is None):
        raise InvalidParameterError("an mPIE checkpoint needs its velocity and anchor")
    illumination = None
    if _recovers_illumination(algorithm) and cp.illumination_corrections is not None:
        illumination = np.ascontiguousarray(cp.illumination_corrections, np.float64)
        if illumination.shape != (problem.model.source_count, 2):
            raise InvalidShapeError("checkpoint illumination corrections do not match the source count")
    arrays = dict(object_spectrum=np.ascontiguousarray(cp.object_spectrum, np.complex128),
                  pupil=np.ascontiguousarray(cp.pupil, np.complex128),
                  velocity=np.ascontiguousarray(cp.velocity, np.complex128) if mpie else None,
                  anchor=np.ascontiguousarray(cp.anchor, np.complex128) if mpie else None,
                  objectives=np.asarray(cp.objectives + [0.0], np.float64), illumination=illumination)
    return arrays


class _SegmentState:
    """The state a device segment ended at: captured arrays, the device's
    results, and derived views for callbacks (computed on first use)."""

    def __init__(self, problem, algorithm, captured, counter, end, results):
        self.problem = problem
        self.algorithm = algorithm
        self.arrays = captured
        self.counter = counter
        self.end = end
        self.results = results

    def object(self) -> np.ndarray:
        return self.results["object"]

    def checkpoint(self) -> ReconstructionCheckpoint:
        a = self.arrays
        return ReconstructionCheckpoint(
            completed_iterations=self.end, algorithm=self.algorithm._name, object_spectrum=a["object_spectrum"],
            pupil=a["pupil"], velocity=a["velocity"], anchor=a["anchor"], momentum_counter=self.counter,
            objectives=[float(v) for v in a["objectives"][:self.end]],
            illumination_corrections=None if a["illumination"] is None else a["illumination"].copy())

    def residual_images(self) -> np.ndarray:
        """Forward intensities of the current object, pupil and illumination
        corrections minus the measurements, zero at masked pixels
        (src/reconstruction/runner.rs:435-454 and 335-395)."""
        from .simulation import forward_intensities

        model = self.problem.model
        changes = dict(pupil=np.ascontiguousarray(self.arrays["pupil"], np.complex128))
        if self.arrays["illumination"] is not None:
            corrections = self.arrays["illumination"]
            changes.update(offset_row=model._offset_row + corrections[:, 0],
                           offset_col=model._offset_col + corrections[:, 1])
        predicted = forward_intensities(model._replace(**changes), self.object())
        measured = self.problem.measurements._data.reshape(predicted.shape)
        residual = predicted - measured
        masks = self.problem.measurements._masks
        if masks is not None:
            residual[~masks.reshape(predicted.shape).astype(bool)] = 0.0
        return residual


_SPECULATION = 16


def _run_resumable(algorithm, problems, callbacks, resume_from, schedule, download):
    """Runs in device segments through fpm_run_batch_resumable: from a
    checkpoint, and/or with host callbacks at iteration boundaries.

    Segments end where a callback needs the state (plan_segment); hooks that
    read only objectives are replayed after each segment in iteration order.
    A stop request inside a segment re-runs the segment from its starting
    state to the stopping iteration (src/reconstruction/runner.rs:76-285).
    """
    if callbacks and len(problems) != 1:
        raise UnsupportedError("callbacks are supported for single-problem runs")
    if resume_from is not None and not isinstance(resume_from, (list, tuple)):
        resume_from = [resume_from]
    if resume_from is not None and len(resume_from) != len(problems):
        raise InvalidParameterError("one checkpoint is needed per problem")
    params = algorithm._params(schedule)
    total = params.iterations
    upload(problems)
    handles = (C.c_void_p * len(problems))(*[p.device_handle() for p in problems])
    ctx = N.context()
    keep = []
    resume = None
    start = 0
    trace = []
    if resume_from is not None:
        arrays = [_checkpoint_arrays(cp, p, algorithm) for cp, p in zip(resume_from, problems)]
        keep.append(arrays)
        start = resume_from[0].completed_iterations
        resume = (N.StateDesc * len(problems))(
            *[_state_desc(a, cp.completed_iterations, cp.momentum_counter) for a, cp in zip(arrays, resume_from)])
        trace = [(it + 1, float(v), 0.0) for it, v in enumerate(resume_from[0].objectives)]
    name = problems[0].name
    context = lambda iteration, objective, state=None: StepContext(  # noqa: E731
        iteration=iteration, objective=objective, trace=trace, problem_name=name, algorithm=algorithm._name,
        _state=state)
    for cb in callbacks:
        cb.on_start(context(start, None))

    def segment(end):
        params.iterations = end
        captured = [_state_arrays(p, algorithm, end) for p in problems]
        capture = (N.StateDesc * len(problems))(*[_state_desc(a, 0, 0) for a in captured])
        results = (N.ResultDesc * len(problems))()
        result_arrays = [_result_arrays(p, params, results[i]) for i, p in enumerate(problems)]
        t0 = time.perf_counter()
        N.check(N.library().fpm_run_batch_resumable(ctx.handle, len(problems), handles, C.byref(params), resume,
                                                    results, capture), ctx.handle)
        seconds = time.perf_counter() - t0
        states = [_SegmentState(p, algorithm, captured[i], capture[i].momentum_counter, end, result_arrays[i])
                  for i, p in enumerate(problems)]
        return states, seconds

    current = start
    elapsed = trace[-1][2] if trace else 0.0
    stopped = False
    while True:
        end = plan_segment(callbacks, current, total, _SPECULATION)
        states, seconds = segment(end)
        stop_at = None
        objectives = states[0].arrays["objectives"]
        for it in range(current + 1, end + 1):
            trace.append((it, float(objectives[it - 1]), elapsed + seconds * (it - current) / (end - current)))
            step = context(it, float(objectives[it - 1]), states[0] if it == end else None)
            requested = False
            for cb in callbacks:
                requested |= bool(cb.on_iteration_end(step))
            if requested:
                stop_at = it
                break
        elapsed += seconds
        if stop_at is not None:
            stopped = True
            if stop_at < end:
                states, seconds = segment(stop_at)
                elapsed += seconds
            end = stop_at
        if stopped or end >= total:
            break
        keep.append(states)
        resume = (N.StateDesc * len(problems))(*[_state_desc(st.arrays, end, st.counter) for st in states])
        current = end
    out = [] if download else [None] * len(problems)
    for p, st in zip(problems, states if download else []):
        a = st.results
        records = trace if len(problems) == 1 else [(it + 1, float(a["objectives"][it]), elapsed)
                                                    for it in range(end)]
        result = ReconstructionResult(
            object=a["object"], object_spectrum=a["object_spectrum"], recovered_pupil=a["pupil"],
            pupil_support=p.model.pupil_support, trace=list(records),
            runtime=RuntimeInfo(elapsed, end, stopped, algorithm._name),
            recovered_frame_gains=_recovered_gains(p, a), recovered_background=_recovered_background(p, a),
            calibrated_illumination=a["illumination"])
        if p.name is not None:
            result.metadata["problem_name"] = p.name
        out.append(result)
    for cb in callbacks:
        cb.on_finish(out[0])
    return out


def last_run_stats() -> dict:
    """Device statistics of the last run (CUDA events on the launching streams).

    kernel_launches: kernels this library launched; engine_launches: frame
    engine launches; run_ms: first kernel start to last kernel end;
    engine_ms_sum / engine_span_ms: frame-engine durations summed / spanned;
    engine_bytes: the engine's algorithmic HBM bytes.
    """
    ctx = N.context()
    st = N.RunStats()
    N.check(N.library().fpm_last_run_stats(ctx.handle, C.byref(st)), ctx.handle)
    out = {name: getattr(st, name) for name, _ in N.RunStats._fields_[:6]}
    out.update({name: getattr(st, name) for name, _ in N.RunStats._fields_[10:14]})
    out["host_chunks"] = [(st.host_done_tiles[k], st.host_done_ms[k]) for k in range(st.host_chunks)]
    out["buckets"] = [(st.bucket_size[k], st.bucket_tiles[k], st.bucket_end_ms[k]) for k in range(st.buckets)]
    return out
