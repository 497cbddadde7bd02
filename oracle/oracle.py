"""ctypes binding of the FP64 C oracle (oracle/fpm_oracle.c).

TEST INFRASTRUCTURE ONLY. The oracle restates hgrecco/fpm-rs's image-plane
forward model and reconstruction loop in complex128 arithmetic. Only the test
suite, ``__graft_entry__.smoke()`` and ``bench.py``'s CPU-baseline leg use
it, always as the checker or the timed CPU reference and never as the product
path. Build it with :func:`build` (gcc, portable C11, no intrinsics).
"""

from __future__ import annotations

import ctypes as C
import os
import subprocess
from dataclasses import dataclass
from typing import Sequence

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libfpm_oracle.so")

SHAPE_POLICIES = {"exact": 0, "minimum": 1, "smooth": 2, "power_of_two": 3}
LOSSES = {"amplitude_mse": 0, "intensity_mse": 1, "poisson_nll": 2, "huber_amplitude": 3}
ALGORITHMS = {"ap": 0, "fpie": 1, "mpie": 2, "epry": 3, "gd": 4, "adaptive_ap": 5}
SCHEDULES = {"sequential": 0, "brightfield_first": 1, "spiral_out": 2, "snr_weighted": 3}


def build(force: bool = False) -> str:
    """Compile the oracle shared library next to its source."""
    src = os.path.join(HERE, "fpm_oracle.c")
    if force or not os.path.exists(LIB_PATH) or os.path.getmtime(LIB_PATH) < os.path.getmtime(src):
        cmd = [
            "gcc", "-O3", "-ffp-contract=off", "-std=gnu11", "-Wall", "-shared", "-fPIC",
            "-o", LIB_PATH, src, "-lm", "-lpthread",
        ]
        subprocess.run(cmd, check=True)
    return LIB_PATH


class OracleError(RuntimeError):
    def __init__(self, code: int, message: str):
        super().__init__(f"oracle status {code}: {message}")
        self.code = code


class _Optics(C.Structure):
    _fields_ = [
        ("wavelength_vacuum_m", C.c_double), ("objective_na", C.c_double),
        ("magnification", C.c_double), ("camera_pixel_size", C.c_double),
        ("illumination_refractive_index", C.c_double),
        ("objective_medium_refractive_index", C.c_double),
        ("has_defocus", C.c_int32), ("defocus_distance", C.c_double),
        ("has_aberration", C.c_int32), ("astigmatism", C.c_double), ("coma", C.c_double),
        ("spherical", C.c_double), ("edge_apodization", C.c_double),
    ]


class _Compiled(C.Structure):
    _fields_ = [
        ("h", C.c_int32), ("w", C.c_int32), ("mh", C.c_int32), ("mw", C.c_int32),
        ("sources", C.c_int32),
        ("start_row", C.POINTER(C.c_int64)), ("start_col", C.POINTER(C.c_int64)),
        ("off_row", C.POINTER(C.c_double)), ("off_col", C.POINTER(C.c_double)),
        ("pupil", C.POINTER(C.c_double)), ("support", C.POINTER(C.c_uint8)),
        ("dkx", C.c_double), ("dky", C.c_double),
        ("low_res_pixel_size", C.c_double), ("high_res_pixel_size", C.c_double),
    ]


class _Problem(C.Structure):
    _fields_ = [
        ("h", C.c_int32), ("w", C.c_int32), ("mh", C.c_int32), ("mw", C.c_int32),
        ("frames", C.c_int32),
        ("start_row", C.POINTER(C.c_int64)), ("start_col", C.POINTER(C.c_int64)),
        ("off_row", C.POINTER(C.c_double)), ("off_col", C.POINTER(C.c_double)),
        ("pupil", C.POINTER(C.c_double)), ("support", C.POINTER(C.c_uint8)),
        ("gains", C.POINTER(C.c_double)), ("background", C.POINTER(C.c_double)),
        ("background_len", C.c_int64),
        ("kx", C.POINTER(C.c_double)), ("ky", C.POINTER(C.c_double)),
        ("data", C.POINTER(C.c_double)), ("weights", C.POINTER(C.c_double)),
        ("masks", C.POINTER(C.c_uint8)),
    ]


class _Params(C.Structure):
    _fields_ = [
        ("algorithm", C.c_int32), ("iterations", C.c_int32), ("batch_size", C.c_int32),
        ("loss_type", C.c_int32), ("schedule", C.c_int32),
        ("object_step", C.c_double), ("epsilon", C.c_double), ("stability", C.c_double),
        ("momentum_interval", C.c_int32), ("momentum_friction", C.c_double),
        ("momentum_feedback", C.c_double),
        ("recover_pupil", C.c_int32), ("constrain_pupil", C.c_int32), ("pupil_step", C.c_double),
        ("recover_gains", C.c_int32), ("gain_step", C.c_double), ("gain_min", C.c_double),
        ("gain_max", C.c_double),
        ("recover_background", C.c_int32), ("background_step", C.c_double),
        ("background_min", C.c_double), ("background_max", C.c_double),
        ("poisson_truncation_threshold", C.c_double),
        ("progress_threshold", C.c_double), ("reduction_factor", C.c_double), ("minimum_object_step", C.c_double),
        ("object_tv_weight", C.c_double), ("object_tv_epsilon", C.c_double), ("pupil_smoothing_weight", C.c_double),
        ("recover_illumination", C.c_int32), ("illumination_step", C.c_double),
        ("illumination_finite_difference", C.c_double), ("illumination_bounds", C.c_double),
        ("initial_spectrum", C.POINTER(C.c_double)),
    ]


class _Output(C.Structure):
    _fields_ = [
        ("object_spectrum", C.POINTER(C.c_double)), ("pupil", C.POINTER(C.c_double)),
        ("objectives", C.POINTER(C.c_double)), ("object", C.POINTER(C.c_double)),
        ("status", C.c_int32),
        ("illumination_corrections", C.POINTER(C.c_double)),
        ("frame_gains", C.POINTER(C.c_double)), ("background", C.POINTER(C.c_double)),
        ("object_steps", C.POINTER(C.c_double)),
    ]


_lib = None


def lib():
    global _lib
    if _lib is None:
        build()
        _lib = C.CDLL(LIB_PATH)
        _lib.orc_last_error.restype = C.c_char_p
        _lib.orc_complex_nrmse.restype = C.c_double
    return _lib


def _check(status: int) -> None:
    if status != 0:
        raise OracleError(status, lib().orc_last_error().decode())


def _ptr(array, ctype):
    if array is None:
        return C.POINTER(ctype)()
    return array.ctypes.data_as(C.POINTER(ctype))


def _c128(a) -> np.ndarray:
    return np.ascontiguousarray(a, dtype=np.complex128)


def _f64(a) -> np.ndarray:
    return np.ascontiguousarray(a, dtype=np.float64)


def optics_struct(optics: dict) -> _Optics:
    o = _Optics()
    o.wavelength_vacuum_m = optics["wavelength_vacuum_m"]
    o.objective_na = optics["objective_na"]
    o.magnification = optics["magnification"]
    o.camera_pixel_size = optics["camera_pixel_size"]
    o.illumination_refractive_index = optics.get("illumination_refractive_index", 1.0)
    o.objective_medium_refractive_index = optics.get("objective_medium_refractive_index", 1.0)
    defocus = optics.get("defocus_distance")
    o.has_defocus = int(defocus is not None)
    o.defocus_distance = defocus or 0.0
    ab = optics.get("pupil_aberration")
    o.has_aberration = int(ab is not None)
    if ab is not None:
        o.astigmatism, o.coma, o.spherical, o.edge_apodization = (
            ab.get("astigmatism", 0.0), ab.get("coma", 0.0), ab.get("spherical", 0.0),
            ab.get("edge_apodization", 0.0))
    return o


# ----------------------------------------------------------------- FFT ----

def fft2(values, inverse: bool = False) -> np.ndarray:
    """Reference-convention 2-D FFT: forward scaled by 1/(h*w), inverse unscaled."""
    out = _c128(values).copy()
    h, w = out.shape
    _check(lib().orc_fft2(_ptr(out, C.c_double), h, w, int(inverse)))
    return out


def fftshift(values) -> np.ndarray:
    a = _c128(values)
    out = np.empty_like(a)
    lib().orc_fftshift(_ptr(a, C.c_double), _ptr(out, C.c_double), *a.shape)
    return out


def ifftshift(values) -> np.ndarray:
    a = _c128(values)
    out = np.empty_like(a)
    lib().orc_ifftshift(_ptr(a, C.c_double), _ptr(out, C.c_double), *a.shape)
    return out


# ------------------------------------------------------------ geometry ----

def planar_kvectors(optics: dict, shape, pitch, reference_index, translation, rotation=(0.0, 0.0, 0.0)):
    rows, cols = shape
    px, py = (pitch, pitch) if np.isscalar(pitch) else pitch
    ref_col, ref_row = reference_index
    kx = np.zeros(rows * cols)
    ky = np.zeros(rows * cols)
    t = _f64(translation)
    r = _f64(rotation)
    o = optics_struct(optics)
    _check(lib().orc_planar_kvectors(C.byref(o), rows, cols, C.c_double(px), C.c_double(py),
                                     C.c_double(ref_col), C.c_double(ref_row), _ptr(t, C.c_double),
                                     _ptr(r, C.c_double), _ptr(kx, C.c_double), _ptr(ky, C.c_double)))
    return kx, ky


def next_smooth(minimum: int) -> int:
    out = C.c_int64()
    lib().orc_next_smooth(C.c_int64(minimum), C.byref(out))
    return out.value


def compile_model(optics: dict, kx, ky, image_shape, reconstruction_shape="smooth") -> dict:
    kx = _f64(kx)
    ky = _f64(ky)
    n = kx.size
    h, w = image_shape
    if isinstance(reconstruction_shape, str):
        policy, emh, emw = SHAPE_POLICIES[reconstruction_shape], 0, 0
    else:
        policy, (emh, emw) = 0, reconstruction_shape
    start_row = np.zeros(n, np.int64)
    start_col = np.zeros(n, np.int64)
    off_row = np.zeros(n)
    off_col = np.zeros(n)
    pupil = np.zeros((h, w), np.complex128)
    support = np.zeros((h, w), np.uint8)
    c = _Compiled()
    c.start_row = _ptr(start_row, C.c_int64)
    c.start_col = _ptr(start_col, C.c_int64)
    c.off_row = _ptr(off_row, C.c_double)
    c.off_col = _ptr(off_col, C.c_double)
    c.pupil = _ptr(pupil, C.c_double)
    c.support = _ptr(support, C.c_uint8)
    o = optics_struct(optics)
    _check(lib().orc_compile(C.byref(o), n, _ptr(kx, C.c_double), _ptr(ky, C.c_double), h, w,
                             policy, emh, emw, C.byref(c)))
    return dict(h=h, w=w, mh=c.mh, mw=c.mw, start_row=start_row, start_col=start_col,
                off_row=off_row, off_col=off_col, pupil=pupil, support=support, kx=kx, ky=ky,
                dkx=c.dkx, dky=c.dky, low_res_pixel_size=c.low_res_pixel_size,
                high_res_pixel_size=c.high_res_pixel_size)


def extract_patch(spectrum, start, shape, offset=(0.0, 0.0)) -> np.ndarray:
    s = _c128(spectrum)
    out = np.zeros(shape, np.complex128)
    _check(lib().orc_extract_patch(_ptr(s, C.c_double), s.shape[0], s.shape[1], C.c_int64(start[0]),
                                   C.c_int64(start[1]), shape[0], shape[1], C.c_double(offset[0]),
                                   C.c_double(offset[1]), _ptr(out, C.c_double)))
    return out


def insert_adjoint(spectrum, start, update, scale, offset=(0.0, 0.0)) -> np.ndarray:
    s = _c128(spectrum).copy()
    u = _c128(update)
    _check(lib().orc_insert_adjoint(_ptr(s, C.c_double), s.shape[0], s.shape[1], C.c_int64(start[0]),
                                    C.c_int64(start[1]), u.shape[0], u.shape[1], C.c_double(offset[0]),
                                    C.c_double(offset[1]), _ptr(u, C.c_double), C.c_double(scale)))
    return s


def object_spectrum(obj) -> np.ndarray:
    o = _c128(obj)
    out = np.empty_like(o)
    _check(lib().orc_object_spectrum(_ptr(o, C.c_double), o.shape[0], o.shape[1], _ptr(out, C.c_double)))
    return out


def state_object(spectrum) -> np.ndarray:
    s = _c128(spectrum)
    out = np.empty_like(s)
    _check(lib().orc_state_object(_ptr(s, C.c_double), s.shape[0], s.shape[1], _ptr(out, C.c_double)))
    return out


def momentum_event(obj, velocity, anchor, friction, feedback):
    o, v, a = _c128(obj).copy(), _c128(velocity).copy(), _c128(anchor).copy()
    _check(lib().orc_momentum_event(_ptr(o, C.c_double), _ptr(v, C.c_double), _ptr(a, C.c_double),
                                    C.c_int64(o.size), C.c_double(friction), C.c_double(feedback)))
    return o, v, a


def truncation_accepts(predicted: float, measured: float, scale: float) -> bool:
    fn = lib().orc_truncation_accepts
    fn.restype = C.c_int32
    fn.argtypes = [C.c_double, C.c_double, C.c_double]
    return bool(fn(predicted, measured, scale))


def complex_nrmse(reference, candidate) -> float:
    r = _c128(reference)
    c = _c128(candidate)
    return lib().orc_complex_nrmse(_ptr(r, C.c_double), _ptr(c, C.c_double), C.c_int64(r.size))


# ------------------------------------------------------------ problems ----

@dataclass
class Problem:
    """A compiled model dict plus measurements, kept alive for ctypes."""

    model: dict
    data: np.ndarray
    weights: np.ndarray | None = None
    masks: np.ndarray | None = None
    gains: np.ndarray | None = None
    background: np.ndarray | None = None

    def struct(self) -> _Problem:
        m = self.model
        self._keep = []

        def keep(a):
            self._keep.append(a)
            return a

        p = _Problem()
        p.h, p.w, p.mh, p.mw = m["h"], m["w"], m["mh"], m["mw"]
        data = keep(_f64(self.data))
        p.frames = data.shape[0]
        p.start_row = _ptr(keep(np.ascontiguousarray(m["start_row"], np.int64)), C.c_int64)
        p.start_col = _ptr(keep(np.ascontiguousarray(m["start_col"], np.int64)), C.c_int64)
        p.off_row = _ptr(keep(_f64(m["off_row"])), C.c_double)
        p.off_col = _ptr(keep(_f64(m["off_col"])), C.c_double)
        p.pupil = _ptr(keep(_c128(m["pupil"])), C.c_double)
        p.support = _ptr(keep(np.ascontiguousarray(m["support"], np.uint8)), C.c_uint8)
        p.gains = _ptr(keep(_f64(self.gains)) if self.gains is not None else None, C.c_double)
        if self.background is not None:
            bg = keep(_f64(self.background).ravel())
            p.background = _ptr(bg, C.c_double)
            p.background_len = bg.size
        p.kx = _ptr(keep(_f64(m["kx"])) if "kx" in m else None, C.c_double)
        p.ky = _ptr(keep(_f64(m["ky"])) if "ky" in m else None, C.c_double)
        p.data = _ptr(data, C.c_double)
        p.weights = _ptr(keep(_f64(self.weights)) if self.weights is not None else None, C.c_double)
        p.masks = _ptr(keep(np.ascontiguousarray(self.masks, np.uint8)) if self.masks is not None else None,
                       C.c_uint8)
        return p


def forward_stack(problem: Problem, spectrum, workers: int = 1) -> np.ndarray:
    s = _c128(spectrum)
    m = problem.model
    frames = len(m["start_row"])
    out = np.zeros((frames, m["h"], m["w"]))
    if problem.data is None or np.asarray(problem.data).shape[0] != frames:
        problem = Problem(m, np.zeros((frames, m["h"], m["w"])), gains=problem.gains,
                          background=problem.background)
    st = problem.struct()
    _check(lib().orc_forward_stack(C.byref(st), _ptr(s, C.c_double), _ptr(out, C.c_double), workers))
    return out


DEFAULTS = {
    "ap": dict(iterations=50, object_step=1.0),
    "fpie": dict(iterations=50, object_step=0.8, stability=0.1),
    "mpie": dict(iterations=50, object_step=0.2, stability=0.05, momentum_interval=30,
                 momentum_friction=0.9, momentum_feedback=0.9),
    "epry": dict(iterations=100, object_step=0.8, pupil_step=0.1, recover_pupil=True,
                 constrain_pupil=True),
    "gd": dict(iterations=100, object_step=0.5),
    "adaptive_ap": dict(iterations=50, object_step=1.0, progress_threshold=0.01, reduction_factor=0.5,
                        minimum_object_step=0.001),
}


def params(algorithm: str, **kw) -> _Params:
    cfg = dict(batch_size=1, epsilon=1e-10, loss_type="amplitude_mse", schedule="sequential",
               stability=0.0, momentum_interval=30, momentum_friction=0.9, momentum_feedback=0.9,
               recover_pupil=False, constrain_pupil=True, pupil_step=0.1, recover_gains=False,
               gain_step=0.2, gain_min=1e-6, gain_max=1e6, recover_background=False,
               background_step=0.2, background_min=0.0, background_max=1e12, poisson_truncation_threshold=0.0,
               progress_threshold=0.01, reduction_factor=0.5, minimum_object_step=0.001, object_tv_weight=0.0,
               object_tv_epsilon=1e-6, pupil_smoothing_weight=0.0, recover_illumination=False,
               illumination_step=0.1, illumination_finite_difference=0.05, illumination_bounds=1.0)
    cfg.update(DEFAULTS[algorithm])
    cfg.update(kw)
    p = _Params()
    p.algorithm = ALGORITHMS[algorithm]
    p.iterations = cfg["iterations"]
    p.batch_size = cfg["batch_size"]
    p.loss_type = LOSSES[cfg["loss_type"]]
    p.schedule = SCHEDULES[cfg["schedule"]]
    for name in ("object_step", "epsilon", "stability", "momentum_friction", "momentum_feedback",
                 "pupil_step", "gain_step", "gain_min", "gain_max", "background_step",
                 "background_min", "background_max", "poisson_truncation_threshold", "progress_threshold",
                 "reduction_factor", "minimum_object_step", "object_tv_weight", "object_tv_epsilon",
                 "pupil_smoothing_weight", "illumination_step", "illumination_finite_difference",
                 "illumination_bounds"):
        setattr(p, name, float(cfg[name]))
    p.momentum_interval = int(cfg["momentum_interval"])
    p.recover_pupil = int(bool(cfg["recover_pupil"]))
    p.constrain_pupil = int(bool(cfg["constrain_pupil"]))
    p.recover_gains = int(bool(cfg["recover_gains"]))
    p.recover_background = int(bool(cfg["recover_background"]))
    p.recover_illumination = int(bool(cfg["recover_illumination"]))
    return p


def _outputs(problem: Problem, prm: _Params):
    m = problem.model
    arrays = dict(
        object_spectrum=np.zeros((m["mh"], m["mw"]), np.complex128),
        pupil=np.zeros((m["h"], m["w"]), np.complex128),
        objectives=np.zeros(prm.iterations),
        object=np.zeros((m["mh"], m["mw"]), np.complex128),
        illumination_corrections=np.zeros((len(m["start_row"]), 2)),
        frame_gains=np.zeros(len(m["start_row"])),
        object_steps=np.zeros(max(prm.iterations, 1)),
        # The recovered background only when recovered (frames x h x w).
        background=np.zeros((len(m["start_row"]), m["h"], m["w"])) if prm.recover_background else None,
    )
    out = _Output()
    out.object_spectrum = _ptr(arrays["object_spectrum"], C.c_double)
    out.pupil = _ptr(arrays["pupil"], C.c_double)
    out.objectives = _ptr(arrays["objectives"], C.c_double)
    out.object = _ptr(arrays["object"], C.c_double)
    out.illumination_corrections = _ptr(arrays["illumination_corrections"], C.c_double)
    out.frame_gains = _ptr(arrays["frame_gains"], C.c_double)
    out.object_steps = _ptr(arrays["object_steps"], C.c_double)
    out.background = _ptr(arrays["background"], C.c_double)
    return out, arrays


def run(problem: Problem, algorithm: str, initial_spectrum=None, **kw) -> dict:
    """orc_run; `initial_spectrum` (centred mh x mw) replaces the default start."""
    prm = params(algorithm, **kw)
    init = None if initial_spectrum is None else _c128(initial_spectrum)
    if init is not None:
        prm.initial_spectrum = _ptr(init, C.c_double)
    st = problem.struct()
    out, arrays = _outputs(problem, prm)
    _check(lib().orc_run(C.byref(st), C.byref(prm), C.byref(out)))
    return arrays


def run_many(problems: Sequence[Problem], algorithm: str, workers: int, **kw) -> list[dict]:
    prm = params(algorithm, **kw)
    structs = (_Problem * len(problems))(*[p.struct() for p in problems])
    outs = (_Output * len(problems))()
    arrays = []
    for i, p in enumerate(problems):
        o, a = _outputs(p, prm)
        outs[i] = o
        arrays.append(a)
    _check(lib().orc_run_many(len(problems), structs, C.byref(prm), outs, workers))
    return arrays


# ------------------------------------------------------------ spectral ----

class _SpectralProblem(C.Structure):
    _fields_ = [
        ("h", C.c_int32), ("w", C.c_int32), ("mh", C.c_int32), ("mw", C.c_int32),
        ("channels", C.c_int32), ("shared_object", C.c_int32),
        ("channel_sources", C.POINTER(C.c_int32)),
        ("start_row", C.POINTER(C.c_int64)), ("start_col", C.POINTER(C.c_int64)),
        ("off_row", C.POINTER(C.c_double)), ("off_col", C.POINTER(C.c_double)),
        ("frame_gains", C.POINTER(C.c_double)),
        ("pupils", C.POINTER(C.c_double)),
        ("exposures", C.c_int32),
        ("contribution_offsets", C.POINTER(C.c_int32)),
        ("contribution_channel", C.POINTER(C.c_int32)), ("contribution_local", C.POINTER(C.c_int32)),
        ("contribution_weight", C.POINTER(C.c_double)),
        ("exposure_gain", C.POINTER(C.c_double)), ("exposure_background", C.POINTER(C.c_double)),
        ("data", C.POINTER(C.c_double)), ("weights", C.POINTER(C.c_double)), ("masks", C.POINTER(C.c_uint8)),
    ]


class _SpectralParams(C.Structure):
    _fields_ = [("iterations", C.c_int32), ("loss_type", C.c_int32), ("object_step", C.c_double),
                ("epsilon", C.c_double)]


@dataclass
class SpectralProblem:
    """Channel models (dicts of compile_model's form, frame gains under
    "frame_gains"), a canonical detector plan and measurements.

    frames: one (gain, background, [(channel, local_frame, spectral_weight), ...])
    per exposure, already canonical (positive weights, unique pairs)."""

    channels: list
    frames: list
    data: np.ndarray | None = None
    shared_object: bool = False
    weights: np.ndarray | None = None
    masks: np.ndarray | None = None

    @property
    def object_count(self) -> int:
        return 1 if self.shared_object else len(self.channels)

    def struct(self) -> _SpectralProblem:
        ch = self.channels
        self._keep = []

        def keep(a):
            self._keep.append(a)
            return a

        p = _SpectralProblem()
        p.h, p.w, p.mh, p.mw = ch[0]["h"], ch[0]["w"], ch[0]["mh"], ch[0]["mw"]
        p.channels = len(ch)
        p.shared_object = int(bool(self.shared_object))
        p.channel_sources = _ptr(keep(np.array([len(c["start_row"]) for c in ch], np.int32)), C.c_int32)
        cat = lambda key, dtype: keep(np.ascontiguousarray(np.concatenate([np.asarray(c[key]) for c in ch]), dtype))
        p.start_row = _ptr(cat("start_row", np.int64), C.c_int64)
        p.start_col = _ptr(cat("start_col", np.int64), C.c_int64)
        p.off_row = _ptr(cat("off_row", np.float64), C.c_double)
        p.off_col = _ptr(cat("off_col", np.float64), C.c_double)
        gains = [np.asarray(c.get("frame_gains", np.ones(len(c["start_row"]))), np.float64) for c in ch]
        p.frame_gains = _ptr(keep(np.ascontiguousarray(np.concatenate(gains))), C.c_double)
        p.pupils = _ptr(keep(_c128(np.stack([c["pupil"] for c in ch]))), C.c_double)
        p.exposures = len(self.frames)
        offsets = np.zeros(len(self.frames) + 1, np.int32)
        chan, local, weight = [], [], []
        for e, (_, _, contributions) in enumerate(self.frames):
            for c, l, w in contributions:
                chan.append(c)
                local.append(l)
                weight.append(w)
            offsets[e + 1] = len(chan)
        p.contribution_offsets = _ptr(keep(offsets), C.c_int32)
        p.contribution_channel = _ptr(keep(np.array(chan, np.int32)), C.c_int32)
        p.contribution_local = _ptr(keep(np.array(local, np.int32)), C.c_int32)
        p.contribution_weight = _ptr(keep(np.array(weight, np.float64)), C.c_double)
        p.exposure_gain = _ptr(keep(np.array([f[0] for f in self.frames], np.float64)), C.c_double)
        p.exposure_background = _ptr(keep(np.array([f[1] for f in self.frames], np.float64)), C.c_double)
        data = self.data if self.data is not None else np.zeros((len(self.frames), p.h, p.w))
        p.data = _ptr(keep(_f64(data)), C.c_double)
        p.weights = _ptr(keep(_f64(self.weights)) if self.weights is not None else None, C.c_double)
        p.masks = _ptr(keep(np.ascontiguousarray(self.masks, np.uint8)) if self.masks is not None else None,
                       C.c_uint8)
        return p


def spectral_forward(problem: SpectralProblem, spectra) -> np.ndarray:
    """Detector intensities of every exposure from centred spectra (object_count, mh, mw)."""
    s = _c128(spectra)
    st = problem.struct()
    out = np.zeros((st.exposures, st.h, st.w))
    _check(lib().orc_spectral_forward(C.byref(st), _ptr(s, C.c_double), _ptr(out, C.c_double)))
    return out


def spectral_run(problem: SpectralProblem, *, iterations=50, object_step=1.0, epsilon=1e-10,
                 loss_type="amplitude_mse", order=None, initial_objects=None, initial_spectra=None,
                 completed_iterations=0) -> dict:
    """Spectral alternating projection; returns centred spectra, objects and objectives."""
    st = problem.struct()
    prm = _SpectralParams(int(iterations), LOSSES[loss_type], float(object_step), float(epsilon))
    k = problem.object_count
    spectra = np.zeros((k, st.mh, st.mw), np.complex128)
    objectives = np.zeros(int(iterations) - int(completed_iterations))
    order_a = None if order is None else np.ascontiguousarray(order, np.int32)
    init_o = None if initial_objects is None else _c128(initial_objects)
    init_s = None if initial_spectra is None else _c128(initial_spectra)
    _check(lib().orc_spectral_run(C.byref(st), C.byref(prm), _ptr(order_a, C.c_int32), _ptr(init_o, C.c_double),
                                  _ptr(init_s, C.c_double), int(completed_iterations), _ptr(spectra, C.c_double),
                                  _ptr(objectives, C.c_double)))
    objects = np.stack([state_object(s) for s in spectra])
    return dict(spectra=spectra, objects=objects, objectives=objectives)


def complex_tv_step(values, weight: float, epsilon: float) -> np.ndarray:
    out = _c128(values).copy()
    _check(lib().orc_complex_tv_step(_ptr(out, C.c_double), out.shape[0], out.shape[1], C.c_double(weight),
                                     C.c_double(epsilon)))
    return out


def quadratic_smoothing_step(values, weight: float) -> np.ndarray:
    out = _c128(values).copy()
    _check(lib().orc_quadratic_smoothing_step(_ptr(out, C.c_double), out.shape[0], out.shape[1], C.c_double(weight)))
    return out


def gd_batch_step(problem: Problem, spectrum, pupil, frames, illumination_gradient: bool = False, corrections=None,
                  **kw):
    """One gradient-descent step over the batch `frames` from the given state.
    With illumination_gradient, also returns the batch's per-source (row,
    column) source-offset gradient (recover_illumination must be set).
    `corrections` (sources x 2 float64, updated in place) carries the
    illumination corrections into and out of the step."""
    prm = params("gd", **kw)
    st = problem.struct()
    s_in, p_in = _c128(spectrum), _c128(pupil)
    s_out, p_out = np.zeros_like(s_in), np.zeros_like(p_in)
    ill = np.zeros((len(problem.model["start_row"]), 2))
    if corrections is not None and (corrections.dtype != np.float64 or not corrections.flags.c_contiguous or
                                    corrections.shape != ill.shape):
        raise ValueError("corrections must be a C-contiguous float64 (sources, 2) array")
    f = np.ascontiguousarray(frames, np.int32)
    _check(lib().orc_gd_batch_step(C.byref(st), C.byref(prm), _ptr(s_in, C.c_double), _ptr(p_in, C.c_double),
                                   _ptr(f, C.c_int32), f.size, _ptr(s_out, C.c_double), _ptr(p_out, C.c_double),
                                   _ptr(ill, C.c_double), _ptr(corrections, C.c_double)))
    return (s_out, p_out, ill) if illumination_gradient else (s_out, p_out)


def frame_loss(problem: Problem, spectrum, pupil, frame: int, loss_type: str) -> float:
    st = problem.struct()
    out = C.c_double()
    s_in, p_in = _c128(spectrum), _c128(pupil)
    _check(lib().orc_frame_loss(C.byref(st), _ptr(s_in, C.c_double), _ptr(p_in, C.c_double), int(frame),
                                LOSSES[loss_type], C.byref(out)))
    return out.value


def canonicalize(problem: Problem, spectrum, pupil):
    """The object/pupil gauge canonicalisation of the given state (copies)."""
    st = problem.struct()
    s_io, p_io = _c128(spectrum).copy(), _c128(pupil).copy()
    _check(lib().orc_canonicalize(C.byref(st), _ptr(s_io, C.c_double), _ptr(p_io, C.c_double)))
    return s_io, p_io
