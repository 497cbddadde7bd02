"""Compiled image-plane model (src/model/image_plane_fpm.rs:57-253).

compile_model resolves illumination to k-vectors, chooses the
reconstruction grid, and compiles integer crop origins, fractional offsets
and the circular pupil in the native library (bit-identical crop origins to
the reference: the same rounding and bounds rules in FP64).
"""

from __future__ import annotations

import ctypes as C
import json
import math
import os

import numpy as np

from . import _native as N
from .errors import InvalidModelError, InvalidParameterError, InvalidShapeError, json_file_errors

_POLICIES = {"minimum": 1, "smooth": 2, "power_of_two": 3}


class ImagePlaneModel:
    """Pupil, Fourier crops, sampling and frame gains used by simulation and reconstruction."""

    def __init__(self, *, image_shape, reconstruction_shape, k_vectors, start_row, start_col, offset_row,
                 offset_col, pupil, pupil_support, frame_gains=None, background=None, dkx=None, dky=None,
                 low_res_pixel_size=None, wavelength=None):
        self._image_shape = (int(image_shape[0]), int(image_shape[1]))
        self._reconstruction_shape = (int(reconstruction_shape[0]), int(reconstruction_shape[1]))
        self._k = np.ascontiguousarray(k_vectors, dtype=np.float64).reshape(-1, 2)
        self._start_row = np.ascontiguousarray(start_row, dtype=np.int64)
        self._start_col = np.ascontiguousarray(start_col, dtype=np.int64)
        self._offset_row = np.ascontiguousarray(offset_row, dtype=np.float64)
        self._offset_col = np.ascontiguousarray(offset_col, dtype=np.float64)
        self._pupil = np.ascontiguousarray(pupil, dtype=np.complex128)
        self._support = np.ascontiguousarray(pupil_support, dtype=np.uint8)
        self._gains = None if frame_gains is None else np.ascontiguousarray(frame_gains, dtype=np.float64)
        self._background = None if background is None else np.ascontiguousarray(background, dtype=np.float64)
        self._dkx, self._dky = dkx, dky
        self._low_res_pixel_size = low_res_pixel_size
        self._wavelength = wavelength
        self._validate()

    def _validate(self) -> None:
        h, w = self._image_shape
        n = self._k.shape[0]
        if n == 0 or any(a.shape != (n,) for a in (self._start_row, self._start_col, self._offset_row, self._offset_col)):
            raise InvalidModelError(f"{n} source k-vectors and crops; counts must be equal and non-zero")
        if self._pupil.shape != (h, w) or self._support.shape != (h, w):
            raise InvalidModelError(f"pupil shape {self._pupil.shape} does not match image shape {(h, w)}")
        if not np.all(np.isfinite(self._pupil)) or np.any(self._support > 1):
            raise InvalidModelError("pupil support or numeric values are invalid")
        if self._gains is not None and (self._gains.shape != (n,) or np.any(~np.isfinite(self._gains)) or np.any(self._gains < 0)):
            raise InvalidModelError("frame gains must be finite and non-negative, one per frame")

    # -- properties mirroring python/fpm_rs/__init__.pyi:2105-2140
    @property
    def image_shape(self):
        return self._image_shape

    @property
    def reconstruction_shape(self):
        return self._reconstruction_shape

    @property
    def source_count(self) -> int:
        return self._k.shape[0]

    @property
    def frame_count(self) -> int:
        return self._k.shape[0]

    @property
    def is_multiplexed(self) -> bool:
        return False

    @property
    def k_vectors(self) -> np.ndarray:
        return self._k.copy()

    @property
    def pupil(self) -> np.ndarray:
        return self._pupil.copy()

    @property
    def pupil_support(self) -> np.ndarray:
        return self._support.copy()

    @property
    def frame_gains(self):
        return None if self._gains is None else self._gains.copy()

    @property
    def crop_origins(self) -> np.ndarray:
        """Integer (start_row, start_col) per source."""
        return np.stack([self._start_row, self._start_col], axis=1)

    @property
    def subpixel_offsets(self) -> np.ndarray:
        """Fractional (row, column) Fourier-grid offsets per source."""
        return np.stack([self._offset_row, self._offset_col], axis=1)

    def with_pupil(self, values) -> "ImagePlaneModel":
        """Returns a copy with replaced pupil values and the same support (Pupil::replace_values)."""
        values = np.ascontiguousarray(values, dtype=np.complex128)
        if values.shape != self._pupil.shape:
            raise InvalidShapeError(f"replacement pupil shape {values.shape} does not match {self._pupil.shape}")
        if not np.all(np.isfinite(values)):
            raise InvalidModelError("pupil contains non-finite complex values")
        return self._replace(pupil=values)

    def _replace(self, **changes) -> "ImagePlaneModel":
        args = dict(image_shape=self._image_shape, reconstruction_shape=self._reconstruction_shape,
                    k_vectors=self._k, start_row=self._start_row, start_col=self._start_col,
                    offset_row=self._offset_row, offset_col=self._offset_col, pupil=self._pupil,
                    pupil_support=self._support, frame_gains=self._gains, background=self._background,
                    dkx=self._dkx, dky=self._dky, low_res_pixel_size=self._low_res_pixel_size,
                    wavelength=self._wavelength)
        args.update(changes)
        return ImagePlaneModel(**args)

    def _descriptor(self):
        """ModelDesc for the C ABI plus the arrays it points into."""
        keep = []

        def k(a):
            keep.append(a)
            return a

        d = N.ModelDesc()
        d.image_height, d.image_width = self._image_shape
        d.recon_height, d.recon_width = self._reconstruction_shape
        d.sources = self.source_count
        d.crop_start_row = N.ptr(k(self._start_row), C.c_int64)
        d.crop_start_col = N.ptr(k(self._start_col), C.c_int64)
        d.offset_row = N.ptr(k(self._offset_row), C.c_double)
        d.offset_col = N.ptr(k(self._offset_col), C.c_double)
        d.pupil = N.ptr(k(self._pupil), C.c_double)
        d.support = N.ptr(k(self._support), C.c_uint8)
        d.frame_gains = N.ptr(k(self._gains) if self._gains is not None else None, C.c_double)
        if self._background is not None:
            bg = k(np.ascontiguousarray(self._background.ravel()))
            d.background = N.ptr(bg, C.c_double)
            d.background_len = bg.size
        kx = k(np.ascontiguousarray(self._k[:, 0]))
        ky = k(np.ascontiguousarray(self._k[:, 1]))
        d.kx = N.ptr(kx, C.c_double)
        d.ky = N.ptr(ky, C.c_double)
        return d, keep

    # -- persistence (ImagePlaneModel::save_json/load_json, src/model/image_plane_fpm.rs:117-134)
    def save_json(self, *, path) -> None:
        with json_file_errors(path):
            self._save_json(path)

    def _save_json(self, path) -> None:
        doc = {
            "format": "fpm-gb300 image-plane model v1",
            "image_shape": list(self._image_shape),
            "reconstruction_shape": list(self._reconstruction_shape),
            "k_vectors": self._k.tolist(),
            "crop_start": [self._start_row.tolist(), self._start_col.tolist()],
            "subpixel_offsets": [self._offset_row.tolist(), self._offset_col.tolist()],
            "pupil": [self._pupil.real.ravel().tolist(), self._pupil.imag.ravel().tolist()],
            "pupil_support": self._support.ravel().tolist(),
            "frame_gains": None if self._gains is None else self._gains.tolist(),
            "background": None if self._background is None else self._background.ravel().tolist(),
            "sampling": {"dkx": self._dkx, "dky": self._dky, "low_res_pixel_size": self._low_res_pixel_size,
                         "wavelength": self._wavelength},
        }
        with open(os.fspath(path), "w") as handle:
            json.dump(doc, handle)
            handle.flush()
            os.fsync(handle.fileno())

    @staticmethod
    def load_json(*, path) -> "ImagePlaneModel":
        with json_file_errors(path):
            return ImagePlaneModel._load_json(path)

    @staticmethod
    def _load_json(path) -> "ImagePlaneModel":
        with open(os.fspath(path)) as handle:
            doc = json.load(handle)
        h, w = doc["image_shape"]
        pupil = (np.asarray(doc["pupil"][0]) + 1j * np.asarray(doc["pupil"][1])).reshape(h, w)
        s = doc.get("sampling", {})
        return ImagePlaneModel(
            image_shape=doc["image_shape"], reconstruction_shape=doc["reconstruction_shape"],
            k_vectors=np.asarray(doc["k_vectors"]), start_row=doc["crop_start"][0], start_col=doc["crop_start"][1],
            offset_row=doc["subpixel_offsets"][0], offset_col=doc["subpixel_offsets"][1], pupil=pupil,
            pupil_support=np.asarray(doc["pupil_support"], dtype=np.uint8).reshape(h, w),
            frame_gains=doc.get("frame_gains"),
            background=None if doc.get("background") is None else np.asarray(doc["background"]),
            dkx=s.get("dkx"), dky=s.get("dky"), low_res_pixel_size=s.get("low_res_pixel_size"),
            wavelength=s.get("wavelength"))


def _shape_args(reconstruction_shape):
    if isinstance(reconstruction_shape, str):
        if reconstruction_shape not in _POLICIES:
            raise InvalidParameterError(
                "reconstruction_shape must be a (height, width) tuple or one of 'minimum', 'smooth', 'power_of_two'")
        return _POLICIES[reconstruction_shape], 0, 0
    mh, mw = reconstruction_shape
    return 0, int(mh), int(mw)


def suggest_reconstruction_shape(optics, illumination, image_shape, reconstruction_shape="smooth"):
    k = illumination.resolve(optics).k_vectors
    kx = np.ascontiguousarray(k[:, 0])
    ky = np.ascontiguousarray(k[:, 1])
    policy, mh, mw = _shape_args(reconstruction_shape)
    out_h, out_w = C.c_int32(mh), C.c_int32(mw)
    o = optics._struct()
    N.check(N.library().fpm_suggest_shape(C.byref(o), kx.size, N.ptr(kx, C.c_double), N.ptr(ky, C.c_double),
                                          int(image_shape[0]), int(image_shape[1]), policy, C.byref(out_h),
                                          C.byref(out_w)))
    return (out_h.value, out_w.value)


def compile_model(optics, illumination, image_shape, reconstruction_shape="smooth") -> ImagePlaneModel:
    """Compile experiment geometry into an immutable image-plane model."""
    k = illumination.resolve(optics).k_vectors
    n = k.shape[0]
    kx = np.ascontiguousarray(k[:, 0])
    ky = np.ascontiguousarray(k[:, 1])
    h, w = int(image_shape[0]), int(image_shape[1])
    policy, mh, mw = _shape_args(reconstruction_shape)
    out_h, out_w = C.c_int32(mh), C.c_int32(mw)
    start_row = np.zeros(n, np.int64)
    start_col = np.zeros(n, np.int64)
    off_row = np.zeros(n)
    off_col = np.zeros(n)
    pupil = np.zeros((h, w), np.complex128)
    support = np.zeros((h, w), np.uint8)
    dkx, dky = C.c_double(), C.c_double()
    o = optics._struct()
    N.check(N.library().fpm_compile_model(
        C.byref(o), n, N.ptr(kx, C.c_double), N.ptr(ky, C.c_double), h, w, policy, C.byref(out_h), C.byref(out_w),
        N.ptr(start_row, C.c_int64), N.ptr(start_col, C.c_int64), N.ptr(off_row, C.c_double),
        N.ptr(off_col, C.c_double), N.ptr(pupil, C.c_double), N.ptr(support, C.c_uint8), C.byref(dkx),
        C.byref(dky)))
    return ImagePlaneModel(
        image_shape=(h, w), reconstruction_shape=(out_h.value, out_w.value), k_vectors=k, start_row=start_row,
        start_col=start_col, offset_row=off_row, offset_col=off_col, pupil=pupil, pupil_support=support,
        frame_gains=np.ones(n), dkx=dkx.value, dky=dky.value, low_res_pixel_size=optics.object_pixel_size,
        wavelength=optics.wavelength_vacuum_m)


def compile_camera_model(model: ImagePlaneModel, camera) -> ImagePlaneModel:
    """CameraModel::compile_reconstruction_model (src/simulation/camera.rs:296-318)."""
    camera.validate_for_frame(model.image_shape[0] * model.image_shape[1])
    scale = camera.photons_per_pixel * camera.gain_counts_per_electron
    gains = model._gains * scale if model._gains is not None else np.full(model.frame_count, scale)
    additive = camera.dark_current_electrons * camera.gain_counts_per_electron + camera.offset_counts
    background = model._background
    if background is not None:
        background = background * scale + additive
    elif additive != 0.0:
        background = np.full(model.image_shape[0] * model.image_shape[1], additive)
    return model._replace(frame_gains=gains, background=background)


def _finite(x) -> bool:
    return x is not None and math.isfinite(x)
