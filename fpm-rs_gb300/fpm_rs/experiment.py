"""Experiment description: optics, LED geometry, illumination and camera.

Mirrors the fpm_rs Python classes of the same names
(python/fpm_rs/__init__.pyi: Optics 1411-1480, ArrayPose 1481-1511,
PlanarLEDArray 1512-1560, DirectionList 1716-1763, KVectorList 1764-1780, Illumination 1871-1895,
CameraModel 1956-2006). Resolution to k-vectors runs in the native library.
"""

from __future__ import annotations

import ctypes as C
import math
from dataclasses import dataclass, field
from fractions import Fraction

import numpy as np

from . import _native as N
from .errors import InvalidParameterError, UnsupportedError


@dataclass(frozen=True)
class PupilAberration:
    """Direct radian weights of the crate's pupil phase terms (src/experiment/optics.rs:84-94)."""

    astigmatism: float = 0.0
    coma: float = 0.0
    spherical: float = 0.0
    edge_apodization: float = 0.0

    def __post_init__(self):
        values = (self.astigmatism, self.coma, self.spherical, self.edge_apodization)
        if any(not math.isfinite(v) for v in values) or self.edge_apodization < 0.0:
            raise InvalidParameterError(
                "pupil_aberration: phase coefficients must be finite and edge apodization must be "
                "finite and non-negative")


class Optics:
    """Physical microscope parameters used to compile an image-plane model."""

    def __init__(self, wavelength_vacuum_m: float, objective_na: float, magnification: float,
                 camera_pixel_size: float, *, illumination_refractive_index: float = 1.0,
                 objective_medium_refractive_index: float = 1.0,
                 defocus_distance: float | None = None,
                 pupil_aberration: PupilAberration | None = None):
        self.wavelength_vacuum_m = float(wavelength_vacuum_m)
        self.objective_na = float(objective_na)
        self.magnification = float(magnification)
        self.camera_pixel_size = float(camera_pixel_size)
        self.illumination_refractive_index = float(illumination_refractive_index)
        self.objective_medium_refractive_index = float(objective_medium_refractive_index)
        self.defocus_distance = None if defocus_distance is None else float(defocus_distance)
        self.pupil_aberration = pupil_aberration
        self._validate()

    def _validate(self) -> None:
        for name in ("wavelength_vacuum_m", "objective_na", "magnification", "camera_pixel_size",
                     "illumination_refractive_index", "objective_medium_refractive_index"):
            value = getattr(self, name)
            if not math.isfinite(value) or value <= 0.0:
                raise InvalidParameterError(f"{name} must be finite and positive, got {value}")
        if self.objective_na > self.objective_medium_refractive_index:
            raise InvalidParameterError("objective_na cannot exceed the medium refractive index")
        pitch = self.object_pixel_size
        limit = self.wavelength_vacuum_m / (2.0 * self.objective_na)
        if not pitch < limit:
            raise InvalidParameterError(
                f"object-plane pitch camera_pixel_size / magnification ({pitch:.6e} m) must be strictly "
                f"less than wavelength_vacuum_m / (2 * objective_na) ({limit:.6e} m)")
        if self.defocus_distance is not None and not math.isfinite(self.defocus_distance):
            raise InvalidParameterError("defocus_distance must be finite")

    @property
    def object_pixel_size(self) -> float:
        return self.camera_pixel_size / self.magnification

    def _struct(self) -> N.Optics:
        o = N.Optics()
        o.wavelength_vacuum_m = self.wavelength_vacuum_m
        o.objective_na = self.objective_na
        o.magnification = self.magnification
        o.camera_pixel_size = self.camera_pixel_size
        o.illumination_refractive_index = self.illumination_refractive_index
        o.objective_medium_refractive_index = self.objective_medium_refractive_index
        o.has_defocus = int(self.defocus_distance is not None)
        o.defocus_distance = self.defocus_distance or 0.0
        ab = self.pupil_aberration
        o.has_aberration = int(ab is not None)
        if ab is not None:
            o.astigmatism, o.coma, o.spherical, o.edge_apodization = (
                ab.astigmatism, ab.coma, ab.spherical, ab.edge_apodization)
        return o


@dataclass(frozen=True)
class ArrayPose:
    """Rigid array-local to sample transform; rotation is extrinsic x, y, then z."""

    translation_m: tuple = (0.0, 0.0, 0.0)
    rotation_rad: tuple = (0.0, 0.0, 0.0)

    @staticmethod
    def identity() -> "ArrayPose":
        return ArrayPose()

    @staticmethod
    def from_translation(translation_m) -> "ArrayPose":
        return ArrayPose(tuple(float(v) for v in translation_m))

    @staticmethod
    def from_translation_and_extrinsic_xyz_radians(translation_m, rotation_rad) -> "ArrayPose":
        return ArrayPose(tuple(float(v) for v in translation_m), tuple(float(v) for v in rotation_rad))

    @staticmethod
    def from_translation_and_extrinsic_xyz_degrees(translation_m, rotation_deg) -> "ArrayPose":
        return ArrayPose(tuple(float(v) for v in translation_m),
                         tuple(math.radians(float(v)) for v in rotation_deg))


class ResolvedSources:
    """Resolved sources (src/experiment/illumination.rs:377-440): transverse
    k-vectors, propagation unit vectors, and source positions for physical
    geometries (None for direction and k-vector lists)."""

    def __init__(self, k_vectors: np.ndarray, directions: np.ndarray, positions_m: np.ndarray | None = None):
        self._k = np.ascontiguousarray(k_vectors, dtype=np.float64)
        self._directions = np.ascontiguousarray(directions, dtype=np.float64)
        self._positions = None if positions_m is None else np.ascontiguousarray(positions_m, dtype=np.float64)

    @property
    def source_count(self) -> int:
        return self._k.shape[0]

    @property
    def k_vectors(self) -> np.ndarray:
        return self._k.copy()

    @property
    def directions(self) -> np.ndarray:
        return self._directions.copy()

    @property
    def positions_m(self) -> np.ndarray | None:
        return None if self._positions is None else self._positions.copy()


class PlanarLEDArray:
    """Planar LED geometry (src/experiment/led_array.rs:292-313)."""

    def __init__(self, shape, pitch_m, reference_index, pose: ArrayPose, *, position_offsets_m=None):
        self.shape = (int(shape[0]), int(shape[1]))
        if np.isscalar(pitch_m):
            self.pitch_m = (float(pitch_m), float(pitch_m))
        else:
            self.pitch_m = (float(pitch_m[0]), float(pitch_m[1]))
        self.reference_index = (float(reference_index[0]), float(reference_index[1]))
        self.pose = pose
        if position_offsets_m is not None and np.any(np.asarray(position_offsets_m) != 0.0):
            raise UnsupportedError("position_offsets_m is not supported on the GB300 device path")
        if self.shape[0] <= 0 or self.shape[1] <= 0:
            raise InvalidParameterError("shape rows and columns must be non-zero")
        self._offsets = (np.zeros((0, 3)) if position_offsets_m is None
                         else np.array(position_offsets_m, dtype=np.float64).reshape(-1, 3))

    @property
    def position_offsets_m(self) -> np.ndarray:
        """Per-LED offsets (src/experiment/led_array.rs:202-204): empty unless
        given; only zero offsets are accepted here."""
        return self._offsets.copy()

    @property
    def source_count(self) -> int:
        return self.shape[0] * self.shape[1]

    def source_index(self, row: int, column: int) -> int:
        return row * self.shape[1] + column

    def source_row_column(self, index: int):
        return (index // self.shape[1], index % self.shape[1])

    def resolve(self, optics: Optics) -> ResolvedSources:
        n = self.source_count
        kx = np.zeros(n)
        ky = np.zeros(n)
        t = np.asarray(self.pose.translation_m, dtype=np.float64)
        r = np.asarray(self.pose.rotation_rad, dtype=np.float64)
        o = optics._struct()
        N.check(N.library().fpm_planar_led_kvectors(
            C.byref(o), self.shape[0], self.shape[1], C.c_double(self.pitch_m[0]), C.c_double(self.pitch_m[1]),
            C.c_double(self.reference_index[0]), C.c_double(self.reference_index[1]),
            N.ptr(t, C.c_double), N.ptr(r, C.c_double), N.ptr(kx, C.c_double), N.ptr(ky, C.c_double)))
        positions, directions = self._positions_and_directions()
        return ResolvedSources(np.stack([kx, ky], axis=1), directions, positions)

    def _positions_and_directions(self):
        """LED positions and source-to-sample directions for the getters
        (led_array.rs:292-313, illumination.rs:385-410): the native
        compilation's operations, in its order and unfused, so k times a
        direction reproduces its k-vector bit for bit."""
        sx, cx = math.sin(self.pose.rotation_rad[0]), math.cos(self.pose.rotation_rad[0])
        sy, cy = math.sin(self.pose.rotation_rad[1]), math.cos(self.pose.rotation_rad[1])
        sz, cz = math.sin(self.pose.rotation_rad[2]), math.cos(self.pose.rotation_rad[2])
        t = [float(v) for v in self.pose.translation_m]
        positions, directions = [], []
        for r in range(self.shape[0]):
            for c in range(self.shape[1]):
                p = ((c - self.reference_index[0]) * self.pitch_m[0], (r - self.reference_index[1]) * self.pitch_m[1], 0.0)
                ax = (p[0], cx * p[1] - sx * p[2], sx * p[1] + cx * p[2])
                ay = (cy * ax[0] + sy * ax[2], ax[1], -sy * ax[0] + cy * ax[2])
                az = (cz * ay[0] - sz * ay[1], sz * ay[0] + cz * ay[1], ay[2])
                positions.append((az[0] + t[0], az[1] + t[1], az[2] + t[2]))
        return np.array(positions, dtype=np.float64), _directions_from_positions(positions)


def _directions_from_positions(positions) -> np.ndarray:
    """Source-to-sample unit vectors -p / |p| (ResolvedSources::from_positions,
    src/experiment/illumination.rs:385-410), |p| as hypot(hypot(x, y), z)."""
    directions = []
    for x, y, z in positions:
        if not (math.isfinite(x) and math.isfinite(y) and math.isfinite(z)):
            raise InvalidParameterError("positions_m: position components must be finite")
        norm = float(np.hypot(np.hypot(x, y), z))
        if not math.isfinite(norm) or norm <= 0.0:
            raise InvalidParameterError("positions_m: no source may coincide with the sample origin")
        directions.append((-x / norm, -y / norm, -z / norm))
    return np.array(directions, dtype=np.float64)


class SourcePositionList:
    """Explicit source positions in sample coordinates, metres
    (src/experiment/illumination.rs:45-72; python/src/config.rs:437-470)."""

    def __init__(self, positions_m):
        self._p = np.array(_pair_rows(positions_m, 3, "positions_m"), dtype=np.float64)

    @property
    def positions_m(self) -> np.ndarray:
        return self._p.copy()

    @property
    def source_count(self) -> int:
        return self._p.shape[0]

    def resolve(self, optics: Optics) -> ResolvedSources:
        optics._validate()
        directions = _directions_from_positions([tuple(float(v) for v in row) for row in self._p])
        k = 2.0 * math.pi * optics.illumination_refractive_index / optics.wavelength_vacuum_m
        return ResolvedSources(np.stack([k * directions[:, 0], k * directions[:, 1]], axis=1), directions, self._p)


_DIRECTION_TOLERANCE = 128.0 * np.finfo(np.float64).eps


def _pair_rows(values, width: int, name: str) -> list:
    """The binding's array copy (python/src/config.rs:1109-1140): a (sources,
    width) float64 array with at least one row, else ValueError."""
    a = np.asarray(values, dtype=np.float64)
    if a.ndim != 2 or a.shape[1] != width or a.shape[0] == 0:
        raise ValueError(f"{name} must have shape (sources, {width})")
    return [[float(x) for x in row] for row in a]


def _mul_add(a: float, b: float, c: float) -> float:
    """f64::mul_add: a * b + c with one rounding (exact rational arithmetic,
    then the correctly rounded conversion)."""
    return float(Fraction(a) * Fraction(b) + Fraction(c))


def _libm(f, x: float) -> float:
    """A libm function that, like Rust's, maps a non-finite input to NaN
    instead of raising."""
    return f(x) if math.isfinite(x) else math.nan


def _direction_vectors(vectors: list, normalize: bool) -> np.ndarray:
    """DirectionList::from_vectors (src/experiment/illumination.rs:91-126)."""
    out = []
    for x, y, z in vectors:
        if not (math.isfinite(x) and math.isfinite(y) and math.isfinite(z)):
            raise InvalidParameterError("unit_vectors: components must be finite")
        norm = float(np.hypot(np.hypot(x, y), z))
        if not math.isfinite(norm) or norm <= 0.0:
            raise InvalidParameterError("unit_vectors: vectors must have non-zero finite norm")
        if normalize:
            x, y, z = x / norm, y / norm, z / norm
        elif abs(norm - 1.0) > _DIRECTION_TOLERANCE:
            raise InvalidParameterError("unit_vectors: vectors must be normalized")
        if z < -_DIRECTION_TOLERANCE:
            raise InvalidParameterError("unit_vectors: directions must lie in the positive-z illumination hemisphere")
        out.append([x, y, max(z, 0.0)])
    return np.array(out, dtype=np.float64)


def _transverse_directions(pairs: list, component) -> np.ndarray:
    """from_transverse_components (src/experiment/illumination.rs:173-192):
    (dx, dy) = component of each pair, z = sqrt(max(1 - (dx^2 + dy^2), 0))
    with the magnitude formed by one fused multiply-add."""
    vectors = []
    for x, y in pairs:
        if not (math.isfinite(x) and math.isfinite(y)):
            raise InvalidParameterError("directions: components must be finite")
        dx, dy = component(x), component(y)
        squared = _mul_add(dx, dx, dy * dy)
        if squared > 1.0 + _DIRECTION_TOLERANCE:
            raise InvalidParameterError("directions: squared transverse direction magnitude cannot exceed one")
        vectors.append([dx, dy, math.sqrt(max(1.0 - squared, 0.0))])
    return _direction_vectors(vectors, False)


class DirectionList:
    """Illumination propagation directions (src/experiment/illumination.rs:76-254),
    stored as unit vectors with non-negative z; resolves to k * (ux, uy)
    with k = 2 pi n_illumination / wavelength. Constructors and getters follow
    python/src/config.rs:483-570."""

    def __init__(self, unit_vectors):
        self._u = _direction_vectors(_pair_rows(unit_vectors, 3, "unit_vectors"), False)

    @staticmethod
    def _of(unit_vectors: np.ndarray) -> "DirectionList":
        directions = DirectionList.__new__(DirectionList)
        directions._u = unit_vectors
        return directions

    @staticmethod
    def from_unit_vectors(values) -> "DirectionList":
        return DirectionList(values)

    @staticmethod
    def from_vectors(values, *, normalize: bool = True) -> "DirectionList":
        """Vectors of any non-zero length, each divided by its norm when
        `normalize` (else they must already be unit length)."""
        return DirectionList._of(_direction_vectors(_pair_rows(values, 3, "vectors"), bool(normalize)))

    @staticmethod
    def from_direction_cosines(values) -> "DirectionList":
        """Transverse direction cosines (dx, dy)."""
        return DirectionList._of(_transverse_directions(_pair_rows(values, 2, "directions"), lambda v: v))

    @staticmethod
    def from_component_angles_radians(values) -> "DirectionList":
        """Independent component angles (theta_x, theta_y): (sin theta_x, sin theta_y)."""
        return DirectionList._of(_transverse_directions(_pair_rows(values, 2, "directions"),
                                                        lambda v: _libm(math.sin, v)))

    @staticmethod
    def from_component_angles_degrees(values) -> "DirectionList":
        pairs = [[math.radians(x), math.radians(y)] for x, y in _pair_rows(values, 2, "directions")]
        return DirectionList._of(_transverse_directions(pairs, lambda v: _libm(math.sin, v)))

    @staticmethod
    def from_polar_angles_radians(values) -> "DirectionList":
        """Polar angle theta and azimuth phi: (sin theta cos phi, sin theta sin phi, cos theta)."""
        return DirectionList._of(DirectionList._polar(_pair_rows(values, 2, "directions")))

    @staticmethod
    def from_polar_angles_degrees(values) -> "DirectionList":
        pairs = [[math.radians(t), math.radians(f)] for t, f in _pair_rows(values, 2, "directions")]
        return DirectionList._of(DirectionList._polar(pairs))

    @staticmethod
    def _polar(pairs: list) -> np.ndarray:
        vectors = []
        for theta, phi in pairs:
            st, ct = _libm(math.sin, theta), _libm(math.cos, theta)
            sp, cp = _libm(math.sin, phi), _libm(math.cos, phi)
            vectors.append([st * cp, st * sp, ct])
        return _direction_vectors(vectors, False)

    @property
    def source_count(self) -> int:
        return self._u.shape[0]

    @property
    def unit_vectors(self) -> np.ndarray:
        return self._u.copy()

    @property
    def direction_cosines(self) -> np.ndarray:
        return self._u[:, :2].copy()

    @property
    def component_angles_rad(self) -> np.ndarray:
        return np.array([[math.asin(x), math.asin(y)] for x, y, _ in self._u], dtype=np.float64).reshape(-1, 2)

    @property
    def component_angles_deg(self) -> np.ndarray:
        return np.array([[math.degrees(x), math.degrees(y)] for x, y in self.component_angles_rad],
                        dtype=np.float64).reshape(-1, 2)

    @property
    def polar_angles_rad(self) -> np.ndarray:
        return np.array([[math.acos(min(max(z, -1.0), 1.0)), math.atan2(y, x)] for x, y, z in self._u],
                        dtype=np.float64).reshape(-1, 2)

    @property
    def polar_angles_deg(self) -> np.ndarray:
        return np.array([[math.degrees(t), math.degrees(f)] for t, f in self.polar_angles_rad],
                        dtype=np.float64).reshape(-1, 2)

    def resolve(self, optics: Optics) -> ResolvedSources:
        optics._validate()
        k = 2.0 * math.pi * optics.illumination_refractive_index / optics.wavelength_vacuum_m
        return ResolvedSources(np.stack([k * self._u[:, 0], k * self._u[:, 1]], axis=1), self._u)


class KVectorList:
    """Explicit transverse wave vectors, float64 (sources, 2) of (kx, ky) rad/m."""

    def __init__(self, k_vectors):
        k = np.asarray(k_vectors, dtype=np.float64)
        if k.ndim != 2 or k.shape[1] != 2 or k.shape[0] == 0:
            raise InvalidParameterError("k_vectors must have shape (sources, 2)")
        if not np.all(np.isfinite(k)):
            raise InvalidParameterError("k_vectors must contain finite values")
        self._k = k

    @property
    def source_count(self) -> int:
        return self._k.shape[0]

    @property
    def k_vectors(self) -> np.ndarray:
        return self._k.copy()

    def resolve(self, optics: Optics) -> ResolvedSources:
        """validate_k_vectors (src/experiment/illumination.rs:873-890): every
        vector must propagate at the illumination wavenumber."""
        optics._validate()
        k = 2.0 * math.pi * optics.illumination_refractive_index / optics.wavelength_vacuum_m
        if np.any(np.hypot(self._k[:, 0], self._k[:, 1]) > k * (1.0 + 128.0 * np.finfo(np.float64).eps)):
            raise InvalidParameterError("k_vectors: vectors must be finite and propagating at the configured vacuum "
                                        "wavelength and illumination refractive index")
        # KVectorList::resolve (src/experiment/illumination.rs:282-299): the
        # direction of (kx, ky) at the illumination wavenumber.
        directions = []
        for kx, ky in self._k:
            dx, dy = float(kx) / k, float(ky) / k
            directions.append([dx, dy, math.sqrt(max(1.0 - _mul_add(dx, dx, dy * dy), 0.0))])
        return ResolvedSources(self._k, np.array(directions, dtype=np.float64))


class SourceContribution:
    """One source's intensity weight within a frame (python/src/config.rs:694-722)."""

    def __init__(self, source: int, intensity_weight: float):
        self.source = int(source)
        self.intensity_weight = float(intensity_weight)


class ResolvedFrame:
    """A frame's source contributions and gain (src/experiment/illumination.rs:764-775)."""

    def __init__(self, contributions: list, gain: float):
        self.contributions = list(contributions)
        self.gain = float(gain)


class ResolvedIllumination:
    """Resolved sources plus the acquisition (src/experiment/illumination.rs:784-852).

    The device path takes only the unit calibration and the sequential
    all-sources plan, so frame f holds source f alone at unit weight, and
    source powers and frame gains are one."""

    def __init__(self, sources: ResolvedSources):
        self._sources = sources

    @property
    def sources(self) -> ResolvedSources:
        return self._sources

    @property
    def source_count(self) -> int:
        return self._sources.source_count

    @property
    def frame_count(self) -> int:
        return self._sources.source_count

    @property
    def is_multiplexed(self) -> bool:
        return False

    @property
    def frames(self) -> list:
        return [ResolvedFrame([SourceContribution(f, 1.0)], 1.0) for f in range(self.frame_count)]

    @property
    def source_power(self) -> np.ndarray:
        return np.ones(self.source_count)

    @property
    def frame_gains(self) -> np.ndarray:
        return np.ones(self.frame_count)

    @property
    def directions(self) -> np.ndarray:
        return self._sources.directions

    @property
    def positions_m(self):
        return self._sources.positions_m

    @property
    def k_vectors(self) -> np.ndarray:
        return self._sources.k_vectors

    @property
    def dense_weights(self) -> np.ndarray:
        return np.eye(self.frame_count, self.source_count)


class Illumination:
    """Geometry plus (unit) calibration and the all-sources sequential acquisition."""

    def __init__(self, geometry, *, calibration=None, acquisition=None):
        if calibration is not None or acquisition is not None:
            raise UnsupportedError(
                "source calibration and multiplexed acquisition plans are not supported on the GB300 device path")
        self.geometry = geometry
        # The unit calibration and the sequential all-sources plan, which are
        # the only ones the device path takes, read as None.
        self.calibration = None
        self.acquisition = None

    def resolve(self, optics: Optics) -> ResolvedIllumination:
        return ResolvedIllumination(self.geometry.resolve(optics))


@dataclass
class CameraModel:
    """Detector response and acquisition noise (src/simulation/camera.rs:249-318).

    Applied on the GPU by fpm_simulate_stack. Noise comes from a counter-based
    Philox-4x32-10 stream keyed by the seed, not the reference's ChaCha12
    stream, so simulated counts match the reference only in distribution.
    """

    photons_per_pixel: float = 1000.0
    gain_counts_per_electron: float = 1.0
    offset_counts: float = 0.0
    read_noise_electrons: float = 0.0
    dark_current_electrons: float = 0.0
    shot_noise: bool = False
    pixel_sensitivity: np.ndarray | None = None
    bit_depth: int | None = 16
    saturation_counts: float | None = None
    quantize: bool = True
    bad_pixels: tuple = field(default_factory=tuple)
    bad_pixel_value_counts: float | None = None

    @staticmethod
    def ideal() -> "CameraModel":
        return CameraModel(photons_per_pixel=1.0, bit_depth=None, quantize=False)

    def maximum_count(self) -> float:
        limit = math.inf
        if self.bit_depth is not None:
            limit = float(2 ** int(self.bit_depth) - 1)
        if self.saturation_counts is not None:
            limit = min(limit, float(self.saturation_counts))
        return limit

    def validate_for_frame(self, frame_len: int) -> None:
        """CameraModel::validate / validate_for_frame (src/simulation/camera.rs)."""
        for name in ("photons_per_pixel", "gain_counts_per_electron"):
            value = float(getattr(self, name))
            if not math.isfinite(value) or value <= 0.0:
                raise InvalidParameterError(f"{name} must be finite and positive")
        if (not math.isfinite(self.offset_counts) or not math.isfinite(self.read_noise_electrons)
                or self.read_noise_electrons < 0.0 or not math.isfinite(self.dark_current_electrons)
                or self.dark_current_electrons < 0.0):
            raise InvalidParameterError(
                "camera noise/offset: offset must be finite; read noise and dark current must be non-negative")
        if self.bit_depth is not None and not 1 <= int(self.bit_depth) <= 32:
            raise InvalidParameterError("bit_depth must be between 1 and 32")
        if self.saturation_counts is not None and (not math.isfinite(self.saturation_counts)
                                                   or self.saturation_counts <= 0.0):
            raise InvalidParameterError("saturation_counts must be finite and positive")
        if self.bad_pixel_value_counts is not None and (not math.isfinite(self.bad_pixel_value_counts)
                                                        or self.bad_pixel_value_counts < 0.0):
            raise InvalidParameterError("bad_pixel_value_counts must be finite and non-negative")
        if self.bad_pixels and self.bad_pixel_value_counts is None and not math.isfinite(self.maximum_count()):
            raise InvalidParameterError("bad_pixels: a finite bad-pixel value or camera maximum is required")
        if self.pixel_sensitivity is not None:
            sens = np.asarray(self.pixel_sensitivity, dtype=np.float64)
            if not np.all(np.isfinite(sens)) or np.any(sens < 0.0):
                raise InvalidParameterError("pixel_sensitivity values must be finite and non-negative")
            if sens.size != frame_len:
                raise InvalidParameterError(f"pixel_sensitivity must contain {frame_len} values")
        if len(set(self.bad_pixels)) != len(self.bad_pixels):
            raise InvalidParameterError("bad_pixels must not repeat")
        if any(int(p) < 0 or int(p) >= frame_len for p in self.bad_pixels):
            raise InvalidParameterError(f"bad_pixels indices must be below the frame size {frame_len}")

    def _descriptor(self, frame_len: int):
        """C-ABI descriptor (fpm_camera_desc) and the arrays it points into."""
        d = N.CameraDesc()
        d.photons_per_pixel = float(self.photons_per_pixel)
        d.gain_counts_per_electron = float(self.gain_counts_per_electron)
        d.offset_counts = float(self.offset_counts)
        d.read_noise_electrons = float(self.read_noise_electrons)
        d.dark_current_electrons = float(self.dark_current_electrons)
        d.shot_noise = int(bool(self.shot_noise))
        d.quantize = int(bool(self.quantize))
        d.maximum_count = float(self.maximum_count())
        keep = []
        if self.pixel_sensitivity is not None:
            sens = np.ascontiguousarray(self.pixel_sensitivity, dtype=np.float64).ravel()
            if sens.size != frame_len:
                raise InvalidParameterError("pixel_sensitivity must have one value per detector pixel")
            keep.append(sens)
            d.pixel_sensitivity = N.ptr(sens, C.c_double)
        bad = np.ascontiguousarray(list(self.bad_pixels), dtype=np.int64)
        keep.append(bad)
        d.bad_pixels = N.ptr(bad, C.c_int64) if bad.size else C.POINTER(C.c_int64)()
        d.bad_pixel_count = int(bad.size)
        d.bad_pixel_value = float("nan") if self.bad_pixel_value_counts is None else float(self.bad_pixel_value_counts)
        return d, keep
