"""Reconstruction callbacks: progress, CSV history, plateau stop, image saves
and Python iteration hooks.

Mirrors the Callback trait (src/callbacks/context.rs:58-91) and its built-in
implementations: ProgressLogger (src/callbacks/progress.rs:6-49), CsvLogger
(src/callbacks/csv_logger.rs:8-50), StopOnPlateau
(src/callbacks/early_stop.rs:6-68), SaveImageEvery / SavePupilEvery /
SaveResidualsEvery (src/callbacks/save_image.rs:11-181) and the Python
IterationCallback (python/src/reconstruction.rs:913-1000), with the
constructor rules of their Python wrappers (python/src/reconstruction.rs:
822-911: a zero interval becomes one).

The device runs whole iterations inside its frame-engine launches, so hooks
run on the host at iteration boundaries from copies of the device state. A
callback tells the runner two things ahead of time: the iterations at which
its hook needs the reconstruction state (object, pupil, residual images or a
checkpoint), and the first iteration at which it could ask to stop. The
runner ends a device segment at every iteration that needs state; hooks that
read only the objective are replayed in order after the segment from the
per-iteration objectives the device records. When a hook asks to stop inside
a segment, the runner re-runs that segment from its starting state up to the
stopping iteration, so the returned state is the one the reference would
return (the resumable device path reproduces an uninterrupted run bit for
bit).
"""

from __future__ import annotations

import math
import struct
import sys
import zlib
from dataclasses import dataclass, field
from pathlib import Path

import numpy as np

_NEVER = sys.maxsize
_is_callable = callable
_EPSILON = float(np.finfo(np.float64).eps)


def _interval(every) -> int:
    every = int(every)
    if every < 0:
        raise OverflowError("can't convert negative int to unsigned")
    return max(every, 1)


def _next_multiple(current: int, every: int) -> int:
    """The first multiple of `every` above `current`."""
    return (current // every + 1) * every


class Callback:
    """Host hook run at iteration boundaries of a device reconstruction.

    Subclasses override the hooks they need. `_next_state(current)` gives
    the first iteration after `current` whose iteration-end hook reads the
    reconstruction state; `_earliest_stop(current)` gives the first
    iteration after `current` at which `on_iteration_end` could return a
    stop request.
    """

    def _next_state(self, current: int) -> int:
        return _NEVER

    def _earliest_stop(self, current: int) -> int:
        return _NEVER

    def on_start(self, context: "StepContext") -> None:
        pass

    def on_iteration_end(self, context: "StepContext") -> bool:
        """Returns True to stop after this iteration."""
        return False

    def on_finish(self, result) -> None:
        pass


@dataclass
class StepContext:
    """What a hook sees at one iteration boundary (src/callbacks/context.rs:34-55).

    `iteration` is one-based (zero at the start hook); `objective` is that
    iteration's weighted mean objective; `trace` holds the records
    (iteration, objective, elapsed_seconds) completed so far. The state
    accessors are available at the iterations a callback declared through
    `_next_state`.
    """

    iteration: int
    objective: float | None
    trace: list
    problem_name: str | None
    algorithm: str
    _state: object = field(default=None, repr=False)

    def _require_state(self):
        if self._state is None:
            raise RuntimeError(f"reconstruction state is not available at iteration {self.iteration}")
        return self._state

    @property
    def object(self) -> np.ndarray:
        """Real-space complex object (the device's inverse FFT of the spectrum)."""
        return self._require_state().object()

    @property
    def object_spectrum(self) -> np.ndarray:
        return self._require_state().arrays["object_spectrum"]

    @property
    def pupil(self) -> np.ndarray:
        return self._require_state().arrays["pupil"]

    def residual_images(self) -> np.ndarray:
        """Predicted minus measured intensity per frame, zero at masked pixels
        (src/reconstruction/runner.rs:384-395)."""
        return self._require_state().residual_images()

    def checkpoint(self):
        return self._require_state().checkpoint()


# -- number formats of the reference's writers --------------------------------


def _shortest_digits(value: float):
    """Shortest round-trip decimal digits and exponent of a finite positive
    float: value = 0.d1d2...dn * 10**point."""
    text = repr(value)
    mantissa, _, exponent = text.partition("e")
    exponent = int(exponent) if exponent else 0
    whole, _, fraction = mantissa.partition(".")
    digits = (whole + fraction).lstrip("0")
    point = len(whole) + exponent - (len(whole + fraction) - len((whole + fraction).lstrip("0")))
    digits = digits.rstrip("0") or "0"
    return digits, point


def shortest_float(value: float) -> str:
    """A float as Rust's shortest round-trip writer prints it in CSV records
    (decimal notation for 1e-5 < |x| < 1e16, else d.ddde<exp>; "NaN", "inf")."""
    value = float(value)
    if math.isnan(value):
        return "NaN"
    if math.isinf(value):
        return "inf" if value > 0 else "-inf"
    sign = "-" if math.copysign(1.0, value) < 0 else ""
    value = abs(value)
    if value == 0.0:
        return sign + "0.0"
    digits, point = _shortest_digits(value)
    n = len(digits)
    if 0 <= point - n and point <= 16:
        return sign + digits + "0" * (point - n) + ".0"
    if 0 < point <= 16:
        return sign + digits[:point] + "." + digits[point:]
    if -5 < point <= 0:
        return sign + "0." + "0" * (-point) + digits
    exponent = point - 1
    if n == 1:
        return f"{sign}{digits}e{exponent}"
    return f"{sign}{digits[0]}.{digits[1:]}e{exponent}"


def scientific(value: float, precision: int = 6) -> str:
    """Rust's `{:.6e}`: mantissa with `precision` decimals, exponent without
    sign padding (1.234500e-3, 2.000000e0, NaN, inf)."""
    value = float(value)
    if math.isnan(value):
        return "NaN"
    if math.isinf(value):
        return "inf" if value > 0 else "-inf"
    mantissa, _, exponent = f"{value:.{precision}e}".partition("e")
    return f"{mantissa}e{int(exponent)}"


# -- grayscale PNG (src/reconstruction/result.rs:415-466) ---------------------


def grayscale_pixels(values, value_range) -> np.ndarray:
    """8-bit pixels of `values` mapped linearly from value_range to 0..255,
    clamped, rounded half away from zero."""
    minimum, maximum = value_range
    span = max(maximum - minimum, _EPSILON)
    scaled = np.clip((np.asarray(values, np.float64) - minimum) / span, 0.0, 1.0) * 255.0
    rounded = np.floor(scaled)
    rounded += (scaled - rounded) >= 0.5
    return rounded.astype(np.uint8)


def _png_chunk(kind: bytes, payload: bytes) -> bytes:
    return struct.pack(">I", len(payload)) + kind + payload + struct.pack(">I", zlib.crc32(kind + payload))


def write_png(path, pixels: np.ndarray) -> None:
    """Writes an 8-bit grayscale PNG (filter type 0 on every row)."""
    pixels = np.ascontiguousarray(pixels, np.uint8)
    height, width = pixels.shape
    raw = np.zeros((height, width + 1), np.uint8)
    raw[:, 1:] = pixels
    header = struct.pack(">IIBBBBB", width, height, 8, 0, 0, 0, 0)
    data = (b"\x89PNG\r\n\x1a\n" + _png_chunk(b"IHDR", header) + _png_chunk(b"IDAT", zlib.compress(raw.tobytes(), 6))
            + _png_chunk(b"IEND", b""))
    Path(path).write_bytes(data)


def read_png(path) -> np.ndarray:
    """Reads an 8-bit grayscale PNG written by `write_png` (filter type 0)."""
    data = Path(path).read_bytes()
    if data[:8] != b"\x89PNG\r\n\x1a\n":
        raise ValueError("not a PNG file")
    pos, width, height, idat = 8, 0, 0, b""
    while pos < len(data):
        (length,) = struct.unpack(">I", data[pos:pos + 4])
        kind = data[pos + 4:pos + 8]
        payload = data[pos + 8:pos + 8 + length]
        if kind == b"IHDR":
            width, height, depth, color = struct.unpack(">IIBB", payload[:10])
            if depth != 8 or color != 0:
                raise ValueError("only 8-bit grayscale PNG files are read")
        elif kind == b"IDAT":
            idat += payload
        pos += 12 + length
    raw = np.frombuffer(zlib.decompress(idat), np.uint8).reshape(height, width + 1)
    if np.any(raw[:, 0] != 0):
        raise ValueError("only unfiltered rows are read")
    return raw[:, 1:].copy()


def save_grayscale(values, path, phase: bool) -> None:
    values = np.asarray(values, np.float64)
    value_range = (-math.pi, math.pi) if phase else (float(values.min()), float(values.max()))
    write_png(path, grayscale_pixels(values, value_range))


def save_signed_grayscale(values, path) -> None:
    values = np.asarray(values, np.float64)
    extent = max(float(np.abs(values).max()) if values.size else 0.0, _EPSILON)
    write_png(path, grayscale_pixels(values, (-extent, extent)))


# -- built-in callbacks -------------------------------------------------------


class ProgressLogger(Callback):
    """Prints `iteration <5 wide>: objective <{:.6e}>` to standard error every
    `every` completed iterations (src/callbacks/progress.rs:38-48)."""

    def __init__(self, *, every: int = 1):
        self.every = _interval(every)

    def on_iteration_end(self, context: StepContext) -> bool:
        if context.iteration % self.every == 0 and context.objective is not None:
            print(f"iteration {context.iteration:>5}: objective {scientific(context.objective)}", file=sys.stderr)
        return False


class CsvLogger(Callback):
    """Replaces `path` at the start hook with the header
    iteration,objective,elapsed_seconds and appends the latest trace record
    at every iteration end (src/callbacks/csv_logger.rs:36-49)."""

    def __init__(self, path):
        self.path = Path(path)
        self._handle = None

    def on_start(self, context: StepContext) -> None:
        if self._handle is not None:
            self._handle.close()
        self._handle = open(self.path, "w", newline="")
        self._handle.write("iteration,objective,elapsed_seconds\n")
        self._handle.flush()

    def on_iteration_end(self, context: StepContext) -> bool:
        if self._handle is not None and context.trace:
            iteration, objective, elapsed = context.trace[-1]
            self._handle.write(f"{int(iteration)},{shortest_float(objective)},{shortest_float(elapsed)}\n")
            self._handle.flush()
        return False

    def on_finish(self, result) -> None:
        if self._handle is not None:
            self._handle.close()
            self._handle = None


class StopOnPlateau(Callback):
    """Stops once the objective has failed to drop by more than
    `minimum_improvement` below its best value for `patience` consecutive
    iterations (src/callbacks/early_stop.rs:6-68). The start hook rebuilds
    the counter from a resumed run's trace."""

    def __init__(self, patience: int, *, minimum_improvement: float = 0.0):
        self.patience = _interval(patience)
        self.minimum_improvement = max(float(minimum_improvement), 0.0)
        self._best = math.inf
        self._stale = 0

    def _observe(self, objective: float) -> None:
        if self._best - objective > self.minimum_improvement:
            self._best = objective
            self._stale = 0
        else:
            self._stale += 1

    def _earliest_stop(self, current: int) -> int:
        return current + max(self.patience - self._stale, 1)

    def on_start(self, context: StepContext) -> None:
        self._best = math.inf
        self._stale = 0
        for _, objective, _ in context.trace:
            self._observe(objective)

    def on_iteration_end(self, context: StepContext) -> bool:
        if context.objective is not None:
            self._observe(context.objective)
        return self._stale >= self.patience


class _DirectoryCallback(Callback):
    def __init__(self, every: int, directory):
        self.every = _interval(every)
        self.directory = Path(directory)

    def _next_state(self, current: int) -> int:
        return _next_multiple(current, self.every)

    def on_start(self, context: StepContext) -> None:
        self.directory.mkdir(parents=True, exist_ok=True)


class SaveImageEvery(_DirectoryCallback):
    """Saves amplitude_<it>.png (min..max) and phase_<it>.png (-pi..pi) of
    the object every `every` iterations (src/callbacks/save_image.rs:11-73)."""

    def on_iteration_end(self, context: StepContext) -> bool:
        if context.iteration % self.every == 0:
            obj = context.object
            save_grayscale(np.abs(obj), self.directory / f"amplitude_{context.iteration:05d}.png", False)
            save_grayscale(np.angle(obj), self.directory / f"phase_{context.iteration:05d}.png", True)
        return False


class SavePupilEvery(_DirectoryCallback):
    """Saves pupil_amplitude_<it>.png and pupil_phase_<it>.png of the
    recovered pupil every `every` iterations (src/callbacks/save_image.rs:75-134)."""

    def on_iteration_end(self, context: StepContext) -> bool:
        if context.iteration % self.every == 0:
            pupil = context.pupil
            save_grayscale(np.abs(pupil), self.directory / f"pupil_amplitude_{context.iteration:05d}.png", False)
            save_grayscale(np.angle(pupil), self.directory / f"pupil_phase_{context.iteration:05d}.png", True)
        return False


class SaveResidualsEvery(_DirectoryCallback):
    """Saves residual_<it>_frame_<frame>.png per measured frame, scaled
    symmetrically around zero (src/callbacks/save_image.rs:136-181)."""

    def on_iteration_end(self, context: StepContext) -> bool:
        if context.iteration % self.every == 0:
            for frame, residual in enumerate(context.residual_images()):
                save_signed_grayscale(residual, self.directory / f"residual_{context.iteration:05d}_frame_{frame:05d}.png")
        return False


class IterationCallback(Callback):
    """Calls `callable(mapping)` every `every` iterations with the keys
    iteration, objective, algorithm_metrics, problem_name and
    physical_illumination_calibration; a falsy return other than None stops
    the run (python/src/reconstruction.rs:936-1000)."""

    def __init__(self, callable, *, every: int = 1):
        if not _is_callable(callable):
            raise TypeError("callable must be callable")
        self.callable = callable
        self.every = _interval(every)

    def _earliest_stop(self, current: int) -> int:
        return _next_multiple(current, self.every)

    def on_iteration_end(self, context: StepContext) -> bool:
        if context.iteration % self.every:
            return False
        values = {
            "iteration": context.iteration,
            "objective": context.objective,
            "algorithm_metrics": [],
            "physical_illumination_calibration": None,
            "problem_name": context.problem_name,
        }
        response = self.callable(values)
        return not (response is None or bool(response))


def plan_segment(callbacks, current: int, total: int, speculation: int) -> int:
    """The iteration a device segment starting after `current` ends at.

    It ends at the first iteration whose hooks need the state, and no later
    than `total`. When a hook could ask to stop earlier than that, the
    segment runs at most `speculation` iterations past `current` or up to
    the first possible stop, whichever is later: a stop inside the segment
    is then undone by re-running it to the stopping iteration.
    """
    if current >= total:
        return total
    end = min([total] + [cb._next_state(current) for cb in callbacks])
    earliest = min((cb._earliest_stop(current) for cb in callbacks), default=_NEVER)
    if earliest < end:
        end = min(end, max(earliest, current + max(int(speculation), 1)))
    return max(end, current + 1)
