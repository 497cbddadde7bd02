"""Checkpoints: resumable reconstruction state and the CheckpointEvery callback.

Mirrors ReconstructionCheckpoint (src/reconstruction/checkpoint.rs:38-146)
and CheckpointEvery (src/callbacks/checkpoint.rs:8-39). The state held is
what this device path keeps between iterations: the centred object
spectrum, the pupil, the mPIE velocity, anchor and momentum counter, the
gradient-descent illumination corrections, and the objective trace. The device works in complex64, so the complex128
arrays stored here restore it exactly and a resumed run reproduces the
uninterrupted one bit for bit.

Files are JSON (format version 2, the reference's current version):
complex arrays as {"shape": [rows, cols], "re": [...], "im": [...]}, row-major.
"""

from __future__ import annotations

import json
import os
import tempfile
from dataclasses import dataclass, field
from pathlib import Path

import numpy as np

from .callbacks import Callback, _interval, _next_multiple
from .errors import InvalidParameterError, json_file_errors

FORMAT_VERSION = 2


def _encode(array: np.ndarray | None):
    if array is None:
        return None
    a = np.ascontiguousarray(array, dtype=np.complex128)
    return {"shape": list(a.shape), "re": a.real.ravel().tolist(), "im": a.imag.ravel().tolist()}


def _decode(value) -> np.ndarray | None:
    if value is None:
        return None
    shape = tuple(int(v) for v in value["shape"])
    re = np.asarray(value["re"], dtype=np.float64)
    im = np.asarray(value["im"], dtype=np.float64)
    if re.size != int(np.prod(shape)) or im.size != re.size:
        raise InvalidParameterError("checkpoint array does not match its shape")
    return (re + 1j * im).reshape(shape)


@dataclass
class ReconstructionCheckpoint:
    """Serializable algorithm state for resuming a compatible run."""

    completed_iterations: int
    algorithm: str
    object_spectrum: np.ndarray
    pupil: np.ndarray
    velocity: np.ndarray | None = None
    anchor: np.ndarray | None = None
    momentum_counter: int = 0
    objectives: list = field(default_factory=list)
    format_version: int = FORMAT_VERSION
    illumination_corrections: np.ndarray | None = None  # (sources, 2) row/column, or None

    def save(self, path) -> None:
        """Atomically serialize this checkpoint (write to a temporary file, then rename)."""
        with json_file_errors(path):
            self._save(path)

    def _save(self, path) -> None:
        path = Path(path)
        doc = {
            "format_version": self.format_version,
            "completed_iterations": int(self.completed_iterations),
            "algorithm": self.algorithm,
            "object_spectrum": _encode(self.object_spectrum),
            "pupil": _encode(self.pupil),
            "algorithm_auxiliary": None if self.velocity is None else {
                "Mpie": {"velocity": _encode(self.velocity), "anchor": _encode(self.anchor),
                         "momentum_counter": int(self.momentum_counter)}},
            "trace": [float(v) for v in self.objectives],
            "illumination_corrections": None if self.illumination_corrections is None else [
                [float(r), float(c)] for r, c in np.asarray(self.illumination_corrections, np.float64)],
        }
        fd, tmp = tempfile.mkstemp(dir=path.parent, prefix=path.name, suffix=".tmp")
        try:
            with os.fdopen(fd, "w") as f:
                json.dump(doc, f)
            os.replace(tmp, path)
        except BaseException:
            if os.path.exists(tmp):
                os.unlink(tmp)
            raise

    @staticmethod
    def load(path) -> "ReconstructionCheckpoint":
        """Read and validate a checkpoint file."""
        with json_file_errors(path):
            return ReconstructionCheckpoint._load(path)

    @staticmethod
    def _load(path) -> "ReconstructionCheckpoint":
        with open(path) as f:
            doc = json.load(f)
        version = int(doc.get("format_version", -1))
        if version != FORMAT_VERSION:
            raise InvalidParameterError(f"unsupported checkpoint format version {version}")
        aux = doc.get("algorithm_auxiliary") or {}
        mpie = aux.get("Mpie")
        cp = ReconstructionCheckpoint(
            completed_iterations=int(doc["completed_iterations"]),
            algorithm=str(doc["algorithm"]),
            object_spectrum=_decode(doc["object_spectrum"]),
            pupil=_decode(doc["pupil"]),
            velocity=_decode(mpie["velocity"]) if mpie else None,
            anchor=_decode(mpie["anchor"]) if mpie else None,
            momentum_counter=int(mpie["momentum_counter"]) if mpie else 0,
            objectives=[float(v) for v in doc.get("trace", [])],
            format_version=version,
            illumination_corrections=None if doc.get("illumination_corrections") is None else np.asarray(
                doc["illumination_corrections"], np.float64).reshape(-1, 2),
        )
        if len(cp.objectives) != cp.completed_iterations:
            raise InvalidParameterError("checkpoint trace length differs from its completed iterations")
        return cp


class CheckpointEvery(Callback):
    """Saves a checkpoint every `every` completed iterations into `directory`
    as checkpoint_<iteration, 5 digits>.json; a zero interval becomes one
    (src/callbacks/checkpoint.rs:8-39)."""

    def __init__(self, every: int, directory):
        self.every = _interval(every)
        self.directory = Path(directory)

    def path_for(self, iteration: int) -> Path:
        return self.directory / f"checkpoint_{iteration:05d}.json"

    def _next_state(self, current: int) -> int:
        return _next_multiple(current, self.every)

    def on_start(self, context) -> None:
        self.directory.mkdir(parents=True, exist_ok=True)

    def on_iteration_end(self, context) -> bool:
        if context.iteration % self.every == 0:
            context.checkpoint().save(self.path_for(context.iteration))
        return False
