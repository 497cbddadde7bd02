"""Exception hierarchy of the fpm_rs Python API (python/src/errors.rs:4-50)."""

from __future__ import annotations

import contextlib
import json
import os


class FpmError(Exception):
    """Base class for errors raised by the device backend."""


class InvalidShapeError(FpmError):
    pass


class InvalidParameterError(FpmError):
    pass


class InvalidModelError(FpmError):
    pass


class InvalidMeasurementsError(FpmError):
    pass


class LengthMismatchError(FpmError):
    pass


class FrameOutOfRangeError(FpmError):
    pass


class NumericalError(FpmError):
    pass


class UnsupportedError(FpmError):
    pass


class DatasetError(FpmError):
    pass


class FpmIoError(FpmError):
    """A file could not be read or written (Error::Io)."""


class SerializationError(FpmError):
    """A file's contents could not be decoded (Error::Serialization)."""


@contextlib.contextmanager
def json_file_errors(path):
    """Maps failures of a JSON file operation as python/src/errors.rs:17-50
    maps Error::Io and Error::Serialization: file-system errors become
    FpmIoError, malformed or incomplete JSON becomes SerializationError."""
    try:
        yield
    except OSError as error:
        raise FpmIoError(f"{os.fspath(path)}: {error}") from error
    except (json.JSONDecodeError, KeyError, TypeError, IndexError) as error:
        raise SerializationError(f"{os.fspath(path)}: {error!r}") from error


class DeviceError(FpmError):
    """A CUDA runtime call failed or no suitable GPU is present."""


class ServerBusyError(FpmError):
    """The serving loop's queue is full; the request was not taken."""


_BY_STATUS = {
    1: InvalidShapeError,
    2: InvalidParameterError,
    3: InvalidModelError,
    4: InvalidMeasurementsError,
    5: LengthMismatchError,
    6: FrameOutOfRangeError,
    7: NumericalError,
    8: UnsupportedError,
    9: DeviceError,
    10: DeviceError,
    11: ServerBusyError,
}


def from_status(status: int, message: str) -> FpmError:
    return _BY_STATUS.get(status, FpmError)(message)
