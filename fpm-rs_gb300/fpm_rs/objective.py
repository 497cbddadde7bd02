"""The reconstruction objective's data term on host intensities.

`intensity_loss` mirrors the Python binding of the same name
(python/src/metrics.rs:248-269); the sum runs in libfpm_gpu.so
(`fpm_intensity_loss`), restating src/algorithms/objective.rs:27-72.
"""

from __future__ import annotations

import ctypes as C

import numpy as np

from . import _native as N

_LOSS_CODES = {"amplitude_mse": 0, "intensity_mse": 1, "poisson_nll": 2, "huber_amplitude": 3}


def intensity_loss(reference, candidate, loss_type: str) -> float:
    """Mean `loss_type` loss of the candidate intensities against the
    reference (measured) intensities, two 2-D float64 arrays with the same
    number of values, summed in row-major order."""
    ref = np.ascontiguousarray(reference, dtype=np.float64)
    cand = np.ascontiguousarray(candidate, dtype=np.float64)
    if ref.ndim != 2 or cand.ndim != 2:
        raise TypeError("reference and candidate must be 2-D float64 arrays")
    if ref.size != cand.size:
        raise ValueError("reference and candidate must have the same shape")
    if loss_type not in _LOSS_CODES:
        raise ValueError("unknown loss_type")
    out = C.c_double()
    N.check(N.library().fpm_intensity_loss(N.ptr(cand, C.c_double), N.ptr(ref, C.c_double), C.c_int64(ref.size),
                                           _LOSS_CODES[loss_type], C.byref(out)))
    return out.value
