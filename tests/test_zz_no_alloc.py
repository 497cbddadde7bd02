"""The allocation-free FFT entry point against the ordinary one.

fpm_fft2_noalloc exists for callers that cannot call cudaMalloc (device
memory owned by another allocator or admitted against a fixed HBM budget;
loops that must not synchronise the device). It keeps its scratch in one
fixed device array, so two calls in a row must both match fpm_fft2 exactly
as any other FP64 transform here does (1e-12 relative). This file is
collected last so that a failure here never hides the rest of the suite.
"""

from __future__ import annotations

import ctypes as C
import threading

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

# (144, 4096) takes the shared-memory power-of-two line path at the longest
# allowed row; 4093 is prime, so (143, 4093) takes the generic-radix path.
SHAPES = [((7, 9), 0), ((729, 729), 1), ((42, 42), 0), ((336, 336), 0), ((768, 768), 1), ((256, 256), 0),
          ((144, 4096), 0), ((143, 4093), 1)]


@pytest.fixture(scope="module")
def lib_and_ctx(native_library):
    lib = C.CDLL(native_library)
    lib.fpm_global_last_error.restype = C.c_char_p
    ctx = C.c_void_p()
    status = lib.fpm_create(C.byref(ctx), 0)
    assert status == 0, lib.fpm_global_last_error()
    yield lib, ctx
    lib.fpm_destroy(ctx)


def _call(lib, ctx, name, values, inverse):
    out = np.array(values, dtype=np.complex128, order="C", copy=True)
    status = getattr(lib, name)(ctx, out.ctypes.data_as(C.POINTER(C.c_double)), out.shape[0], out.shape[1],
                                int(inverse))
    return status, out


def test_noalloc_matches_fft2_on_consecutive_calls(lib_and_ctx):
    lib, ctx = lib_and_ctx
    rng = np.random.default_rng(11)
    for call in range(2):
        for shape, inverse in SHAPES:
            values = rng.standard_normal(shape) + 1j * rng.standard_normal(shape)
            status, expected = _call(lib, ctx, "fpm_fft2", values, inverse)
            assert status == 0
            status, got = _call(lib, ctx, "fpm_fft2_noalloc", values, inverse)
            assert status == 0, f"call {call} shape {shape}"
            scale = max(1.0, float(np.abs(expected).max()))
            assert np.abs(got - expected).max() <= 1e-12 * scale, f"call {call} shape {shape}"


@pytest.mark.parametrize("shape", [(769, 769), (1, 4097)])
def test_noalloc_rejects_shapes_beyond_its_scratch(lib_and_ctx, shape):
    lib, ctx = lib_and_ctx
    status, _ = _call(lib, ctx, "fpm_fft2_noalloc", np.zeros(shape, np.complex128), 0)
    assert status == 1  # FPM_ERR_INVALID_SHAPE
    buf = C.create_string_buffer(512)
    lib.fpm_last_error(ctx, buf, len(buf))
    assert b"exceeds its fixed scratch" in buf.value


def test_noalloc_allocates_no_device_memory(lib_and_ctx):
    torch = pytest.importorskip("torch")
    lib, ctx = lib_and_ctx
    rng = np.random.default_rng(5)
    cases = [(shape, inverse, rng.standard_normal(shape) + 1j * rng.standard_normal(shape))
             for shape, inverse in SHAPES]
    for shape, inverse, values in cases:  # warm-up: the array and its kernels are resident afterwards
        assert _call(lib, ctx, "fpm_fft2_noalloc", values, inverse)[0] == 0
    torch.cuda.synchronize(0)
    free_before, _ = torch.cuda.mem_get_info(0)
    for _ in range(3):
        for shape, inverse, values in cases:
            assert _call(lib, ctx, "fpm_fft2_noalloc", values, inverse)[0] == 0
    torch.cuda.synchronize(0)
    free_after, _ = torch.cuda.mem_get_info(0)
    assert free_after == free_before


def test_noalloc_and_fft2_alternate_on_one_context_from_two_threads(lib_and_ctx):
    lib, ctx = lib_and_ctx
    rng = np.random.default_rng(23)
    values = rng.standard_normal((336, 336)) + 1j * rng.standard_normal((336, 336))
    status, expected = _call(lib, ctx, "fpm_fft2", values, 0)
    assert status == 0
    failures = []

    def worker(first):
        names = ("fpm_fft2_noalloc", "fpm_fft2") if first else ("fpm_fft2", "fpm_fft2_noalloc")
        for k in range(8):
            status, got = _call(lib, ctx, names[k % 2], values, 0)
            if status != 0 or np.abs(got - expected).max() > 1e-12 * max(1.0, float(np.abs(expected).max())):
                failures.append((names[k % 2], k, status))

    threads = [threading.Thread(target=worker, args=(first,)) for first in (True, False)]
    for t in threads:
        t.start()
    for t in threads:
        t.join()
    assert not failures
