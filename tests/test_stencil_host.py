"""The device stencil function (fpm::offset_frame_param in csrc/kernels.h,
used by the illumination update and checkpoint resume) against the oracle's
crop rules: CropIndices::validate_subpixel_inside and interpolation_axis
(src/model/crop.rs:105-113, 266-313). Compiled for the host with g++; the
same inline code runs on the device."""

from __future__ import annotations

import os
import shutil
import subprocess

import numpy as np
import pytest

import oracle

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def stencil_binary(tmp_path_factory):
    gxx = shutil.which("g++")
    cuda_include = "/usr/local/cuda/include"
    if gxx is None or not os.path.isdir(cuda_include):
        pytest.skip("g++ or the CUDA headers are unavailable")
    out = str(tmp_path_factory.mktemp("stencil") / "stencil_check")
    subprocess.run([gxx, "-O2", "-std=c++17", "-I", cuda_include, "-I", os.path.join(ROOT, "fpm-rs_gb300", "csrc"),
                    os.path.join(ROOT, "tests", "native", "stencil_check.cpp"), "-o", out], check=True)
    return out


def test_offset_stencil_matches_oracle_crop_rules(stencil_binary):
    rng = np.random.default_rng(12)
    n, m = 8, 16
    cases = []
    for _ in range(400):
        start = rng.integers(0, m - n + 1, size=2)
        offset = rng.choice([-1.5, -1.0, -0.5, -1e-13, 0.0, 1e-13, 0.3, 0.5, 0.999, 1.0, 1.2]) + \
            rng.uniform(-0.2, 0.2, size=2) * rng.integers(0, 2, size=2)
        cases.append((int(start[0]), int(start[1]), float(offset[0]), float(offset[1])))
    cases += [(0, 0, -1e-13, 0.0), (8, 8, 0.0, 0.0), (8, 8, 1e-6, 0.0), (7, 8, 0.5, 0.0), (0, 4, -0.01, 0.0)]
    text = "".join(f"{n} {m} {sr} {sc} {orow!r} {ocol!r}\n" for sr, sc, orow, ocol in cases)
    lines = subprocess.run([stencil_binary], input=text, capture_output=True, text=True,
                           check=True).stdout.splitlines()
    assert len(lines) == len(cases)
    rows, cols = np.indices((m, m))
    ramp = (1000.0 * rows + cols).astype(np.complex128)  # bilinear sampling of a ramp returns the position
    valid_seen = invalid_seen = 0
    for (sr, sc, orow, ocol), line in zip(cases, lines):
        f = line.split()
        valid = f[0] == "1"
        try:
            patch = oracle.extract_patch(ramp, (sr, sc), (n, n), (orow, ocol))
            expected_valid = True
        except oracle.OracleError:
            expected_valid = False
        assert valid == expected_valid, (sr, sc, orow, ocol, line)
        if not valid:
            invalid_seen += 1
            continue
        valid_seen += 1
        lr, lc, ur, uc = (int(v) for v in f[1:5])
        w00, w01, w10, w11 = (float(v) for v in f[5:9])
        assert abs(w00 + w01 + w10 + w11 - 1.0) <= 1e-6
        position = (lr + (w10 + w11) * ur) * 1000.0 + lc + (w01 + w11) * uc
        assert abs(position - patch[0, 0].real) <= 2e-3, (sr, sc, orow, ocol, line, patch[0, 0])
    assert valid_seen > 100 and invalid_seen > 20
