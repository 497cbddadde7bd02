"""The ctypes mirrors in fpm_rs/_native.py and oracle/oracle.py against the
C struct layouts (include/fpm_gpu.h, oracle/fpm_oracle.h): a C program
generated from the ctypes field lists prints sizeof and every field's
offsetof, compiled with the host C compiler."""

from __future__ import annotations

import ctypes as C
import os
import shutil
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, os.path.join(ROOT, "fpm-rs_gb300"))

C_NAMES = {
    "Optics": "fpm_optics", "ModelDesc": "fpm_model_desc", "MeasurementDesc": "fpm_measurement_desc",
    "AlgorithmParams": "fpm_algorithm_params", "CameraDesc": "fpm_camera_desc", "StateDesc": "fpm_state_desc",
    "SpectralModelDesc": "fpm_spectral_model_desc", "SpectralParams": "fpm_spectral_params",
    "SpectralResultDesc": "fpm_spectral_result_desc", "ResultDesc": "fpm_result_desc", "RunStats": "fpm_run_stats",
    "ServerConfig": "fpm_server_config", "RequestInfo": "fpm_request_info", "ServerStats": "fpm_server_stats",
}


ORACLE_NAMES = {
    "_Optics": "orc_optics", "_Compiled": "orc_compiled", "_Problem": "orc_problem", "_Params": "orc_params",
    "_Output": "orc_output", "_SpectralProblem": "orc_spectral_problem", "_SpectralParams": "orc_spectral_params",
}


def _check_layout(tmp_path, module, names, header, include):
    gcc = shutil.which("gcc")
    if gcc is None:
        pytest.skip("gcc is unavailable")
    lines = ['#include <stddef.h>', '#include <stdio.h>', f'#include "{header}"', "int main(void) {"]
    expected = []
    for py_name, c_name in names.items():
        cls = getattr(module, py_name)
        lines.append(f'    printf("{py_name} %zu\\n", sizeof({c_name}));')
        expected.append(f"{py_name} {C.sizeof(cls)}")
        for field, _ in cls._fields_:
            lines.append(f'    printf("{py_name}.{field} %zu\\n", offsetof({c_name}, {field}));')
            expected.append(f"{py_name}.{field} {getattr(cls, field).offset}")
    lines += ["    return 0;", "}"]
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines) + "\n")
    exe = tmp_path / "layout"
    subprocess.run([gcc, "-std=gnu11", "-I", include, str(src), "-o", str(exe)], check=True)
    got = subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.split("\n")
    assert [g for g in got if g] == expected


def test_ctypes_structs_match_the_c_header(tmp_path):
    from fpm_rs import _native as N

    _check_layout(tmp_path, N, C_NAMES, "fpm_gpu.h", os.path.join(ROOT, "include"))


def test_oracle_ctypes_structs_match_the_oracle_header(tmp_path):
    import oracle

    _check_layout(tmp_path, oracle, ORACLE_NAMES, "fpm_oracle.h", os.path.join(ROOT, "oracle"))
