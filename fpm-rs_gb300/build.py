"""Builds libfpm_gpu.so (the C-ABI device backend) in-tree for sm_103a.

Usage: python fpm-rs_gb300/build.py [--force]

Translation units compile in parallel with nvcc and link into one shared
library next to this file. The CUDA runtime is linked statically so the
library loads without a matching libcudart on the library path.
"""

from __future__ import annotations

import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libfpm_gpu.so")
SOURCES = ["engine_n256.cu", "engine_n256_gd.cu", "engine_n128.cu", "engine_n128_gd.cu", "engine_n64.cu",
           "engine_n64_gd.cu", "engine_n32.cu", "engine_n32_gd.cu", "engine.cu", "engine_l2.cu", "grid.cu", "camera.cu", "noalloc.cu", "runtime.cpp", "server.cpp"]
HEADERS = ["fpm_common.cuh", "kernels.h", "twiddle256.cuh", "engine_impl.cuh"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
# Host code is compiled without floating-point contraction: GCC would otherwise
# fuse a * b + c into one rounding wherever the target has FMA (always on
# aarch64), and the model compilation (pose rotation, k-vectors, crop offsets)
# must round as the reference does, on every host architecture.
FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off",
         "--expt-relaxed-constexpr", "-I", os.path.join(ROOT, "include"), "-I", CSRC]


def nvcc() -> str:
    for candidate in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", "nvcc"):
        if candidate and (os.path.isabs(candidate) and os.path.exists(candidate) or not os.path.isabs(candidate)):
            return candidate
    return "nvcc"


def _stale(target: str, deps: list[str]) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def build(force: bool = False, verbose: bool = False) -> str:
    os.makedirs(BUILD, exist_ok=True)
    headers = [os.path.join(CSRC, h) for h in HEADERS] + [os.path.join(ROOT, "include", "fpm_gpu.h")]
    jobs = []
    objects = []
    for src in SOURCES:
        path = os.path.join(CSRC, src)
        obj = os.path.join(BUILD, src + ".o")
        objects.append(obj)
        if force or _stale(obj, [path] + headers):
            cmd = [nvcc(), *ARCH, *FLAGS, "-c", path, "-o", obj]
            if verbose:
                cmd.insert(1, "-Xptxas=-v")
            jobs.append((cmd, subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT)))
    failed = []
    for cmd, proc in jobs:
        out, _ = proc.communicate()
        text = out.decode(errors="replace")
        if proc.returncode != 0:
            failed.append(" ".join(cmd) + "\n" + text)
        elif verbose and text.strip():
            print(text)
    if failed:
        raise RuntimeError("nvcc failed:\n" + "\n".join(failed))
    if force or jobs or _stale(LIB, objects):
        cmd = [nvcc(), *ARCH, "-shared", "-cudart", "static", "-o", LIB, *objects]
        subprocess.run(cmd, check=True)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
