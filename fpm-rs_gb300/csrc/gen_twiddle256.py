"""Writes twiddle256.cuh: the 256 roots exp(-2*pi*i*k/256) rounded once from float64 to float32."""

import math
import os
import struct


def f32(x: float) -> float:
    return struct.unpack("f", struct.pack("f", x))[0]


def main() -> None:
    lines = [
        "// Generated by gen_twiddle256.py: w_256^k = exp(-2*pi*i*k/256) rounded to float.",
        "// Row k holds (cos(2*pi*k/256), -sin(2*pi*k/256)).",
        "#pragma once",
        "#include <cuda_runtime.h>",
        "static __constant__ float2 c_tw256[256] = {",
    ]
    for k in range(256):
        c = f32(math.cos(2 * math.pi * k / 256))
        s = f32(-math.sin(2 * math.pi * k / 256))
        lines.append(f"    {{{c!r}f, {s!r}f}},")
    lines.append("};")
    path = os.path.join(os.path.dirname(os.path.abspath(__file__)), "twiddle256.cuh")
    with open(path, "w") as handle:
        handle.write("\n".join(lines) + "\n")


if __name__ == "__main__":
    main()
