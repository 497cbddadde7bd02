"""The Rust #[repr(C)] mirrors shown in INTEGRATION.md list the same fields,
in the same order, as the C structs of include/fpm_gpu.h."""

from __future__ import annotations

import os
import re

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _c_structs(text):
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    out = {}
    for body, name in re.findall(r"typedef struct\s*\{(.*?)\}\s*(fpm_\w+)\s*;", text, flags=re.S):
        fields = []
        for decl in body.split(";"):
            decl = " ".join(decl.split())
            if not decl:
                continue
            # "const double *kx, *ky" -> type "const double", declarators "*kx", "*ky"
            first, *rest = [d.strip() for d in decl.split(",")]
            names = [first.split()[-1]] + rest
            fields += [re.sub(r"[\*\s]|\[.*\]", "", n) for n in names]
        out[name] = fields
    return out


def _rust_structs(text):
    out = {}
    for name, body in re.findall(r"#\[repr\(C\)\] pub struct (Fpm\w+) \{(.*?)\}", text, flags=re.S):
        out[name] = re.findall(r"pub (\w+):", body)
    return out


def _snake(name):
    return "fpm" + re.sub(r"([A-Z])", lambda m: "_" + m.group(1).lower(), name[3:])


def test_rust_mirrors_match_the_c_header():
    with open(os.path.join(ROOT, "include", "fpm_gpu.h")) as f:
        c = _c_structs(f.read())
    with open(os.path.join(ROOT, "INTEGRATION.md")) as f:
        rust = _rust_structs(f.read())
    assert len(rust) >= 10
    for name, fields in rust.items():
        if not fields:
            continue  # opaque handles (FpmJob)
        c_name = _snake(name)
        assert c_name in c, name
        assert fields == c[c_name], (name, fields, c[c_name])
