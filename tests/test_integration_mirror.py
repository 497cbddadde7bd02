"""The Rust binding include/fpm_gpu.rs mirrors include/fpm_gpu.h: every
#[repr(C)] struct lists the C struct's fields in the same order, and every
entry point the header declares has an extern "C" declaration."""

from __future__ import annotations

import os
import re

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _read(*parts):
    with open(os.path.join(ROOT, *parts)) as f:
        return f.read()


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


def _c_functions(text):
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return set(re.findall(r"^(?:int32_t|const char \*)\s*(fpm_\w+)\s*\(", text, flags=re.M))


def _rust_structs(text):
    out = {}
    for name, body in re.findall(r"#\[repr\(C\)\] pub struct (Fpm\w+) \{(.*?)\}", text, flags=re.S):
        out[name] = re.findall(r"pub (\w+):", body)
    return out


def _snake(name):
    return "fpm" + re.sub(r"([A-Z])", lambda m: "_" + m.group(1).lower(), name[3:])


def test_rust_structs_match_the_c_header():
    c = _c_structs(_read("include", "fpm_gpu.h"))
    rust = _rust_structs(_read("include", "fpm_gpu.rs"))
    assert len(rust) >= 11
    for name, fields in rust.items():
        if not fields:
            continue  # opaque handles (FpmJob)
        c_name = _snake(name)
        assert c_name in c, name
        assert fields == c[c_name], (name, fields, c[c_name])
    # Every C struct that crosses the boundary has its mirror.
    assert {_snake(n) for n in rust if rust[n]} == set(c)


def test_every_entry_point_has_a_rust_declaration():
    declared = set(re.findall(r"pub fn (fpm_\w+)\(", _read("include", "fpm_gpu.rs")))
    assert _c_functions(_read("include", "fpm_gpu.h")) == declared
