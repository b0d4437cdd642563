"""The Python ctypes mirror and include/qpeps.h agree on every struct layout.

A tiny C program compiled against the header prints sizeof/offsetof of each
field; the ctypes Structures must match byte for byte (CPU only).
"""
from __future__ import annotations

import subprocess

import pytest

from conftest import ROOT

STRUCTS = {
    "qpeps_u128": "U128",
    "qpeps_layer": "Layer",
    "qpeps_result": "Result",
    "qpeps_options": "Options",
    "qpeps_serve_config": "ServeConfig",
    "qpeps_serve_completion": "ServeCompletion",
    "qpeps_serve_stats": "ServeStats",
    "qpeps_tuning": "Tuning",
    "qpeps_explicit_result": "ExplicitResult",
}


def test_struct_layouts_match_the_header(qp, tmp_path):
    lines = ['#include <stdio.h>', '#include <stddef.h>', '#include "qpeps.h"', "int main(void) {"]
    for cname, pyname in STRUCTS.items():
        cls = getattr(qp, pyname)
        lines.append(f'printf("{cname} size %zu\\n", sizeof({cname}));')
        for field, _ in cls._fields_:
            lines.append(f'printf("{cname} {field} %zu\\n", offsetof({cname}, {field}));')
    lines += ["return 0;", "}"]
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines))
    exe = tmp_path / "layout"
    subprocess.run(["gcc", "-std=c11", "-I", str(ROOT / "include"), str(src), "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout
    want = {}
    for line in out.strip().split("\n"):
        cname, field, value = line.split()
        want[(cname, field)] = int(value)
    for cname, pyname in STRUCTS.items():
        cls = getattr(qp, pyname)
        assert want[(cname, "size")] == __import__("ctypes").sizeof(cls), cname
        for field, _ in cls._fields_:
            assert want[(cname, field)] == getattr(cls, field).offset, (cname, field)
