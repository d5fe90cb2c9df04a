"""The ctypes mirrors in fvgb300/_lib.py against the C headers.

A small C program includes include/fv_serve.h (which brings in
fv_bridge.h and fv_types.h), is compiled with the host C compiler, and
prints sizeof and offsetof of every field of every struct the Python side
mirrors; the test compares them with the ctypes layouts, so a field added
to a header without its mirror (or the reverse) fails here, without a GPU."""
from __future__ import annotations

import shutil
import subprocess
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]

STRUCTS = ["GpuSearchResult", "IvfPqGpuTables", "IvfSqGpuTables", "IvfRabitqGpuTables", "Fp16GpuTables",
           "FvFp8GpuTables", "FvIvfOptions", "FvScanOptions", "FvIndexConfig", "FvSearchParams", "FvLatencyStats",
           "FvIndexInfo", "FvServeConfig", "FvRequest", "FvServeStats"]


@pytest.fixture(scope="module")
def c_layouts(tmp_path_factory):
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no host C compiler")
    from fvgb300 import _lib

    lines = ["#include <stdio.h>", "#include <stddef.h>", '#include "fv_serve.h"', "int main(void) {"]
    for name in STRUCTS:
        lines.append(f'  printf("{name} sizeof %zu\\n", sizeof({name}));')
        for field, _ in getattr(_lib, name)._fields_:
            lines.append(f'  printf("{name} {field} %zu\\n", offsetof({name}, {field}));')
    lines += ["  return 0;", "}"]
    d = tmp_path_factory.mktemp("abi")
    src = d / "layout.c"
    src.write_text("\n".join(lines) + "\n")
    # the header as C11 and as C++17 (the library's own translation units)
    builds = [(cc, ["-std=c11"])]
    cxx = shutil.which("g++") or shutil.which("c++")
    if cxx:
        builds.append((cxx, ["-x", "c++", "-std=c++17"]))
    layouts = {}
    for i, (comp, flags) in enumerate(builds):
        exe = d / f"layout{i}"
        r = subprocess.run([comp, *flags, "-I", str(ROOT / "include"), str(src), "-o", str(exe)],
                           capture_output=True, text=True)
        assert r.returncode == 0, f"{comp} {' '.join(flags)}: {r.stderr}"
        out = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout
        for line in out.splitlines():
            struct, field, value = line.split()
            prev = layouts.setdefault(struct, {}).setdefault(field, int(value))
            assert prev == int(value), (struct, field, "C and C++ layouts differ")
    return layouts


@pytest.mark.parametrize("name", STRUCTS)
def test_ctypes_mirror_matches_the_header(c_layouts, name):
    from fvgb300 import _lib

    cls = getattr(_lib, name)
    got = c_layouts[name]
    assert got["sizeof"] == __import__("ctypes").sizeof(cls), name
    for field, _ in cls._fields_:
        assert got[field] == getattr(cls, field).offset, (name, field)
