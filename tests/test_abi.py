"""The C-ABI library loads and exports every function include/*.h declares
(CPU only: no compute calls)."""
from __future__ import annotations

import ctypes
import re

from conftest import ROOT

DECL = re.compile(r"^\s*(?:const\s+)?[A-Za-z_][A-Za-z0-9_]*\s*\*?\s*\b((?:cuda|fv)_[A-Za-z0-9_]+)\s*\(", re.M)


def declared_functions():
    names = set()
    for h in (ROOT / "include").glob("*.h"):
        text = re.sub(r"/\*.*?\*/", "", h.read_text(), flags=re.S)
        names.update(DECL.findall(text))
    return sorted(names)


def test_headers_declare_the_drop_in_entry_points():
    names = declared_functions()
    for required in ("cuda_flat_scan_batch", "cuda_init_device", "cuda_sync_stream"):
        assert required in names


def test_library_exports_every_declared_symbol(built_lib):
    lib = ctypes.CDLL(str(built_lib))
    missing = [n for n in declared_functions() if not hasattr(lib, n)]
    assert not missing, f"declared but not exported: {missing}"


def test_python_binding_covers_every_declared_symbol(built_lib):
    from fvgb300 import _lib

    missing = [n for n in declared_functions() if n not in _lib.SIGNATURES]
    assert not missing, f"no ctypes signature for: {missing}"
    lib = _lib.lib()
    assert lib.fv_version().startswith(b"fvgb300")


def test_struct_layouts_match_reference():
    """GpuSearchResult is 8 bytes, align 8 (types.h:39-42); table structs keep
    the reference field order (types.h:85-111, 131-138)."""
    from fvgb300 import _lib

    assert ctypes.sizeof(_lib.GpuSearchResult) == 8
    assert ctypes.alignment(_lib.GpuSearchResult) in (4, 8)
    assert ctypes.sizeof(_lib.IvfPqGpuTables) == 6 * 8 + 5 * 4 + 4  # padded to 8
    assert ctypes.sizeof(_lib.IvfSqGpuTables) == 7 * 8 + 3 * 4 + 4
    assert ctypes.sizeof(_lib.Fp16GpuTables) == 3 * 8 + 3 * 4 + 4
    assert [f[0] for f in _lib.IvfPqGpuTables._fields_][:6] == [
        "d_centroids", "d_pq_codebooks", "d_pq_codes", "d_ivf_offsets", "d_ivf_vec_ids", "d_vectors"]


def test_tune_knobs_roundtrip(built_lib):
    """fv_tune_set / fv_tune_get (host only)."""
    import pytest
    from fvgb300 import scan
    from fvgb300._lib import FvError

    assert scan.tune_get("tc.prepass") == -1
    assert scan.tune_get("tc.table") == 1
    with scan.tuned(tc_prepass_stride=16):
        assert scan.tune_get("tc.prepass_stride") == 16
    assert scan.tune_get("tc.prepass_stride") == 0
    with pytest.raises(FvError):
        scan.tune_set("no.such.knob", 1)


def test_committed_tuning_table_is_compiled_in(built_lib):
    """Every entry of tuning/gb300.json is what the library applies to its
    own shape (the table build.py compiles in), and nothing applies to a
    shape outside every range."""
    import json

    from conftest import ROOT
    from fvgb300 import scan

    doc = json.loads((ROOT / "flashvector-gpu_gb300" / "tuning" / "gb300.json").read_text())
    assert doc["entries"]
    for e in doc["entries"]:
        sh = e["shape"]
        got = scan.tune_lookup(e["precision"], e["metric"], sh["dim"], sh["n"], sh["nq"], sh["k"])
        assert got == {k: e["knobs"][k] for k in ("pair", "prepass", "stride", "overfetch")}, e["name"]
        assert e["measured"]["recall_at_10"] >= e["measured"]["recall_target"]
    assert scan.tune_lookup("fp16", "cosine", 7, 100, 3, 5) is None
    with scan.tuned(tc_table=0):
        sh = doc["entries"][0]["shape"]
        assert scan.tune_lookup(doc["entries"][0]["precision"], doc["entries"][0]["metric"], sh["dim"], sh["n"],
                                sh["nq"], sh["k"]) is None
