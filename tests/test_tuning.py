"""The committed autotuner table (flashvector-gpu_gb300/tuning/gb300.json,
compiled into libfvgb300 by build.py) against the benchmark configurations:
every configuration's shape is covered by an entry measured at exactly that
shape (not stretched from a neighbouring one), and the library's lookup
returns that entry's knobs. CPU only: the lookups are host functions."""
from __future__ import annotations

import ctypes as C
import json

import pytest

from conftest import ROOT

TUNING = ROOT / "flashvector-gpu_gb300" / "tuning" / "gb300.json"

# (precision, metric, dim, N, queries, k): the fp16 inner-product scan at
# 1 / 64 / 1,024 queries and k 10 / 100, the fp8 L2 scan at 10M x 96
TC_SHAPES = [("fp16", "ip", 768, 1_000_000, nq, k) for nq in (1, 64, 1024) for k in (10, 100)] + \
            [("fp8", "l2", 96, 10_000_000, 10_000, 100)]
# (mode, dim, N, nlist, queries, nprobe): IVF-PQ / IVF-RaBitQ over 10M rows in
# 16,384 lists at nprobe 8 / 32 / 128, the serving configuration's IVF-SQ8
IVF_SHAPES = [(m, 128, 10_000_000, 16384, 10_000, npb) for m in ("pq", "rabitq") for npb in (8, 32, 128)] + \
             [("sq8", 768, 1_000_000, 4096, 1024, npb) for npb in (16, 64)]


def _covers(e, **v):
    return all(e[key][0] <= val <= e[key][1] for key, val in v.items())


def _first(entries, pred):
    return next((e for e in entries if pred(e)), None)


@pytest.fixture(scope="module")
def table():
    return json.loads(TUNING.read_text())


@pytest.mark.parametrize("shape", TC_SHAPES, ids=lambda s: "_".join(map(str, s)))
def test_tensor_core_shape_has_its_measured_entry(built_lib, table, shape):
    from fvgb300 import _lib

    precision, metric, dim, n, nq, k = shape
    e = _first(table["entries"], lambda e: e["precision"] == precision and e["metric"] == metric and
               _covers(e, dim=dim, n=n, nq=nq, k=k))
    assert e is not None, shape
    assert (e["shape"]["dim"], e["shape"]["n"], e["shape"]["nq"], e["shape"]["k"]) == (dim, n, nq, k)
    out = (C.c_int32 * 4)()
    assert _lib.lib().fv_tune_lookup(1 if precision == "fp8" else 0, {"l2": 0, "ip": 2}[metric], dim, n, nq, k,
                                     out) == 0
    kn = e["knobs"]
    assert list(out) == [kn["pair"], kn["prepass"], kn["stride"], kn["overfetch"]]


@pytest.mark.parametrize("shape", IVF_SHAPES, ids=lambda s: "_".join(map(str, s)))
def test_ivf_shape_has_its_measured_entry(built_lib, table, shape):
    from fvgb300 import _lib

    mode, dim, n, nlist, nq, nprobe = shape
    e = _first(table.get("ivf_entries", []), lambda e: e["mode"] == mode and
               _covers(e, dim=dim, n=n, nlist=nlist, nq=nq, nprobe=nprobe))
    assert e is not None, shape
    s = e["shape"]
    assert (s["dim"], s["n"], s["nlist"], s["nq"], s["nprobe"]) == (dim, n, nlist, nq, nprobe)
    assert e["measured"]["all_answers_equal"]
    out = (C.c_int32 * 3)()
    assert _lib.lib().fv_tune_lookup_ivf({"pq": 0, "sq8": 1, "rabitq": 2}[mode], dim, n, nlist, nq, nprobe,
                                         out) == 0
    kn = e["knobs"]
    assert list(out) == [kn["pipeline"], kn["split"], kn["tc_coarse"]]
