"""Thin torch-facing wrappers over the C-ABI search entry points.

Each wrapper takes CUDA tensors, calls the exported C function with their
device pointers on the current torch stream, and returns the (Q, k)
results as a structured pair of tensors (ids uint32-as-int32 view, float32
distances). These are the calls the parity tests and the benchmark make;
they add no computation of their own.
"""
from __future__ import annotations

import ctypes as C

import torch

from . import _lib
from ._lib import call

METRIC = {"l2": 0, "cosine": 1, "ip": 2}


def _ptr(t):
    return None if t is None else C.c_void_p(t.data_ptr())


def _stream(stream=None):
    s = stream if stream is not None else torch.cuda.current_stream()
    return C.c_void_p(s.cuda_stream)


def _metric(m):
    return METRIC[m] if isinstance(m, str) else int(m)


def split_results(res: torch.Tensor):
    """(Q, k, 2) int32 storage of GpuSearchResult -> (ids int64, distances f32)."""
    ids = res[..., 0].to(torch.int64) & 0xFFFFFFFF
    dist = res[..., 1].view(torch.float32)
    return ids, dist


def empty_results(nq: int, k: int, device="cuda") -> torch.Tensor:
    return torch.empty((nq, k, 2), dtype=torch.int32, device=device)


def flat_scan(vectors, queries, k, metric="l2", mask=None, vec_ids=None, out=None, stream=None):
    """cuda_flat_scan_batch: exact fp32 scan + top-k (k clamped to 256)."""
    n = vectors.shape[0] if vectors is not None else 0
    dim = queries.shape[1]
    nq = queries.shape[0]
    kk = min(k, 256)
    if out is None:
        out = empty_results(nq, kk, queries.device)
    call("cuda_flat_scan_batch", _ptr(vectors) if n else None, _ptr(vec_ids), n, dim, _ptr(queries), nq, k,
         _metric(metric), _ptr(mask), _ptr(out), _stream(stream))
    return out


def distance_matrix(queries, base, metric="l2", stream=None):
    out = torch.empty((queries.shape[0], base.shape[0]), dtype=torch.float32, device=queries.device)
    call("cuda_compute_distances_warp", _ptr(queries), _ptr(base), queries.shape[0], base.shape[0],
         queries.shape[1], _metric(metric), _ptr(out), _stream(stream))
    return out


def bitonic_sort(keys, vals, stream=None):
    ko = torch.empty_like(keys)
    vo = torch.empty_like(vals)
    call("cuda_bitonic_sort_test", _ptr(keys), _ptr(vals), _ptr(ko), _ptr(vo), keys.shape[0], _stream(stream))
    return ko, vo


def device_status() -> int:
    v = C.c_uint32(0)
    call("fv_read_device_status", C.byref(v))
    return v.value


def launch_count() -> int:
    return int(_lib.lib().fv_launch_count())


# ----------------------------------------------------------- reduced precision
def padded_dim(dim: int, multiple: int = 16) -> int:
    return (dim + multiple - 1) // multiple * multiple


def encode_fp16(vectors, pd=None, stream=None):
    """fv_encode_fp16_padded: fp16 rows (reference rounding) + ||x||^2."""
    n, dim = vectors.shape
    pd = pd or padded_dim(dim)
    out = torch.empty((n, pd), dtype=torch.int16, device=vectors.device)
    norms = torch.empty((n,), dtype=torch.float32, device=vectors.device)
    call("fv_encode_fp16_padded", _ptr(vectors), n, dim, pd, _ptr(out), _ptr(norms), _stream(stream))
    return out, norms


def fp8_padded_dim(dim: int) -> int:
    """Row length of an fp8 table: dim codes + three norm digits, to 16."""
    return padded_dim(dim + 3)


def encode_fp8(vectors, pd=None, stream=None):
    """fv_encode_fp8: e4m3 rows at the table's power-of-two scale, three
    norm digits, the scale (per row, all equal) and compensated ||x||^2."""
    n, dim = vectors.shape
    pd = pd or fp8_padded_dim(dim)
    out = torch.empty((n, pd), dtype=torch.uint8, device=vectors.device)
    scales = torch.empty((n,), dtype=torch.float32, device=vectors.device)
    norms = torch.empty((n,), dtype=torch.float32, device=vectors.device)
    call("fv_encode_fp8", _ptr(vectors), n, dim, pd, _ptr(out), _ptr(scales), _ptr(norms), _stream(stream))
    return out, scales, norms


class Fp16Table:
    """Device-resident fp16 flat table (+ optional fp32 copy for rescoring)."""

    def __init__(self, vectors, keep_fp32=True, stream=None):
        self.n, self.dim = vectors.shape
        self.pd = padded_dim(self.dim)
        self.fp16, self.norms = encode_fp16(vectors, self.pd, stream)
        self.fp32 = vectors if keep_fp32 else None
        self.struct = _lib.Fp16GpuTables(self.fp16.data_ptr(), self.norms.data_ptr(),
                                         self.fp32.data_ptr() if self.fp32 is not None else None,
                                         self.n, self.dim, self.pd)


def encode_fp8_per_vector(vectors, pd=None, stream=None):
    """fv_encode_fp8_per_vector: e4m3 rows with per-vector scales max|x|/448
    (the scale_mode 1 layout) + compensated ||x||^2."""
    n, dim = vectors.shape
    pd = pd or padded_dim(dim)
    out = torch.empty((n, pd), dtype=torch.uint8, device=vectors.device)
    scales = torch.empty((n,), dtype=torch.float32, device=vectors.device)
    norms = torch.empty((n,), dtype=torch.float32, device=vectors.device)
    call("fv_encode_fp8_per_vector", _ptr(vectors), n, dim, pd, _ptr(out), _ptr(scales), _ptr(norms),
         _stream(stream))
    return out, scales, norms


class Fp8Table:
    """Device-resident fp8 flat table (+ optional fp32 copy for rescoring).
    per_vector=False: one power-of-two table scale with norm digits (scale
    mode 0); True: per-vector scales max|x|/448 (scale mode 1)."""

    def __init__(self, vectors, keep_fp32=True, stream=None, per_vector=False):
        self.n, self.dim = vectors.shape
        self.per_vector = per_vector
        if per_vector:
            self.pd = padded_dim(self.dim)
            self.fp8, self.scales, self.norms = encode_fp8_per_vector(vectors, self.pd, stream)
        else:
            self.pd = fp8_padded_dim(self.dim)
            self.fp8, self.scales, self.norms = encode_fp8(vectors, self.pd, stream)
        self.fp32 = vectors if keep_fp32 else None
        self.struct = _lib.FvFp8GpuTables(self.fp8.data_ptr(), self.scales.data_ptr(), self.norms.data_ptr(),
                                          self.fp32.data_ptr() if self.fp32 is not None else None,
                                          self.n, self.dim, self.pd, 1 if per_vector else 0)


def options(overfetch=0, boundary_fp64=1, boundary_eps=0.0, splits=0):
    return _lib.FvScanOptions(overfetch, boundary_fp64, boundary_eps, splits)


def fp16_search(table, queries, k, metric="ip", mask=None, opts=None, out=None, stream=None, dropin=False):
    nq = queries.shape[0]
    if out is None:
        out = empty_results(nq, min(k, 256), queries.device)
    if dropin:
        call("cuda_fp16_tc_search_batch", C.byref(table.struct), _ptr(queries), nq, k, _metric(metric), _ptr(mask),
             _ptr(out), _stream(stream))
    else:
        o = opts if opts is not None else options()
        call("fv_fp16_search_batch_ex", C.byref(table.struct), _ptr(queries), nq, k, _metric(metric), _ptr(mask),
             C.byref(o), _ptr(out), _stream(stream))
    return out


def fp8_search(table, queries, k, metric="l2", mask=None, opts=None, out=None, stream=None):
    nq = queries.shape[0]
    if out is None:
        out = empty_results(nq, min(k, 256), queries.device)
    o = opts if opts is not None else options()
    call("fv_fp8_search_batch", C.byref(table.struct), _ptr(queries), nq, k, _metric(metric), _ptr(mask),
         C.byref(o), _ptr(out), _stream(stream))
    return out


def tune_set(key: str, value: int) -> None:
    """Process-wide tuning knob (fv_tune_set): tc.prepass, tc.prepass_stride, tc.prepass_margin."""
    call("fv_tune_set", key.encode(), int(value))


def tune_get(key: str) -> int:
    v = C.c_int64(0)
    call("fv_tune_get", key.encode(), C.byref(v))
    return v.value


def tune_lookup(precision: str, metric: str, dim: int, n: int, nq: int, k: int):
    """The committed autotuner knobs the library applies to this shape, or None."""
    out = (C.c_int32 * 4)()
    code = _lib.lib().fv_tune_lookup(1 if precision == "fp8" else 0, _metric(metric), dim, n, nq, k, out)
    if code != 0:
        return None
    return {"pair": out[0], "prepass": out[1], "stride": out[2], "overfetch": out[3]}


def tune_lookup_ivf(mode: str, dim: int, n: int, nlist: int, nq: int, nprobe: int):
    """The committed IVF autotuner knobs the library applies to this shape, or None."""
    out = (C.c_int32 * 3)()
    code = _lib.lib().fv_tune_lookup_ivf({"pq": 0, "sq8": 1, "rabitq": 2}[mode], dim, n, nlist, nq, nprobe, out)
    if code != 0:
        return None
    return {"pipeline": out[0], "split": out[1], "tc_coarse": out[2]}


class tuned:
    """Context manager that sets knobs and restores them on exit."""

    def __init__(self, **knobs):
        self.knobs = {k.replace("_", ".", 1): v for k, v in knobs.items()}
        self.saved = {}

    def __enter__(self):
        for k, v in self.knobs.items():
            self.saved[k] = tune_get(k)
            tune_set(k, v)
        return self

    def __exit__(self, *exc):
        for k, v in self.saved.items():
            tune_set(k, v)


def profile_enable(on: bool = True) -> None:
    call("fv_profile_enable", 1 if on else 0)


def profile_summary() -> dict:
    """Per-kernel {name: {"launches": n, "ms": total}} since the last call."""
    import json

    buf = C.create_string_buffer(1 << 16)
    call("fv_profile_summary", buf, len(buf))
    return json.loads(buf.value.decode())


class Graph:
    """A captured sequence of library calls on one stream (fv_graph_*).

        g = Graph.capture(lambda: ivf.search(q_buf, 10, 32, 400, out=out_buf), stream)
        g.launch(stream)   # replays the same calls on the same buffers
    """

    def __init__(self, handle):
        self._h = handle

    @classmethod
    def capture(cls, fn, stream):
        s = C.c_void_p(stream.cuda_stream)
        call("fv_graph_begin", s)
        try:
            with torch.cuda.stream(stream):
                fn()
        except Exception:
            h = C.c_void_p()
            _lib.lib().fv_graph_end(s, C.byref(h))
            if h.value:
                _lib.lib().fv_graph_destroy(h)
            raise
        h = C.c_void_p()
        call("fv_graph_end", s, C.byref(h))
        return cls(h)

    def launch(self, stream):
        call("fv_graph_launch", self._h, C.c_void_p(stream.cuda_stream))

    @property
    def kernels(self) -> int:
        return int(_lib.lib().fv_graph_kernel_count(self._h))

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and h.value:
            _lib.lib().fv_graph_destroy(h)
            self._h = None
