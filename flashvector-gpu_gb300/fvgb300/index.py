"""GpuVectorIndex: the reference engine's search/add interface for the scan
path (crates/engine/src/index.rs), backed by the native engine in
libfvgb300.so (fv_index_* in include/fv_bridge.h).

Method names and argument meanings follow the reference: build,
add_vectors, delete_ids, batch_search_fp16_tc, batch_search_ivf_mode,
batch_search_ivf_device_ptr, plus batch_search_flat (the exact fp32 scan the
reference runs for its live-insert buffer) and batch_search_fp8. Results
come back as (ids, distances) arrays of shape (num_queries, top_k); filter
masks are packed u32 words over logical ids (or a bool array, packed as the
reference's Python binding does, py_index.rs:73-81).
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import numpy as np

from . import _lib
from ._lib import call
from .datasets import pack_bools

METRIC = {"l2": 0, "cosine": 1, "ip": 2, "inner_product": 2}
ENGINE = {"flat": 0, "fp16": 1, "fp8": 2, "pq": 3, "sq8": 4, "rabitq": 5}
BUILD_FP16, BUILD_FP8, BUILD_IVF_PQ, BUILD_IVF_SQ8, BUILD_IVF_RABITQ = 1, 2, 4, 8, 16


@dataclass
class IndexConfig:
    """IndexConfig of types.h:74-82 for the scan engines."""
    dim: int
    nlist: int = 256
    m_pq: int = 16
    metric: int | str = 0
    build_flags: int = BUILD_FP16 | BUILD_IVF_PQ | BUILD_IVF_SQ8 | BUILD_IVF_RABITQ
    kmeans_iters: int = 10
    pq_iters: int = 10
    train_rows: int = 0
    streams: int = 4
    kmeans_iters_given: int = 0
    seed: int = 0
    max_elements: int = 0  # accepted for signature compatibility; capacity grows on demand

    def to_c(self):
        m = METRIC[self.metric] if isinstance(self.metric, str) else int(self.metric)
        return _lib.FvIndexConfig(self.dim, m, self.nlist, self.m_pq, self.build_flags, self.kmeans_iters,
                                  self.pq_iters, self.train_rows, self.streams, self.kmeans_iters_given, self.seed)


def _f32(a):
    return np.ascontiguousarray(np.asarray(a, dtype=np.float32))


def _mask_words(mask):
    if mask is None:
        return None, 0
    m = np.asarray(mask)
    if m.dtype == bool:
        m = pack_bools(m)
    m = np.ascontiguousarray(m, dtype=np.uint32)
    return m, m.shape[0]


class GpuVectorIndex:
    def __init__(self, config: IndexConfig):
        self.config = config
        self._h = C.c_void_p()
        call("fv_index_create", C.byref(config.to_c()), C.byref(self._h))

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and h.value:
            _lib.lib().fv_index_destroy(h)
            self._h = None

    # ------------------------------------------------------------- build
    def build(self, dataset):
        x = _f32(dataset).reshape(-1, self.config.dim)
        if x.shape[0] == 0:
            raise ValueError("Dataset cannot be empty")
        call("fv_index_build", self._h, x.ctypes.data_as(C.c_void_p), x.shape[0])

    def build_device(self, d_vectors, d_init_centroids=None):
        """Build from a CUDA tensor of rows; optional CUDA tensor of initial
        coarse centroids (nlist rows)."""
        n = d_vectors.shape[0]
        call("fv_index_build_device", self._h, C.c_void_p(d_vectors.data_ptr()), n,
             None if d_init_centroids is None else C.c_void_p(d_init_centroids.data_ptr()))

    def add_vectors(self, vectors) -> np.ndarray:
        x = _f32(vectors).reshape(-1, self.config.dim)
        ids = np.zeros(x.shape[0], dtype=np.uint32)
        if x.shape[0]:
            call("fv_index_add", self._h, x.ctypes.data_as(C.c_void_p), x.shape[0], ids.ctypes.data_as(C.c_void_p))
        return ids

    def delete_ids(self, ids) -> int:
        a = np.ascontiguousarray(np.asarray(ids, dtype=np.uint32).reshape(-1))
        out = C.c_uint32(0)
        call("fv_index_delete", self._h, a.ctypes.data_as(C.c_void_p), a.shape[0], C.byref(out))
        return out.value

    # ------------------------------------------------------------ search
    def _search(self, engine, queries, num_queries, top_k, nprobe=0, rerank_k=0, filter_mask=None, scan=None):
        q = _f32(queries).reshape(-1, self.config.dim)[:num_queries]
        out = np.zeros((num_queries, top_k, 2), dtype=np.uint32)
        words, nwords = _mask_words(filter_mask)
        params = _lib.FvSearchParams(ENGINE[engine], top_k, nprobe, rerank_k,
                                     scan if scan is not None else _lib.FvScanOptions(0, 1, 0.0, 0))
        call("fv_index_search", self._h, C.byref(params), q.ctypes.data_as(C.c_void_p), num_queries,
             None if words is None else words.ctypes.data_as(C.c_void_p), nwords, out.ctypes.data_as(C.c_void_p))
        return out[..., 0].copy(), out[..., 1].view(np.float32).copy()

    def batch_search_flat(self, queries, num_queries, top_k, filter_mask=None):
        return self._search("flat", queries, num_queries, top_k, filter_mask=filter_mask)

    def batch_search_fp16_tc(self, queries, num_queries, top_k, filter_mask=None, scan=None):
        return self._search("fp16", queries, num_queries, top_k, filter_mask=filter_mask, scan=scan)

    def batch_search_fp8(self, queries, num_queries, top_k, filter_mask=None, scan=None):
        return self._search("fp8", queries, num_queries, top_k, filter_mask=filter_mask, scan=scan)

    def batch_search_ivf_mode(self, queries, num_queries, top_k, nprobe, rerank_k, mode="pq", filter_mask=None):
        """mode: "pq", "sq8" or "rabitq" (IvfQuantMode, index.rs:41-45)."""
        return self._search(mode, queries, num_queries, top_k, nprobe, rerank_k, filter_mask)

    def batch_search_ivf(self, queries, num_queries, top_k, nprobe, rerank_k):
        return self.batch_search_ivf_mode(queries, num_queries, top_k, nprobe, rerank_k, "pq")

    def batch_search_ivf_device_ptr(self, d_queries, num_queries, top_k, nprobe, rerank_k, mode="pq"):
        """d_queries: a CUDA tensor (or raw device pointer) of fp32 queries."""
        ptr = d_queries if isinstance(d_queries, int) else d_queries.data_ptr()
        out = np.zeros((num_queries, top_k, 2), dtype=np.uint32)
        params = _lib.FvSearchParams(ENGINE[mode], top_k, nprobe, rerank_k, _lib.FvScanOptions(0, 1, 0.0, 0))
        call("fv_index_search_device", self._h, C.byref(params), C.c_void_p(ptr), num_queries,
             out.ctypes.data_as(C.c_void_p))
        return out[..., 0].copy(), out[..., 1].view(np.float32).copy()

    # --------------------------------------------------------- snapshots
    def save_snapshot(self, path) -> None:
        """GpuVectorIndex::save_snapshot (index.rs:845-1031): a FLSHVEC1 file."""
        code = _lib.lib().fv_index_save_snapshot(self._h, str(path).encode())
        if code != 0:
            raise _lib.FvError(f"fv_index_save_snapshot ({_lib.lib().fv_snapshot_error().decode()})", code)

    @classmethod
    def load_snapshot(cls, path, config: IndexConfig | None = None) -> "GpuVectorIndex":
        """GpuVectorIndex::load_snapshot (index.rs:1033-1260). The file sets dim,
        metric, nlist and m_pq; `config` may add build flags (FP8) and streams."""
        h = C.c_void_p()
        c = config.to_c() if config is not None else None
        code = _lib.lib().fv_index_load_snapshot(str(path).encode(), None if c is None else C.byref(c), C.byref(h))
        if code != 0:
            raise _lib.FvError(f"fv_index_load_snapshot ({_lib.lib().fv_snapshot_error().decode()})", code)
        obj = cls.__new__(cls)
        obj._h = h
        inf = obj.info()
        obj.config = IndexConfig(dim=inf["dim"], nlist=inf["nlist"], m_pq=inf["m_pq"], metric=inf["metric"],
                                 build_flags=config.build_flags if config else
                                 BUILD_FP16 | BUILD_IVF_PQ | BUILD_IVF_SQ8 | BUILD_IVF_RABITQ)
        return obj

    # ------------------------------------------------------------ status
    def metrics(self) -> dict:
        s = _lib.FvLatencyStats()
        call("fv_index_stats", self._h, C.byref(s))
        return {f: getattr(s, f) for f, _ in s._fields_}

    def info(self) -> dict:
        i = _lib.FvIndexInfo()
        call("fv_index_info", self._h, C.byref(i))
        return {f: getattr(i, f) for f, _ in i._fields_}

    def num_vectors(self) -> int:
        return self.info()["num_vectors"]

    def delta_len(self) -> int:
        return self.info()["delta_len"]

    def tombstone_count(self) -> int:
        return self.info()["tombstones"]

    def ivf_tables(self):
        """(IvfPqGpuTables, IvfSqGpuTables, FvIvfOptions) device views."""
        pq, sq, opt = _lib.IvfPqGpuTables(), _lib.IvfSqGpuTables(), _lib.FvIvfOptions()
        call("fv_index_ivf_tables", self._h, C.byref(pq), C.byref(sq), C.byref(opt))
        return pq, sq, opt

    def rabitq_tables(self):
        """(IvfRabitqGpuTables, FvIvfOptions) device views (list-major)."""
        t, opt = _lib.IvfRabitqGpuTables(), _lib.FvIvfOptions()
        call("fv_index_rabitq_tables", self._h, C.byref(t), C.byref(opt))
        return t, opt

    def export_ivf(self) -> dict:
        """The built IVF tables as host arrays (for checking the build)."""
        inf = self.info()
        n, dim, nlist, m = inf["num_vectors"], inf["dim"], inf["nlist"], inf["m_pq"]
        spec = {"centroids": (0, (nlist, dim), np.float32), "offsets": (6, (nlist + 1,), np.uint32),
                "vec_ids": (7, (n,), np.uint32), "sq_mins": (3, (dim,), np.float32),
                "sq_scales": (4, (dim,), np.float32), "sq_codes": (5, (n, dim), np.uint8)}
        if m and self.config.build_flags & BUILD_IVF_PQ:
            spec["codebooks"] = (1, (m, 256, dim // m), np.float32)
            spec["pq_codes"] = (2, (n, m), np.uint8)
        if self.config.build_flags & BUILD_IVF_RABITQ:
            P = _lib.lib().fv_rabitq_padded_dim(dim)
            spec["rot_signs"] = (8, (3 * P,), np.float32)
            spec["rot_centroids"] = (9, (nlist, P), np.float32)
            spec["rabitq_bits"] = (10, (n, P // 32), np.uint32)
            spec["rabitq_meta"] = (11, (n, 4), np.float32)
        out = {"nlist": nlist}
        if "rot_signs" in spec:
            out["padded_dim"] = spec["rot_centroids"][1][1]
        for key, (table, shape, dt) in spec.items():
            a = np.zeros(shape, dtype=dt)
            call("fv_index_export_ivf", self._h, table, a.ctypes.data_as(C.c_void_p), a.nbytes)
            out[key] = a
        return out


def snapshot_manifest(path) -> dict:
    """The manifest of a FLSHVEC1 snapshot (no GPU needed)."""
    import json

    need = C.c_size_t(0)
    code = _lib.lib().fv_snapshot_inspect(str(path).encode(), None, 0, C.byref(need))
    if code != 0:
        raise _lib.FvError(f"fv_snapshot_inspect ({_lib.lib().fv_snapshot_error().decode()})", code)
    buf = C.create_string_buffer(need.value)
    call("fv_snapshot_inspect", str(path).encode(), buf, need.value, None)
    return json.loads(buf.value.decode())
