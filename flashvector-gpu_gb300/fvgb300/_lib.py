"""ctypes binding of libfvgb300.so (the C ABI declared in include/fv_bridge.h).

The library is loaded from this package directory (built in-tree by
flashvector-gpu_gb300/build.py). There is no fallback: if the shared library
is missing or fails to load, every entry point raises.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

LIB_PATH = Path(__file__).resolve().parent / "libfvgb300.so"

P = C.c_void_p
U32 = C.c_uint32
I32 = C.c_int
SZ = C.c_size_t
F32 = C.c_float


class GpuSearchResult(C.Structure):
    _fields_ = [("id", C.c_uint32), ("distance", C.c_float)]
    _pack_ = 8


class IvfPqGpuTables(C.Structure):
    _fields_ = [("d_centroids", P), ("d_pq_codebooks", P), ("d_pq_codes", P), ("d_ivf_offsets", P),
                ("d_ivf_vec_ids", P), ("d_vectors", P), ("num_vectors", U32), ("dim", U32), ("nlist", U32),
                ("m_pq", U32), ("sub_dim", U32)]


class IvfSqGpuTables(C.Structure):
    _fields_ = [("d_centroids", P), ("d_sq_mins", P), ("d_sq_scales", P), ("d_sq_codes", P), ("d_ivf_offsets", P),
                ("d_ivf_vec_ids", P), ("d_vectors", P), ("num_vectors", U32), ("dim", U32), ("nlist", U32)]


class IvfRabitqGpuTables(C.Structure):
    _fields_ = [("d_centroids", P), ("d_rot_centroids", P), ("d_rabitq_bits", P), ("d_rabitq_meta", P),
                ("d_rot_signs", P), ("d_ivf_offsets", P), ("d_ivf_vec_ids", P), ("d_vectors", P),
                ("num_vectors", U32), ("dim", U32), ("padded_dim", U32), ("words_per_vec", U32), ("nlist", U32)]


class Fp16GpuTables(C.Structure):
    _fields_ = [("d_vectors_fp16", P), ("d_vec_norms_sq", P), ("d_vectors", P), ("num_vectors", U32), ("dim", U32),
                ("padded_dim", U32)]


class FvFp8GpuTables(C.Structure):
    _fields_ = [("d_vectors_fp8", P), ("d_scales", P), ("d_vec_norms_sq", P), ("d_vectors", P),
                ("num_vectors", U32), ("dim", U32), ("padded_dim", U32), ("scale_mode", U32)]


class FvIvfOptions(C.Structure):
    _fields_ = [("codes_list_major", U32), ("reserved", U32 * 3)]


class FvScanOptions(C.Structure):
    _fields_ = [("overfetch", U32), ("boundary_fp64", U32), ("boundary_eps", F32), ("splits", U32)]


class FvIndexConfig(C.Structure):
    _fields_ = [("dim", U32), ("metric", U32), ("nlist", U32), ("m_pq", U32), ("build_flags", U32),
                ("kmeans_iters", U32), ("pq_iters", U32), ("train_rows", U32), ("streams", U32),
                ("kmeans_iters_given", U32),
                ("seed", C.c_uint64)]


class FvSearchParams(C.Structure):
    _fields_ = [("engine", U32), ("top_k", U32), ("nprobe", U32), ("rerank_k", U32), ("scan", FvScanOptions)]


class FvLatencyStats(C.Structure):
    _fields_ = [("count", C.c_uint64)] + [(n, C.c_double) for n in
                                          ("p50_us", "p90_us", "p99_us", "p999_us", "min_us", "max_us", "mean_us",
                                           "qps")]


class FvIndexInfo(C.Structure):
    _fields_ = [(n, U32) for n in ("num_vectors", "delta_len", "tombstones", "dim", "padded_dim", "nlist", "m_pq",
                                   "metric", "next_id", "reserved")] + [("device_bytes", C.c_uint64)]


class FvServeConfig(C.Structure):
    _fields_ = [("max_batch", U32), ("max_wait_us", U32), ("inflight", U32), ("group_by_params", U32),
                ("queue_capacity", U32), ("scratch_budget_kb", U32), ("graphs", U32), ("reserved", U32)]


class FvRequest(C.Structure):
    _fields_ = [("engine", U32), ("top_k", U32), ("nprobe", U32), ("rerank_k", U32), ("filter_id", C.c_int32),
                ("reserved", U32)]


class FvServeStats(C.Structure):
    _fields_ = [("total_requests", C.c_uint64), ("total_batches", C.c_uint64), ("avg_batch_size", C.c_double),
                ("completed", C.c_uint64), ("failed", C.c_uint64)] + \
               [(n, C.c_double) for n in ("qps", "p50_us", "p90_us", "p99_us", "p999_us", "max_us", "mean_us",
                                          "queue_p50_us", "queue_p99_us")] + \
               [("max_inflight", U32), ("graph_instantiations", U32), ("scratch_waits", C.c_uint64),
                ("scratch_split", C.c_uint64), ("scratch_peak_bytes", C.c_uint64), ("scratch_pool_bytes", C.c_uint64),
                ("graph_fallbacks", C.c_uint64)]


# int (*)(void* user, const FvRequest*, const float* queries, uint32_t nq, uint32_t dim, uint32_t k_stride,
#         GpuSearchResult* out)
FvServeExecutor = C.CFUNCTYPE(I32, P, C.POINTER(FvRequest), C.POINTER(F32), U32, U32, U32,
                              C.POINTER(GpuSearchResult))


# name -> (restype, argtypes); every function declared in include/fv_bridge.h and include/fv_serve.h
SIGNATURES = {
    "cuda_init_device": (I32, [I32]),
    "cuda_set_device": (I32, [I32]),
    "cuda_get_device_count": (I32, [P]),
    "cuda_get_device_memory": (I32, [P, P]),
    "cuda_device_synchronize": (I32, []),
    "cuda_malloc_device": (I32, [P, SZ]),
    "cuda_free_device": (I32, [P]),
    "cuda_malloc_host": (I32, [P, SZ]),
    "cuda_free_host": (I32, [P]),
    "cuda_memcpy_h2d_async": (I32, [P, P, SZ, P]),
    "cuda_memcpy_d2h_async": (I32, [P, P, SZ, P]),
    "cuda_memset_device_async": (I32, [P, I32, SZ, P]),
    "cuda_host_get_device_pointer": (I32, [P, P]),
    "cuda_create_stream": (I32, [P]),
    "cuda_destroy_stream": (I32, [P]),
    "cuda_sync_stream": (I32, [P]),
    "cuda_flat_scan_batch": (I32, [P, P, U32, U32, P, U32, U32, I32, P, P, P]),
    "fv_flat_scan_batch_noalloc": (I32, [P, P, U32, U32, P, U32, U32, I32, P, P, P]),
    "cuda_compute_distances_warp": (I32, [P, P, U32, U32, U32, I32, P, P]),
    "cuda_bitonic_sort_test": (I32, [P, P, P, P, U32, P]),
    "cuda_ivf_pq_search_batch": (I32, [P, P, U32, U32, U32, U32, I32, P, P, P]),
    "cuda_ivf_sq_search_batch": (I32, [P, P, U32, U32, U32, U32, I32, P, P, P]),
    "fv_ivf_pq_search_ex": (I32, [P, P, P, U32, U32, U32, U32, I32, P, P, P]),
    "fv_ivf_sq_search_ex": (I32, [P, P, P, U32, U32, U32, U32, I32, P, P, P]),
    "cuda_ivf_rabitq_search_batch": (I32, [P, P, U32, U32, U32, U32, I32, P, P, P]),
    "fv_ivf_rabitq_search_ex": (I32, [P, P, P, U32, U32, U32, U32, I32, P, P, P]),
    "fv_ivf_relayout_codes": (I32, [P, P, U32, U32, P, P]),
    "fv_build_pq_encode": (I32, [P, U32, U32, U32, P, P, P]),
    "fv_build_sq8": (I32, [P, U32, U32, P, P, P, P]),
    "fv_build_ivf_lists": (I32, [P, U32, U32, P, P, P]),
    "fv_rabitq_padded_dim": (U32, [U32]),
    "fv_rabitq_rot_signs": (None, [U32, C.c_uint64, P]),
    "fv_build_rabitq": (I32, [P, U32, U32, P, U32, P, P, U32, P, P, P, P]),
    "cuda_fp16_tc_search_batch": (I32, [P, P, U32, U32, I32, P, P, P]),
    "fv_fp16_search_batch_ex": (I32, [P, P, U32, U32, I32, P, P, P, P]),
    "fv_fp8_search_batch": (I32, [P, P, U32, U32, I32, P, P, P, P]),
    "fv_encode_fp16_padded": (I32, [P, U32, U32, U32, P, P, P]),
    "fv_encode_fp8": (I32, [P, U32, U32, U32, P, P, P, P]),
    "fv_encode_fp8_per_vector": (I32, [P, U32, U32, U32, P, P, P, P]),
    "fv_index_create": (I32, [P, P]),
    "fv_index_destroy": (I32, [P]),
    "fv_index_build": (I32, [P, P, U32]),
    "fv_index_build_device": (I32, [P, P, U32, P]),
    "fv_index_add": (I32, [P, P, U32, P]),
    "fv_index_delete": (I32, [P, P, U32, P]),
    "fv_index_search": (I32, [P, P, P, U32, P, U32, P]),
    "fv_index_search_device": (I32, [P, P, P, U32, P]),
    "fv_index_stats": (I32, [P, P]),
    "fv_index_info": (I32, [P, P]),
    "fv_index_ivf_tables": (I32, [P, P, P, P]),
    "fv_index_rabitq_tables": (I32, [P, P, P]),
    "fv_index_export_ivf": (I32, [P, U32, P, SZ]),
    "fv_index_save_snapshot": (I32, [P, C.c_char_p]),
    "fv_index_load_snapshot": (I32, [C.c_char_p, P, P]),
    "fv_snapshot_inspect": (I32, [C.c_char_p, C.c_char_p, SZ, P]),
    "fv_snapshot_error": (C.c_char_p, []),
    "fv_graph_begin": (I32, [P]),
    "fv_graph_end": (I32, [P, P]),
    "fv_graph_launch": (I32, [P, P]),
    "fv_graph_kernel_count": (C.c_uint64, [P]),
    "fv_graph_destroy": (I32, [P]),
    "fv_version": (C.c_char_p, []),
    "fv_read_device_status": (I32, [P]),
    "fv_launch_count": (C.c_uint64, []),
    "fv_profile_enable": (I32, [I32]),
    "fv_profile_summary": (I32, [C.c_char_p, SZ]),
    "fv_set_stream_scratch": (I32, [P, P, SZ]),
    "fv_tune_set": (I32, [C.c_char_p, C.c_int64]),
    "fv_tune_get": (I32, [C.c_char_p, P]),
    "fv_tune_lookup": (I32, [I32, I32, U32, C.c_uint64, U32, U32, P]),
    "fv_tune_lookup_ivf": (I32, [I32, U32, C.c_uint64, U32, U32, U32, P]),
    "fv_release_stream_scratch": (I32, [P]),
    "fv_serve_create": (I32, [P, P, P]),
    "fv_serve_create_with_executor": (I32, [U32, P, FvServeExecutor, P, P]),
    "fv_serve_destroy": (I32, [P]),
    "fv_serve_add_filter": (I32, [P, P, U32, P]),
    "fv_serve_remove_filter": (I32, [P, C.c_int32]),
    "fv_serve_submit": (I32, [P, P, P, P]),
    "fv_serve_wait": (I32, [P, C.c_uint64, P, U32, U32, P]),
    "fv_serve_replay": (I32, [P, P, P, P, U32, P, U32, P]),
    "fv_serve_scratch_estimate": (I32, [P, P, U32, P]),
    "fv_serve_stats": (I32, [P, P]),
    "fv_serve_reset_stats": (I32, [P]),
}

_lib = None


def lib() -> C.CDLL:
    """The loaded library; raises if it has not been built."""
    global _lib
    if _lib is None:
        if not LIB_PATH.exists():
            raise RuntimeError(f"{LIB_PATH} is missing: build it with flashvector-gpu_gb300/build.py "
                               "(there is no CPU fallback)")
        handle = C.CDLL(str(LIB_PATH))
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(handle, name)
            fn.restype = res
            fn.argtypes = args
        _lib = handle
    return _lib


class FvError(RuntimeError):
    def __init__(self, fn: str, code: int):
        super().__init__(f"{fn} failed with code {code}")
        self.code = code


def check(fn: str, code: int) -> None:
    if code != 0:
        raise FvError(fn, code)


def call(name: str, *args) -> int:
    """Calls `name` and raises FvError on a non-zero return."""
    code = getattr(lib(), name)(*args)
    check(name, code)
    return code
