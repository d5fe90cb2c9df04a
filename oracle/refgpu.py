"""ctypes front end of the reference's own CUDA kernels (oracle/_ref/libfvref.so).

TEST INFRASTRUCTURE ONLY. The library is the reference's kernels for this
path (kernels/src/{ivf_pq_lookup,ivf_quant_lookup,sparse_hybrid}.cu) compiled
unchanged for sm_103a by `make -C oracle ref` (see oracle/Makefile). It is
used by tests/golden/make_ivf_golden.py to record the reference's outputs as
committed fixtures, and by oracle/ref_gpu_bench.py to time the reference's
kernels on the same GPU. Neither the product nor the tests' parity checks
load it: the checks read the committed fixtures.

Every wrapper takes torch CUDA tensors, passes their device pointers through
the reference's C ABI (kernels/include/cuda_bridge.h:96-162), and returns the
call's status. Callers must size the validity mask to at least ceil(N/32)
words: the reference's kernels read it without a bounds check
(kernels/src/distance_metrics.cuh:17-20).
"""
from __future__ import annotations

import ctypes as C
import subprocess
from pathlib import Path

HERE = Path(__file__).resolve().parent
LIB_PATH = HERE / "_ref" / "libfvref.so"

P = C.c_void_p
U32 = C.c_uint32
I32 = C.c_int
METRICS = {"l2": 0, "cosine": 1, "ip": 2}


class IvfPqGpuTables(C.Structure):  # kernels/include/types.h:85-97
    _fields_ = [("d_centroids", P), ("d_pq_codebooks", P), ("d_pq_codes", P), ("d_ivf_offsets", P),
                ("d_ivf_vec_ids", P), ("d_vectors", P), ("num_vectors", U32), ("dim", U32), ("nlist", U32),
                ("m_pq", U32), ("sub_dim", U32)]


class IvfSqGpuTables(C.Structure):  # kernels/include/types.h:100-111
    _fields_ = [("d_centroids", P), ("d_sq_mins", P), ("d_sq_scales", P), ("d_sq_codes", P), ("d_ivf_offsets", P),
                ("d_ivf_vec_ids", P), ("d_vectors", P), ("num_vectors", U32), ("dim", U32), ("nlist", U32)]


class IvfRabitqGpuTables(C.Structure):  # kernels/include/types.h:114-128
    _fields_ = [("d_centroids", P), ("d_rot_centroids", P), ("d_rabitq_bits", P), ("d_rabitq_meta", P),
                ("d_rot_signs", P), ("d_ivf_offsets", P), ("d_ivf_vec_ids", P), ("d_vectors", P),
                ("num_vectors", U32), ("dim", U32), ("padded_dim", U32), ("words_per_vec", U32), ("nlist", U32)]


class Fp16GpuTables(C.Structure):  # kernels/include/types.h:131-138
    _fields_ = [("d_vectors_fp16", P), ("d_vec_norms_sq", P), ("d_vectors", P), ("num_vectors", U32), ("dim", U32),
                ("padded_dim", U32)]


_lib = None


def available() -> bool:
    return LIB_PATH.exists() or (HERE / "_ref" / "kernels" / "src").is_dir()


def lib():
    """Load libfvref.so, compiling it from the staged sources if needed."""
    global _lib
    if _lib is None:
        if not LIB_PATH.exists():
            subprocess.run(["make", "-s", "ref"], cwd=HERE, check=True)
        _lib = C.CDLL(str(LIB_PATH))
        search = [P, P, U32, U32, U32, U32, I32, P, P, P]
        for name in ("cuda_ivf_pq_search_batch", "cuda_ivf_sq_search_batch", "cuda_ivf_rabitq_search_batch"):
            f = getattr(_lib, name)
            f.restype = I32
            f.argtypes = search
        _lib.cuda_fp16_tc_search_batch.restype = I32
        _lib.cuda_fp16_tc_search_batch.argtypes = [P, P, U32, U32, I32, P, P, P]
        _lib.cuda_flat_scan_batch.restype = I32
        _lib.cuda_flat_scan_batch.argtypes = [P, P, U32, U32, P, U32, U32, I32, P, P, P]
    return _lib


def _ptr(t):
    return None if t is None else C.c_void_p(t.data_ptr())


def _stream():
    import torch

    return C.c_void_p(torch.cuda.current_stream().cuda_stream)


def _check_mask(mask, n):
    if mask is not None:
        assert mask.numel() >= (n + 31) // 32, "the reference reads ceil(N/32) mask words unchecked"


class IvfTables:
    """Reference-layout IVF tables (codes indexed by vector id) as device
    tensors; `t` holds host arrays keyed as oracle.build_ivf returns them."""

    def __init__(self, mode, t, vectors):
        import numpy as np
        import torch

        def dev(a):
            a = np.ascontiguousarray(a)
            if a.dtype == np.uint32:
                a = a.view(np.int32)
            return torch.from_numpy(a).cuda()

        self.mode = mode
        self.keep = []
        self.centroids = dev(np.asarray(t["centroids"], dtype=np.float32))
        self.nlist, self.dim = self.centroids.shape
        self.offsets = dev(np.asarray(t["offsets"], dtype=np.uint32))
        self.vec_ids = dev(np.asarray(t["vec_ids"], dtype=np.uint32))
        self.vectors = None if vectors is None else dev(np.asarray(vectors, dtype=np.float32))
        self.n = int(self.vec_ids.numel())
        v = _ptr(self.vectors)
        if mode == "pq":
            cb = dev(np.asarray(t["codebooks"], dtype=np.float32))
            codes = dev(np.asarray(t["pq_codes"], dtype=np.uint8))
            self.keep = [cb, codes]
            m_pq, sub_dim = cb.shape[0], cb.shape[2]
            self.struct = IvfPqGpuTables(self.centroids.data_ptr(), cb.data_ptr(), codes.data_ptr(),
                                         self.offsets.data_ptr(), self.vec_ids.data_ptr(), v, self.n, self.dim,
                                         self.nlist, m_pq, sub_dim)
        elif mode == "sq8":
            mins = dev(np.asarray(t["sq_mins"], dtype=np.float32))
            scales = dev(np.asarray(t["sq_scales"], dtype=np.float32))
            codes = dev(np.asarray(t["sq_codes"], dtype=np.uint8))
            self.keep = [mins, scales, codes]
            self.struct = IvfSqGpuTables(self.centroids.data_ptr(), mins.data_ptr(), scales.data_ptr(),
                                         codes.data_ptr(), self.offsets.data_ptr(), self.vec_ids.data_ptr(), v,
                                         self.n, self.dim, self.nlist)
        else:
            P_ = int(t["padded_dim"])
            rot_c = dev(np.asarray(t["rot_centroids"], dtype=np.float32))
            bits = dev(np.asarray(t["rabitq_bits"], dtype=np.uint32))
            meta = dev(np.asarray(t["rabitq_meta"], dtype=np.float32))
            signs = dev(np.asarray(t["rot_signs"], dtype=np.float32))
            self.keep = [rot_c, bits, meta, signs]
            self.struct = IvfRabitqGpuTables(self.centroids.data_ptr(), rot_c.data_ptr(), bits.data_ptr(),
                                             meta.data_ptr(), signs.data_ptr(), self.offsets.data_ptr(),
                                             self.vec_ids.data_ptr(), v, self.n, self.dim, P_, P_ // 32, self.nlist)

    def search(self, queries, k, nprobe, rerank_k, metric, mask, out):
        _check_mask(mask, self.n)
        fn = {"pq": "cuda_ivf_pq_search_batch", "sq8": "cuda_ivf_sq_search_batch",
              "rabitq": "cuda_ivf_rabitq_search_batch"}[self.mode]
        return getattr(lib(), fn)(C.byref(self.struct), _ptr(queries), queries.shape[0], k, nprobe, rerank_k,
                                  METRICS[metric], _ptr(mask), _ptr(out), _stream())


def fp16_search(table_fp16, norms, n, dim, padded_dim, queries, k, metric, mask, out):
    """cuda_fp16_tc_search_batch over an fp16 table [n][padded_dim]."""
    _check_mask(mask, n)
    t = Fp16GpuTables(table_fp16.data_ptr(), norms.data_ptr(), None, n, dim, padded_dim)
    return lib().cuda_fp16_tc_search_batch(C.byref(t), _ptr(queries), queries.shape[0], k, METRICS[metric],
                                           _ptr(mask), _ptr(out), _stream())


def flat_scan(vectors, vec_ids, queries, k, metric, mask, out):
    """cuda_flat_scan_batch over fp32 rows [n][dim]."""
    n, dim = vectors.shape
    _check_mask(mask, n)
    return lib().cuda_flat_scan_batch(_ptr(vectors), _ptr(vec_ids), n, dim, _ptr(queries), queries.shape[0], k,
                                      METRICS[metric], _ptr(mask), _ptr(out), _stream())
