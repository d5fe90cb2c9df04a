"""Device-resident IVF-PQ / IVF-SQ8 tables and the calls that search them.

A table holds the reference's layout (IvfPqGpuTables / IvfSqGpuTables:
centroids, codebooks or SQ8 min/scale, code rows by vector id, posting-list
offsets and ids, the fp32 rows for the rerank) as torch CUDA tensors, plus an
optional list-major copy of the code rows for the contiguous-scan path.
"""
from __future__ import annotations

import ctypes as C

import numpy as np
import torch

from . import _lib
from ._lib import call
from .scan import _metric, _ptr, _stream, empty_results


def _dev(a, dtype=None, device="cuda"):
    if isinstance(a, torch.Tensor):
        return a.to(device).contiguous()
    arr = np.ascontiguousarray(a)
    if arr.dtype == np.uint32:
        arr = arr.view(np.int32)
    t = torch.from_numpy(arr)
    if dtype is not None:
        t = t.to(dtype)
    return t.to(device).contiguous()


def relayout_codes(codes_by_id, vec_ids, stream=None):
    n, row = codes_by_id.shape
    out = torch.empty_like(codes_by_id)
    call("fv_ivf_relayout_codes", _ptr(codes_by_id), _ptr(vec_ids), n, row, _ptr(out), _stream(stream))
    return out


class IvfTable:
    """mode "pq" or "sq8"; `t` is a dict of host or device arrays with the keys
    centroids, offsets, vec_ids and (pq) codebooks, pq_codes / (sq8) sq_mins,
    sq_scales, sq_codes."""

    def __init__(self, mode, t, vectors=None, list_major=False, device="cuda"):
        self.mode = mode
        self.centroids = _dev(t["centroids"], device=device)
        self.nlist, self.dim = self.centroids.shape
        self.offsets = _dev(t["offsets"], device=device)
        self.vec_ids = _dev(t["vec_ids"], device=device)
        self.vectors = None if vectors is None else _dev(vectors, device=device)
        self.n = self.vec_ids.shape[0]
        if mode == "pq":
            self.codebooks = _dev(t["codebooks"], device=device)
            self.codes = _dev(t["pq_codes"], device=device)
            self.m_pq = self.codebooks.shape[0]
            self.sub_dim = self.codebooks.shape[2]
        else:
            self.sq_mins = _dev(t["sq_mins"], device=device)
            self.sq_scales = _dev(t["sq_scales"], device=device)
            self.codes = _dev(t["sq_codes"], device=device)
        self.list_major = list_major
        self.codes_lm = relayout_codes(self.codes, self.vec_ids) if list_major else None
        self._build_structs()

    def _build_structs(self):
        vec = self.vectors.data_ptr() if self.vectors is not None else None
        codes = (self.codes_lm if self.list_major else self.codes).data_ptr()
        if self.mode == "pq":
            self.struct = _lib.IvfPqGpuTables(self.centroids.data_ptr(), self.codebooks.data_ptr(), codes,
                                              self.offsets.data_ptr(), self.vec_ids.data_ptr(), vec, self.n, self.dim,
                                              self.nlist, self.m_pq, self.sub_dim)
        else:
            self.struct = _lib.IvfSqGpuTables(self.centroids.data_ptr(), self.sq_mins.data_ptr(),
                                              self.sq_scales.data_ptr(), codes, self.offsets.data_ptr(),
                                              self.vec_ids.data_ptr(), vec, self.n, self.dim, self.nlist)
        self.options = _lib.FvIvfOptions(1 if self.list_major else 0)

    def search(self, queries, k, nprobe, rerank_k, metric="l2", mask=None, out=None, stream=None, dropin=None):
        """cuda_ivf_{pq,sq}_search_batch (reference layout) or the fv_*_ex call
        (list-major layout)."""
        nq = queries.shape[0]
        if out is None:
            out = empty_results(nq, min(k, 256), queries.device)
        dropin = (not self.list_major) if dropin is None else dropin
        args = (_ptr(queries), nq, k, nprobe, rerank_k, _metric(metric), _ptr(mask), _ptr(out), _stream(stream))
        if dropin:
            name = "cuda_ivf_pq_search_batch" if self.mode == "pq" else "cuda_ivf_sq_search_batch"
            call(name, C.byref(self.struct), *args)
        else:
            name = "fv_ivf_pq_search_ex" if self.mode == "pq" else "fv_ivf_sq_search_ex"
            call(name, C.byref(self.struct), C.byref(self.options), *args)
        return out
