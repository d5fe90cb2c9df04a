"""Device-resident IVF-PQ / IVF-SQ8 / IVF-RaBitQ tables and the calls that
search them.

A table holds the reference's layout (IvfPqGpuTables / IvfSqGpuTables /
IvfRabitqGpuTables: centroids, codebooks, SQ8 min/scale or the RaBitQ
rotation, code rows by vector id, posting-list offsets and ids, the fp32 rows
for the rerank) as torch CUDA tensors, plus an optional list-major copy of
the code rows for the contiguous-scan path.
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


# the engine's RaBitQ rotation seed (index.rs:435-441)
RABITQ_SEED = 0x5F37_59DF_CAFE_BABE


def rabitq_padded_dim(dim) -> int:
    return int(_lib.lib().fv_rabitq_padded_dim(dim))


def rabitq_rot_signs(padded_dim, seed=RABITQ_SEED):
    out = np.zeros(3 * padded_dim, dtype=np.float32)
    _lib.lib().fv_rabitq_rot_signs(padded_dim, seed, out.ctypes.data_as(C.c_void_p))
    return out


def build_rabitq(vectors, centroids, assign, seed=RABITQ_SEED, stream=None):
    """GPU RaBitQ encoder (fv_build_rabitq): `assign` is an int tensor of
    nearest-centroid ids or a k = 1 result tensor [n, 1, 2] / [n, 2]. Returns
    a dict with padded_dim, rot_signs, rot_centroids, rabitq_bits, rabitq_meta
    (device tensors)."""
    vectors = vectors.contiguous()
    centroids = centroids.contiguous()
    n, dim = vectors.shape
    nlist = centroids.shape[0]
    dev = vectors.device
    if assign.dtype in (torch.int32, torch.int64) and assign.dim() == 1:
        res = torch.zeros((n, 2), dtype=torch.int32, device=dev)
        res[:, 0] = assign.to(torch.int32)
    else:
        res = assign.reshape(n, 2).contiguous()
    P = rabitq_padded_dim(dim)
    signs = torch.from_numpy(rabitq_rot_signs(P, seed)).to(dev)
    rot_c = torch.empty((nlist, P), dtype=torch.float32, device=dev)
    bits = torch.empty((n, P // 32), dtype=torch.int32, device=dev)
    meta = torch.empty((n, 4), dtype=torch.float32, device=dev)
    call("fv_build_rabitq", _ptr(vectors), n, dim, _ptr(centroids), nlist, _ptr(res), _ptr(signs), P, _ptr(rot_c),
         _ptr(bits), _ptr(meta), _stream(stream))
    return {"padded_dim": P, "rot_signs": signs, "rot_centroids": rot_c, "rabitq_bits": bits, "rabitq_meta": meta}


_SEARCH = {"pq": ("cuda_ivf_pq_search_batch", "fv_ivf_pq_search_ex"),
           "sq8": ("cuda_ivf_sq_search_batch", "fv_ivf_sq_search_ex"),
           "rabitq": ("cuda_ivf_rabitq_search_batch", "fv_ivf_rabitq_search_ex")}


class IvfTable:
    """mode "pq", "sq8" or "rabitq"; `t` is a dict of host or device arrays
    with the keys centroids, offsets, vec_ids and (pq) codebooks, pq_codes /
    (sq8) sq_mins, sq_scales, sq_codes / (rabitq) padded_dim, rot_signs,
    rot_centroids, rabitq_bits, rabitq_meta."""

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
        elif mode == "sq8":
            self.sq_mins = _dev(t["sq_mins"], device=device)
            self.sq_scales = _dev(t["sq_scales"], device=device)
            self.codes = _dev(t["sq_codes"], device=device)
        else:
            self.padded_dim = int(t["padded_dim"])
            self.rot_signs = _dev(t["rot_signs"], device=device)
            self.rot_centroids = _dev(t["rot_centroids"], device=device)
            self.codes = _dev(t["rabitq_bits"], device=device)
            self.meta = _dev(t["rabitq_meta"], device=device)
        self.list_major = list_major
        self.codes_lm = self.meta_lm = None
        if list_major:
            if mode == "rabitq":
                self.codes_lm = relayout_codes(self.codes.view(torch.uint8).reshape(self.n, -1),
                                               self.vec_ids).view(torch.int32).reshape(self.n, -1)
                self.meta_lm = relayout_codes(self.meta.view(torch.uint8).reshape(self.n, -1),
                                              self.vec_ids).view(torch.float32).reshape(self.n, 4)
            else:
                self.codes_lm = relayout_codes(self.codes, self.vec_ids)
        self._build_structs()

    def _build_structs(self):
        vec = self.vectors.data_ptr() if self.vectors is not None else None
        codes = (self.codes_lm if self.list_major else self.codes).data_ptr()
        if self.mode == "pq":
            self.struct = _lib.IvfPqGpuTables(self.centroids.data_ptr(), self.codebooks.data_ptr(), codes,
                                              self.offsets.data_ptr(), self.vec_ids.data_ptr(), vec, self.n, self.dim,
                                              self.nlist, self.m_pq, self.sub_dim)
        elif self.mode == "sq8":
            self.struct = _lib.IvfSqGpuTables(self.centroids.data_ptr(), self.sq_mins.data_ptr(),
                                              self.sq_scales.data_ptr(), codes, self.offsets.data_ptr(),
                                              self.vec_ids.data_ptr(), vec, self.n, self.dim, self.nlist)
        else:
            meta = (self.meta_lm if self.list_major else self.meta).data_ptr()
            self.struct = _lib.IvfRabitqGpuTables(self.centroids.data_ptr(), self.rot_centroids.data_ptr(), codes,
                                                  meta, self.rot_signs.data_ptr(), self.offsets.data_ptr(),
                                                  self.vec_ids.data_ptr(), vec, self.n, self.dim, self.padded_dim,
                                                  self.padded_dim // 32, self.nlist)
        self.options = _lib.FvIvfOptions(1 if self.list_major else 0)

    def search(self, queries, k, nprobe, rerank_k, metric="l2", mask=None, out=None, stream=None, dropin=None):
        """cuda_ivf_{pq,sq,rabitq}_search_batch (reference layout) or the
        fv_*_ex call (list-major layout)."""
        nq = queries.shape[0]
        if out is None:
            out = empty_results(nq, min(k, 256), queries.device)
        dropin = (not self.list_major) if dropin is None else dropin
        args = (_ptr(queries), nq, k, nprobe, rerank_k, _metric(metric), _ptr(mask), _ptr(out), _stream(stream))
        dropin_name, ex_name = _SEARCH[self.mode]
        if dropin:
            call(dropin_name, C.byref(self.struct), *args)
        else:
            call(ex_name, C.byref(self.struct), C.byref(self.options), *args)
        return out
