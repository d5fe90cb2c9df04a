"""SearchBatcher: the reference's micro-batching queue
(crates/server/src/batcher.rs:82-259) over the native continuous-batching
loop of libfvgb300 (fv_serve_* in include/fv_serve.h).

Names follow the reference: BatchKey (algorithm, top_k, ef_or_nprobe,
rerank_k), BatcherStats (total_requests, total_batches, avg_batch_size),
SearchBatcher.for_index / with_executor / submit / stats. submit() here
returns a ticket (the reference awaits a oneshot); wait() or search()
blocks for the answer. The native loop keeps several batches in flight,
batches requests with different filters together and, for IVF, requests
with different k / nprobe / rerank_k (group_by_params=True restores the
reference's equal-key rule).
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import numpy as np

from . import _lib
from ._lib import FvError, call
from .datasets import pack_bools

ALGORITHM = {"flat": 0, "fp16": 1, "fp16_tc": 1, "fp8": 2, "ivf_pq": 3, "ivf-pq": 3, "ivf": 3, "pq": 3,
             "ivf_sq8": 4, "ivf-sq8": 4, "sq8": 4, "ivf_rabitq": 5, "ivf-rabitq": 5, "rabitq": 5}
ALGORITHM_NAME = {0: "flat", 1: "fp16", 2: "fp8", 3: "ivf_pq", 4: "ivf_sq8", 5: "ivf_rabitq"}


@dataclass(frozen=True)
class BatchKey:
    """batcher.rs:55-61. algorithm: an engine name (flat, fp16, fp8, ivf_pq,
    ivf_sq8, ivf_rabitq); ef_or_nprobe is the IVF nprobe."""
    algorithm: str
    top_k: int
    ef_or_nprobe: int = 0
    rerank_k: int = 0

    def request(self, filter_id: int = -1) -> _lib.FvRequest:
        return _lib.FvRequest(ALGORITHM[self.algorithm.lower()], self.top_k, self.ef_or_nprobe, self.rerank_k,
                              filter_id, 0)


@dataclass(frozen=True)
class BatcherStats:
    """batcher.rs:63-68."""
    total_requests: int
    total_batches: int
    avg_batch_size: float


def _config(max_wait_us, max_batch_size, inflight, group_by_params, queue_capacity, scratch_budget_kb=0,
            graphs=False):
    return _lib.FvServeConfig(max_batch_size, max_wait_us, inflight, 1 if group_by_params else 0, queue_capacity,
                              scratch_budget_kb, 1 if graphs else 0, 0)


class SearchBatcher:
    def __init__(self, handle: C.c_void_p, dim: int, keepalive=None):
        self._h = handle
        self.dim = dim
        self._keepalive = keepalive  # index or executor callback the native loop uses

    @classmethod
    def for_index(cls, index, max_wait_us: int = 350, max_batch_size: int = 64, inflight: int = 4,
                  group_by_params: bool = False, queue_capacity: int = 0,
                  scratch_budget_kb: int = 0, graphs: bool = False) -> "SearchBatcher":
        """batcher.rs:89-125 (defaults: 350 us window, 64 requests). Batches
        are admitted by scratch memory: together those in flight hold at most
        scratch_budget_kb KiB (0: 512 MiB) of device scratch. graphs: each
        batch's kernels run as one CUDA graph (FvServeConfig.graphs)."""
        h = C.c_void_p()
        cfg = _config(max_wait_us, max_batch_size, inflight, group_by_params, queue_capacity, scratch_budget_kb,
                      graphs)
        call("fv_serve_create", index._h, C.byref(cfg), C.byref(h))
        return cls(h, index.config.dim, keepalive=index)

    @classmethod
    def with_executor(cls, dim: int, executor, max_wait_us: int = 350, max_batch_size: int = 64, inflight: int = 1,
                      group_by_params: bool = True) -> "SearchBatcher":
        """batcher.rs:127-226: executor(key, queries[nq, dim], num_queries)
        returns num_queries * key.top_k (id, distance) pairs (a sequence or an
        (n, 2) array), or raises; a failure fails every request of the batch."""

        def trampoline(user, reqs, queries, nq, d, k_stride, out):
            try:
                r0 = reqs[0]
                key = BatchKey(ALGORITHM_NAME.get(r0.engine, str(r0.engine)), r0.top_k, r0.nprobe, r0.rerank_k)
                q = np.ctypeslib.as_array(queries, shape=(nq * d,)).reshape(nq, d).copy()
                res = executor(key, q, nq)
                for qi in range(nq):
                    k = reqs[qi].top_k
                    for r in range(min(k, k_stride)):
                        item = res[qi * key.top_k + r] if qi * key.top_k + r < len(res) else None
                        if item is None:
                            continue
                        out[qi * k_stride + r].id = int(item[0])
                        out[qi * k_stride + r].distance = float(item[1])
                return 0
            except Exception:  # noqa: BLE001 -- reported as the batch's status
                return -2

        cb = _lib.FvServeExecutor(trampoline)
        h = C.c_void_p()
        cfg = _config(max_wait_us, max_batch_size, inflight, group_by_params, 0)
        call("fv_serve_create_with_executor", dim, C.byref(cfg), cb, None, C.byref(h))
        return cls(h, dim, keepalive=cb)

    def close(self):
        if self._h is not None and self._h.value:
            _lib.lib().fv_serve_destroy(self._h)
        self._h = None

    def __del__(self):
        self.close()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    # ------------------------------------------------------------ filters
    def add_filter(self, mask) -> int:
        """A filter over logical ids: packed u32 words or a bool array."""
        m = np.asarray(mask)
        if m.dtype == bool:
            m = pack_bools(m)
        m = np.ascontiguousarray(m, dtype=np.uint32)
        out = C.c_int32(-1)
        call("fv_serve_add_filter", self._h, m.ctypes.data_as(C.c_void_p), m.shape[0], C.byref(out))
        return out.value

    def remove_filter(self, filter_id: int) -> None:
        call("fv_serve_remove_filter", self._h, filter_id)

    # ------------------------------------------------------------ requests
    def submit(self, key: BatchKey, query, filter_id: int = -1) -> int:
        q = np.ascontiguousarray(np.asarray(query, dtype=np.float32).reshape(-1))
        if q.shape[0] != self.dim:
            raise ValueError(f"query has {q.shape[0]} values, expected {self.dim}")
        req = key.request(filter_id)
        t = C.c_uint64(0)
        call("fv_serve_submit", self._h, C.byref(req), q.ctypes.data_as(C.c_void_p), C.byref(t))
        return t.value

    def wait(self, ticket: int, top_k: int, timeout_ms: int = 0):
        """(ids, distances, latency_us) of a submitted request."""
        out = np.zeros((top_k, 2), dtype=np.uint32)
        lat = C.c_double(0.0)
        call("fv_serve_wait", self._h, ticket, out.ctypes.data_as(C.c_void_p), top_k, timeout_ms, C.byref(lat))
        return out[:, 0].copy(), out[:, 1].view(np.float32).copy(), lat.value

    def search(self, key: BatchKey, query, filter_id: int = -1, timeout_ms: int = 0):
        return self.wait(self.submit(key, query, filter_id), key.top_k, timeout_ms)

    def replay(self, keys, queries, arrivals_ns, filter_ids=None):
        """Open-loop replay: request i arrives arrivals_ns[i] after the start.
        Returns (ids [n, kmax], distances [n, kmax], status [n]); entries past
        a request's top_k are sentinels."""
        n = len(keys)
        q = np.ascontiguousarray(np.asarray(queries, dtype=np.float32).reshape(n, self.dim))
        fids = [-1] * n if filter_ids is None else list(filter_ids)
        reqs = (_lib.FvRequest * n)(*[k.request(int(f)) for k, f in zip(keys, fids)])
        arr = np.ascontiguousarray(np.asarray(arrivals_ns, dtype=np.uint64))
        kmax = max(k.top_k for k in keys) if n else 1
        out = np.zeros((n, kmax, 2), dtype=np.uint32)
        out[..., 0] = 0xFFFFFFFF
        out[..., 1] = np.float32(1e30).view(np.uint32)
        status = np.zeros(n, dtype=np.int32)
        call("fv_serve_replay", self._h, reqs, q.ctypes.data_as(C.c_void_p), arr.ctypes.data_as(C.c_void_p), n,
             out.ctypes.data_as(C.c_void_p), kmax, status.ctypes.data_as(C.c_void_p))
        return out[..., 0].copy(), out[..., 1].view(np.float32).copy(), status

    # -------------------------------------------------------------- stats
    def stats(self) -> BatcherStats:
        s = self.serve_stats()
        return BatcherStats(s["total_requests"], s["total_batches"], s["avg_batch_size"])

    def serve_stats(self) -> dict:
        s = _lib.FvServeStats()
        call("fv_serve_stats", self._h, C.byref(s))
        return {f: getattr(s, f) for f, _ in s._fields_ if f != "reserved"}

    def reset_stats(self) -> None:
        call("fv_serve_reset_stats", self._h)

    def scratch_estimate(self, key: BatchKey, num_queries: int) -> int:
        """Scratch bytes one batch of `num_queries` requests like `key` takes
        (what admission charges against the budget)."""
        out = C.c_uint64(0)
        req = key.request()
        call("fv_serve_scratch_estimate", self._h, C.byref(req), num_queries, C.byref(out))
        return out.value


__all__ = ["ALGORITHM", "BatchKey", "BatcherStats", "FvError", "SearchBatcher"]
