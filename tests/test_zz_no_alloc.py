"""The allocation-free flat scan, fv_flat_scan_batch_noalloc.

It exists for callers that may not allocate device memory (a thread running
while a CUDA graph is captured in global mode, a latency-critical serving
thread, a host whose memory all belongs to its own pool). Its heaps live in
a fixed 8 MiB device array instead of a per-stream arena. These tests call
it through the C ABI and require its output to equal cuda_flat_scan_batch's
bit for bit (the tolerance of every exact-scan test here) on two calls in a
row -- the second call finds the first call's data still in the shared
array -- and check that a call too large for the array is refused.

The file name sorts last so that a run stopping at the first failure has
run every other test before this one.
"""
from __future__ import annotations

import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _call(name, base, queries, k, metric=0, mask=None, vec_ids=None):
    import torch

    from fvgb300 import _lib

    nq = queries.shape[0]
    out = torch.full((nq, min(k, 256), 2), -7, dtype=torch.int32, device="cuda")
    rc = getattr(_lib.lib(), name)(
        C.c_void_p(base.data_ptr()), None if vec_ids is None else C.c_void_p(vec_ids.data_ptr()), base.shape[0],
        base.shape[1], C.c_void_p(queries.data_ptr()), nq, k, metric,
        None if mask is None else C.c_void_p(mask.data_ptr()), C.c_void_p(out.data_ptr()),
        C.c_void_p(torch.cuda.current_stream().cuda_stream))
    return rc, out


def test_noalloc_matches_allocating_scan_twice(cuda):
    torch = cuda
    g = torch.Generator(device="cuda").manual_seed(5)
    # enough rows and queries that the scan splits the base range (the heaps
    # then go through the fixed array), two different inputs back to back
    cases = [(60000, 64, 100, 10, 0), (33000, 40, 70, 25, 2)]
    for n, dim, nq, k, metric in cases:
        base = torch.randn((n, dim), generator=g, device="cuda")
        queries = torch.randn((nq, dim), generator=g, device="cuda")
        words = torch.randint(-2**31, 2**31 - 1, ((n + 31) // 32,), generator=g, device="cuda", dtype=torch.int32)
        rc_ref, ref = _call("cuda_flat_scan_batch", base, queries, k, metric, mask=words)
        rc, got = _call("fv_flat_scan_batch_noalloc", base, queries, k, metric, mask=words)
        torch.cuda.synchronize()
        assert rc_ref == 0 and rc == 0
        assert torch.equal(ref, got)
        ids = got[..., 0].cpu().numpy().view(np.uint32)
        assert np.all(ids != 0xFFFFFFFF)


def test_noalloc_refuses_work_beyond_the_array(cuda):
    torch = cuda
    # 1024 queries x 256 results x the split count the scan picks for a
    # million rows needs far more than 8 MiB of heaps: refused, nothing run
    base = torch.zeros((1_000_000, 4), device="cuda")
    queries = torch.zeros((1024, 4), device="cuda")
    rc, out = _call("fv_flat_scan_batch_noalloc", base, queries, 256)
    torch.cuda.synchronize()
    assert rc == -6  # FV_ERR_SCRATCH_LIMIT
    assert torch.all(out == -7)  # outputs untouched


def test_noalloc_at_the_array_limit(cuda):
    """k = 256 over 20,000 rows: the scan splits the base into 32 ranges
    (the merge sorts at most 8,192 keys per query, 8,192 / 256 = 32), so 128
    queries need 128 x 32 x 256 x 8 bytes = exactly the 8 MiB array -- run,
    bit-identical to cuda_flat_scan_batch, twice, for L2 and cosine -- and
    129 queries need more -- refused, nothing written."""
    torch = cuda
    g = torch.Generator(device="cuda").manual_seed(11)
    base = torch.randn((20000, 48), generator=g, device="cuda")
    for metric in (0, 1):
        for rep in range(2):
            queries = torch.randn((128, 48), generator=g, device="cuda")
            rc_ref, ref = _call("cuda_flat_scan_batch", base, queries, 256, metric)
            rc, got = _call("fv_flat_scan_batch_noalloc", base, queries, 256, metric)
            torch.cuda.synchronize()
            assert rc_ref == 0 and rc == 0, (metric, rep, rc)
            assert torch.equal(ref, got), (metric, rep)
    queries = torch.randn((129, 48), generator=g, device="cuda")
    rc, out = _call("fv_flat_scan_batch_noalloc", base, queries, 256, 0)
    torch.cuda.synchronize()
    assert rc == -6 and torch.all(out == -7)
