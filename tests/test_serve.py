"""The continuous-batching loop's host logic (no GPU): the native server
driven by a host executor, after the reference's batcher tests
(crates/server/src/batcher.rs:261-362)."""
from __future__ import annotations

import threading
import time

import numpy as np
import pytest

from fvgb300._lib import FvError
from fvgb300.serve import BatchKey, SearchBatcher


def tag_executor(calls, delay=0.0, seen=None):
    """batcher.rs:270-287: result id = tag * 100 + rank, tag = query[0]."""

    def run(key, queries, nq):
        calls.append(nq)
        if seen is not None:
            seen.append(key)
        if delay:
            time.sleep(delay)
        out = []
        for qi in range(nq):
            tag = int(queries[qi, 0])
            out.extend((tag * 100 + r, float(r)) for r in range(key.top_k))
        return out

    return run


def test_micro_batcher_coalesces_concurrent_queries():
    calls = []
    b = SearchBatcher.with_executor(4, tag_executor(calls, delay=0.01), max_wait_us=5000, max_batch_size=32)
    key = BatchKey("ivf_pq", 4, 32, 0)
    results = {}

    def client(qid):
        ids, dist, _ = b.search(key, np.full(4, qid, np.float32))
        results[qid] = (ids, dist)

    threads = [threading.Thread(target=client, args=(i,)) for i in range(8)]
    for t in threads:
        t.start()
    for t in threads:
        t.join()
    for qid, (ids, dist) in results.items():
        assert len(ids) == 4 and ids[0] == qid * 100 and dist[1] == 1.0
    st = b.stats()
    assert st.total_requests == 8
    assert st.total_batches < 8, f"expected coalesced batches < 8, got {st.total_batches}"
    assert len(calls) == st.total_batches
    b.close()


def test_micro_batcher_separates_distinct_keys():
    """batcher.rs:327-361: requests with different keys never share a batch."""
    seen = []
    b = SearchBatcher.with_executor(4, tag_executor([], seen=seen), max_wait_us=2000, max_batch_size=16)
    k1 = BatchKey("fp16", 2, 64, 0)
    k2 = BatchKey("ivf_sq8", 5, 8, 32)
    t1, t2 = b.submit(k1, np.ones(4, np.float32)), b.submit(k2, np.full(4, 2.0, np.float32))
    r1, r2 = b.wait(t1, 2), b.wait(t2, 5)
    assert len(r1[0]) == 2 and len(r2[0]) == 5
    assert r2[0][0] == 200
    assert len({(k.algorithm, k.top_k) for k in seen}) == len(seen) == 2
    b.close()


def test_heterogeneous_ivf_requests_share_a_launch():
    """Without group_by_params, IVF requests with different k / nprobe /
    rerank share one batch; flat and tensor-core requests batch per k."""
    batches = []

    def run(key, queries, nq):
        batches.append(nq)
        time.sleep(0.02)
        return [(int(queries[i, 0]), 0.0) for i in range(nq) for _ in range(key.top_k)]

    b = SearchBatcher.with_executor(2, run, max_wait_us=20000, max_batch_size=64, group_by_params=False)
    keys = [BatchKey("ivf_pq", 10, 16, 0), BatchKey("ivf_pq", 100, 64, 400), BatchKey("ivf_pq", 10, 64, 0),
            BatchKey("ivf_pq", 1, 1, 1)]
    tickets = [(b.submit(k, np.array([i, 0], np.float32)), k) for i, k in enumerate(keys)]
    for i, (t, k) in enumerate(tickets):
        ids, _, _ = b.wait(t, k.top_k)
        assert ids[0] == i
    assert sum(batches) == 4 and len(batches) <= 2  # the first may go alone (idle GPU), the rest together
    b.close()


def test_concurrent_inflight_batches():
    """Several batches run at once (one stream each on the GPU)."""
    active = [0, 0]
    lock = threading.Lock()

    def run(key, queries, nq):
        with lock:
            active[0] += 1
            active[1] = max(active[1], active[0])
        time.sleep(0.05)
        with lock:
            active[0] -= 1
        return [(0, 0.0)] * (nq * key.top_k)

    b = SearchBatcher.with_executor(2, run, max_wait_us=0, max_batch_size=1, inflight=4)
    key = BatchKey("flat", 1)
    tickets = [b.submit(key, np.zeros(2, np.float32)) for _ in range(8)]
    for t in tickets:
        b.wait(t, 1)
    assert active[1] >= 2
    s = b.serve_stats()
    assert s["max_inflight"] >= 2 and s["completed"] == 8 and s["total_batches"] == 8
    b.close()


def test_replay_latency_accounting():
    """Open-loop replay: latency runs from the scheduled arrival; with a
    busy executor later requests queue, so p99 > p50 and queue delays show."""
    b = SearchBatcher.with_executor(2, tag_executor([], delay=0.004), max_wait_us=0, max_batch_size=4, inflight=1)
    n = 40
    keys = [BatchKey("flat", 3)] * n
    q = np.zeros((n, 2), np.float32)
    q[:, 0] = np.arange(n)
    arrivals = np.arange(n, dtype=np.uint64) * 200_000  # 5k requests/s against a 4 ms executor
    ids, dist, status = b.replay(keys, q, arrivals)
    assert np.all(status == 0)
    assert np.array_equal(ids[:, 0], np.arange(n) * 100)
    s = b.serve_stats()
    assert s["completed"] == n and s["failed"] == 0
    assert s["p99_us"] >= s["p50_us"] > 0
    assert s["queue_p99_us"] > 0
    assert s["qps"] > 0
    assert s["avg_batch_size"] > 1.0  # requests accumulated behind the busy executor
    b.reset_stats()
    assert b.serve_stats()["completed"] == 0
    b.close()


def test_errors_and_admission():
    def fail(key, queries, nq):
        raise RuntimeError("executor failure")

    b = SearchBatcher.with_executor(2, fail, max_wait_us=0)
    t = b.submit(BatchKey("flat", 2), np.zeros(2, np.float32))
    with pytest.raises(FvError):
        b.wait(t, 2)
    assert b.serve_stats()["failed"] == 1
    with pytest.raises(FvError):
        b.submit(BatchKey("flat", 300), np.zeros(2, np.float32))  # top_k > 256
    with pytest.raises(FvError):
        b.submit(BatchKey("flat", 2), np.zeros(2, np.float32), filter_id=7)  # unknown filter
    with pytest.raises(ValueError):
        b.submit(BatchKey("flat", 2), np.zeros(3, np.float32))
    fid = b.add_filter(np.array([True, False, True]))
    b.remove_filter(fid)
    with pytest.raises(FvError):
        b.remove_filter(fid)
    b.close()


def test_queue_capacity():
    import ctypes as C

    from fvgb300 import _lib

    gate = threading.Event()

    cb = _lib.FvServeExecutor(lambda u, r, q, nq, d, ks, out: (gate.wait(5), 0)[1])
    h = C.c_void_p()
    cfg = _lib.FvServeConfig(1, 0, 1, 1, 2, 0, 0, 0)
    _lib.call("fv_serve_create_with_executor", 2, C.byref(cfg), cb, None, C.byref(h))
    b = SearchBatcher(h, 2, keepalive=cb)
    key = BatchKey("flat", 1)
    first = b.submit(key, np.zeros(2, np.float32))  # dispatched; the executor blocks
    time.sleep(0.05)
    held = [b.submit(key, np.zeros(2, np.float32)) for _ in range(2)]
    with pytest.raises(FvError) as e:
        b.submit(key, np.zeros(2, np.float32))
    assert e.value.code == -7  # FV_ERR_QUEUE_FULL
    gate.set()
    for t in [first] + held:
        b.wait(t, 1)
    b.close()
