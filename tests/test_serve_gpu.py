"""The serving loop on the GPU: every answer served in a mixed batch is
the answer the engine's blocking search gives that request alone
(fv_index_search: same clamps, filter AND tombstones, live-insert merge)."""
from __future__ import annotations

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def gen_clustered(n, dim, clusters, seed, sigma=0.25):
    rng = np.random.default_rng(seed)
    centers = rng.uniform(-1, 1, size=(clusters, dim)).astype(np.float32)
    return (centers[np.arange(n) % clusters] + np.float32(sigma) * rng.standard_normal((n, dim))).astype(np.float32)


@pytest.fixture(scope="module")
def served(cuda):
    from fvgb300.index import (BUILD_FP8, BUILD_FP16, BUILD_IVF_PQ, BUILD_IVF_RABITQ, BUILD_IVF_SQ8, GpuVectorIndex,
                               IndexConfig)

    x = gen_clustered(6000, 64, 24, 11)
    idx = GpuVectorIndex(IndexConfig(dim=64, nlist=32, m_pq=8, metric="l2",
                                     build_flags=BUILD_FP16 | BUILD_FP8 | BUILD_IVF_PQ | BUILD_IVF_SQ8 |
                                     BUILD_IVF_RABITQ))
    idx.build(x)
    extra = gen_clustered(300, 64, 24, 12)
    idx.add_vectors(extra)
    idx.delete_ids([3, 5, 6000, 6001, 4242])
    return idx, np.vstack([x, extra])


def make_mix(n, rng, dim, engines):
    from fvgb300.serve import BatchKey

    keys, fids = [], []
    for i in range(n):
        eng = engines[rng.integers(len(engines))]
        k = int(rng.choice([1, 10, 100]))
        npb = int(rng.choice([4, 16])) if eng.startswith("ivf") else 0
        rr = int(rng.choice([0, 64, 1])) if eng.startswith("ivf") else 0
        keys.append(BatchKey(eng, k, npb, rr))
        fids.append(int(rng.integers(-1, 2)))
    q = gen_clustered(n, dim, 24, int(rng.integers(1 << 30)))
    return keys, fids, q


def alone(idx, key, q, filt):
    from fvgb300.serve import ALGORITHM

    eng = ALGORITHM[key.algorithm]
    if eng == 0:
        return idx.batch_search_flat(q[None], 1, key.top_k, filt)
    if eng in (1, 2):
        return (idx.batch_search_fp16_tc if eng == 1 else idx.batch_search_fp8)(q[None], 1, key.top_k, filt)
    return idx.batch_search_ivf_mode(q[None], 1, key.top_k, key.ef_or_nprobe, key.rerank_k,
                                     {3: "pq", 4: "sq8", 5: "rabitq"}[eng], filt)


@pytest.mark.parametrize("graphs", [False, True])
@pytest.mark.parametrize("group", [False, True])
def test_identical_alone_and_in_the_mix(served, group, graphs):
    """graphs: every batch runs as one CUDA graph (captured, applied to the
    stream's executable of its launch shape)."""
    from fvgb300.serve import SearchBatcher

    idx, rows = served
    rng = np.random.default_rng(5 + group)
    n_ids = rows.shape[0]
    filters = [rng.random(n_ids) < 0.2, (np.arange(n_ids) % 3) == 0]
    engines = ["flat", "fp16", "fp8", "ivf_pq", "ivf_sq8", "ivf_rabitq"]
    keys, fids, q = make_mix(160, rng, 64, engines)
    with SearchBatcher.for_index(idx, max_wait_us=2000, max_batch_size=64, inflight=3,
                                 group_by_params=group, graphs=graphs) as b:
        fid_map = [b.add_filter(f) for f in filters]
        sfids = [fid_map[f] if f >= 0 else -1 for f in fids]
        # a burst: everything arrives at once, so the batches are mixed
        ids, dist, status = b.replay(keys, q, np.zeros(len(keys), dtype=np.uint64), sfids)
        s = b.serve_stats()
    assert np.all(status == 0)
    assert s["completed"] == len(keys) and s["avg_batch_size"] > 1.0
    assert (s["graph_instantiations"] > 0) == graphs
    for i, key in enumerate(keys):
        filt = filters[fids[i]] if fids[i] >= 0 else None
        a_ids, a_dist = alone(idx, key, q[i], filt)
        k = key.top_k
        assert np.array_equal(ids[i, :k], a_ids[0]), (i, key)
        assert np.array_equal(dist[i, :k], a_dist[0]), (i, key)
        if filt is not None:
            valid = ids[i, :k][ids[i, :k] != 0xFFFFFFFF]
            assert np.all(filt[valid])
        assert not np.isin(ids[i, :k], [3, 5, 6000, 6001, 4242]).any()


def test_poisson_arrivals_report_latency(served):
    from fvgb300.serve import BatchKey, SearchBatcher

    idx, rows = served
    rng = np.random.default_rng(9)
    n = 400
    gaps = rng.exponential(1e9 / 20000.0, n)  # 20k requests/s
    arrivals = np.cumsum(gaps).astype(np.uint64)
    keys = [BatchKey("ivf_sq8", 10, 16, 64) if i % 2 else BatchKey("fp16", 10) for i in range(n)]
    q = gen_clustered(n, 64, 24, 77)
    with SearchBatcher.for_index(idx, max_wait_us=200, max_batch_size=128, inflight=4) as b:
        ids, _, status = b.replay(keys, q, arrivals)
        s = b.serve_stats()
    assert np.all(status == 0) and np.all(ids[:, 0] != 0xFFFFFFFF)
    assert s["completed"] == n and s["qps"] > 0 and s["p99_us"] >= s["p50_us"] > 0


def test_graph_launches_reuse_executables(served):
    """The same bursts served twice with graphs: batches of a launch shape
    already seen on the stream update its executable instead of building one
    (fewer instantiations than batches), and every pass gives the answers of
    the kernel-by-kernel launch."""
    from fvgb300.serve import BatchKey, SearchBatcher

    idx, rows = served
    q = gen_clustered(256, 64, 24, 31)
    keys = [BatchKey("fp16", 10), BatchKey("ivf_sq8", 10, 16, 64), BatchKey("fp8", 100), BatchKey("flat", 10)]
    with SearchBatcher.for_index(idx, max_wait_us=0, max_batch_size=64, inflight=1) as b:
        want = [_burst(b, key, q) for key in keys]
    with SearchBatcher.for_index(idx, max_wait_us=0, max_batch_size=64, inflight=1, graphs=True) as b:
        got1 = [_burst(b, key, q) for key in keys]
        built = b.serve_stats()["graph_instantiations"]
        got2 = [_burst(b, key, q) for key in keys]
        s = b.serve_stats()
    assert built > 0 and s["graph_instantiations"] < s["total_batches"]
    for w, g1, g2 in zip(want, got1, got2):
        for a in (g1, g2):
            assert np.all(a[2] == 0)
            assert np.array_equal(a[0], w[0]) and np.array_equal(a[1], w[1])


@pytest.mark.parametrize("graphs", [False, True])
def test_serving_survives_index_updates(served, graphs):
    """Writers wait for the batches in flight; requests after an update see it."""
    from fvgb300.serve import BatchKey, SearchBatcher

    idx, rows = served
    marker = np.full((1, 64), 40.0, dtype=np.float32)
    with SearchBatcher.for_index(idx, max_wait_us=0, inflight=2, graphs=graphs) as b:
        key = BatchKey("flat", 5)
        before = b.search(key, marker[0])[0]
        new_id = int(idx.add_vectors(marker)[0])
        after = b.search(key, marker[0])[0]
        assert after[0] == new_id and before[0] != new_id
        idx.delete_ids([new_id])
        assert b.search(key, marker[0])[0][0] != new_id


def _burst(b, key, q):
    return b.replay([key] * q.shape[0], q, np.zeros(q.shape[0], dtype=np.uint64))


def test_batches_admitted_by_scratch_memory(served):
    """A budget that holds one full batch's scratch (plus a little): a burst
    of batches is held back until scratch frees up instead of growing device
    memory; the scratch held in flight never exceeds the budget; the answers
    are still those of the blocking search. A budget below one full batch
    cuts batches smaller; a budget below one request fails the requests with
    FV_ERR_SCRATCH_LIMIT."""
    from fvgb300.serve import BatchKey, SearchBatcher

    idx, rows = served
    key = BatchKey("fp16", 100)
    with SearchBatcher.for_index(idx, max_wait_us=0, max_batch_size=64, inflight=4) as probe:
        full, single = probe.scratch_estimate(key, 64), probe.scratch_estimate(key, 1)
    assert full > 4 * single > 0
    q = gen_clustered(320, 64, 24, 31)

    budget_kb = (full * 3 // 2 + 1023) // 1024
    with SearchBatcher.for_index(idx, max_wait_us=0, max_batch_size=64, inflight=4,
                                 scratch_budget_kb=budget_kb) as b:
        ids, dist, status = _burst(b, key, q)
        s = b.serve_stats()
    assert np.all(status == 0) and s["completed"] == q.shape[0]
    assert s["scratch_pool_bytes"] == budget_kb * 1024
    assert full <= s["scratch_peak_bytes"] <= s["scratch_pool_bytes"]
    assert s["scratch_waits"] > 0 and s["max_inflight"] <= 2
    for i in range(0, q.shape[0], 23):
        a_ids, a_dist = alone(idx, key, q[i], None)
        assert np.array_equal(ids[i], a_ids[0]) and np.array_equal(dist[i], a_dist[0]), i

    small_kb = (full // 2 + 1023) // 1024
    with SearchBatcher.for_index(idx, max_wait_us=0, max_batch_size=64, inflight=4,
                                 scratch_budget_kb=small_kb) as b:
        ids2, dist2, status2 = _burst(b, key, q)
        s2 = b.serve_stats()
    assert np.all(status2 == 0) and s2["scratch_split"] > 0
    assert s2["scratch_peak_bytes"] <= s2["scratch_pool_bytes"]
    assert np.array_equal(ids2, ids) and np.array_equal(dist2, dist)

    with SearchBatcher.for_index(idx, max_wait_us=0, max_batch_size=64, inflight=4, scratch_budget_kb=1) as b:
        _, _, status3 = _burst(b, key, q[:8])
        s3 = b.serve_stats()
    assert np.all(status3 == -6) and s3["failed"] == 8 and s3["scratch_peak_bytes"] == 0
