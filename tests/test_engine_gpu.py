"""The native engine (GpuVectorIndex mirror) end to end, after the reference's
integration tests (tests/e2e_search_test.rs, python/tests/test_bindings.py).

The tables the engine builds on the GPU are exported and checked against
the oracle's restatement of the reference's encoders, and the engine's IVF
answers must equal the oracle's search over those same tables."""
from __future__ import annotations

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def gen_clustered(n, dim, clusters, seed, sigma=0.18):
    """e2e_search_test.rs:156-177 shape: centres U(-1, 1), row i in cluster i % c."""
    rng = np.random.default_rng(seed)
    centers = rng.uniform(-1, 1, size=(clusters, dim)).astype(np.float32)
    return (centers[np.arange(n) % clusters] + np.float32(sigma) * rng.standard_normal((n, dim))).astype(np.float32)


def make_index(x, nlist, m_pq, metric="l2", flags=None, **kw):
    from fvgb300.index import (BUILD_FP8, BUILD_FP16, BUILD_IVF_PQ, BUILD_IVF_RABITQ, BUILD_IVF_SQ8, GpuVectorIndex,
                               IndexConfig)

    cfg = IndexConfig(dim=x.shape[1], nlist=nlist, m_pq=m_pq, metric=metric,
                      build_flags=flags or (BUILD_FP16 | BUILD_FP8 | BUILD_IVF_PQ | BUILD_IVF_SQ8 | BUILD_IVF_RABITQ),
                      **kw)
    idx = GpuVectorIndex(cfg)
    idx.build(x)
    return idx


@pytest.fixture(scope="module")
def e2e(cuda):
    x = gen_clustered(1500, 96, 12, 202)
    return x, make_index(x, 24, 12)


def test_built_tables_match_oracle_encoders(cuda, oracle_mod, e2e):
    """Assignment = nearest centroid; residual PQ codes, SQ8 min/scale/codes
    equal the oracle's restatement of cluster.rs / quant.rs on the exported
    centroids and codebooks."""
    x, idx = e2e
    t = idx.export_ivf()
    nlist = t["nlist"]
    assert nlist == 24 and t["offsets"][-1] == x.shape[0]
    assign = np.zeros(x.shape[0], dtype=np.uint32)
    for l in range(nlist):
        assign[t["vec_ids"][t["offsets"][l]:t["offsets"][l + 1]]] = l
    assert np.array_equal(np.sort(t["vec_ids"]), np.arange(x.shape[0]))
    nearest = oracle_mod.exact_knn(t["centroids"], x, 1)["id"][:, 0]
    assert np.array_equal(assign, nearest)
    res = oracle_mod.residuals(x, t["centroids"], assign)
    assert np.array_equal(oracle_mod.pq_encode(res, t["codebooks"]), t["pq_codes"])
    mins, scales = oracle_mod.sq8_fit(res)
    assert np.array_equal(mins, t["sq_mins"]) and np.array_equal(scales, t["sq_scales"])
    assert np.array_equal(oracle_mod.sq8_encode(res, mins, scales), t["sq_codes"])
    # RaBitQ (index.rs:435-441: the engine's seed, the rows' own assignment)
    rq = oracle_mod.rabitq_encode(x, t["centroids"], assign)
    assert t["padded_dim"] == rq["padded_dim"] == 128
    assert np.array_equal(rq["rot_signs"], t["rot_signs"])
    for key in ("rot_centroids", "rabitq_bits", "rabitq_meta"):
        assert np.array_equal(rq[key].view(np.uint32), t[key].view(np.uint32)), key


@pytest.mark.parametrize("mode", ["pq", "sq8", "rabitq"])
def test_ivf_recall_and_parity_at_reference_params(cuda, oracle_mod, e2e, mode):
    """e2e_search_test.rs:231-277: nprobe 12, rerank 256, recall@10 >= 0.80
    for the first 8 rows as queries; answers equal the oracle on the
    engine's own tables. The 512 rerank (2-stage in the reference) too."""
    x, idx = e2e
    t = idx.export_ivf()
    q = x[:8]
    for rerank in (256, 512):
        ids, dist = idx.batch_search_ivf_mode(q, 8, 10, 12, rerank, mode)
        fn = {"pq": oracle_mod.ivf_pq_search, "sq8": oracle_mod.ivf_sq_search,
              "rabitq": oracle_mod.ivf_rabitq_search}[mode]
        ref = fn(t, x, q, 10, 12, rerank)
        assert np.array_equal(ids, ref["id"]) and np.array_equal(dist, ref["distance"])
        truth = oracle_mod.exact_knn(x, q, 10)
        assert oracle_mod.recall(ids, truth["id"]) >= 0.80


@pytest.mark.parametrize("metric", ["l2", "cosine"])
def test_fp16_self_query(cuda, metric):
    """e2e_search_test.rs:291-319: self-query nearest neighbour is row 0."""
    x = gen_clustered(512, 64, 8, 303)
    idx = make_index(x, 8, 8, metric)
    ids, _ = idx.batch_search_fp16_tc(x[:4], 4, 10)
    assert ids.shape == (4, 10) and ids[0, 0] == 0


def test_bitmask_filtering_all_engines(cuda):
    """e2e_search_test.rs:322-433: tenant / timestamp / ACL filter as a
    packed mask; no engine returns a masked-out id."""
    x = gen_clustered(600, 64, 6, 404)
    ids_all = np.arange(600)
    allowed = (ids_all % 3 == 0) & (1000 + ids_all >= 1100) & (ids_all % 2 == 0)
    from fvgb300.datasets import pack_bools

    words = pack_bools(allowed)
    idx = make_index(x, 12, 8)
    q = x[:1]
    runs = {
        "flat": idx.batch_search_flat(q, 1, 10, words),
        "fp16": idx.batch_search_fp16_tc(q, 1, 10, words),
        "fp8": idx.batch_search_fp8(q, 1, 10, words),
        "ivf_pq": idx.batch_search_ivf_mode(q, 1, 10, 12, 64, "pq", words),
        "ivf_sq8": idx.batch_search_ivf_mode(q, 1, 10, 12, 64, "sq8", words),
        "ivf_rabitq": idx.batch_search_ivf_mode(q, 1, 10, 12, 64, "rabitq", words),
    }
    for name, (ids, _) in runs.items():
        valid = ids[ids != 0xFFFFFFFF]
        assert valid.size > 0, name
        assert np.all(allowed[valid]), f"{name} returned a masked-out id"


def test_delta_insert_and_tombstones(cuda):
    """e2e_search_test.rs:436-471: a marker vector added to the live-insert
    buffer gets id = initial count and comes back at rank 0; deleting id 0
    removes it from every engine's answers."""
    x = gen_clustered(400, 32, 4, 505)
    idx = make_index(x, 8, 8)
    marker = np.full((1, 32), 50.0, dtype=np.float32)
    assert idx.add_vectors(marker).tolist() == [400]
    assert idx.delta_len() == 1
    for search in (lambda q: idx.batch_search_flat(q, 1, 5), lambda q: idx.batch_search_fp16_tc(q, 1, 5),
                   lambda q: idx.batch_search_ivf_mode(q, 1, 5, 8, 32, "pq"),
                   lambda q: idx.batch_search_ivf_mode(q, 1, 5, 8, 32, "sq8"),
                   lambda q: idx.batch_search_ivf_mode(q, 1, 5, 8, 32, "rabitq")):
        ids, dist = search(marker)
        assert ids[0, 0] == 400
        assert np.all(dist[0, :-1] <= dist[0, 1:])
    assert idx.delete_ids([0]) == 1
    assert idx.delete_ids([0]) == 0
    assert idx.tombstone_count() == 1
    q0 = x[:1]
    for ids, _ in (idx.batch_search_flat(q0, 1, 10), idx.batch_search_fp16_tc(q0, 1, 10),
                   idx.batch_search_ivf_mode(q0, 1, 10, 8, 32, "pq"),
                   idx.batch_search_ivf_mode(q0, 1, 10, 8, 32, "sq8"),
                   idx.batch_search_ivf_mode(q0, 1, 10, 8, 32, "rabitq")):
        assert np.all(ids != 0)
    # deleting a live-insert id removes it too
    assert idx.delete_ids([400]) == 1
    ids, _ = idx.batch_search_flat(marker, 1, 5)
    assert np.all(ids != 400)


def test_merge_matches_reference_rule(cuda, oracle_mod):
    """With live inserts the answer is the stable merge of the main and
    live-insert scans (index.rs:1353-1387): equal to an exact search over
    main + inserted rows (ties: main before inserted)."""
    rng = np.random.default_rng(8)
    x = np.rint(rng.uniform(0, 10, (3000, 16))).astype(np.float32)
    extra = np.rint(rng.uniform(0, 10, (300, 16))).astype(np.float32)
    idx = make_index(x, 16, 4)
    ids_new = idx.add_vectors(extra)
    assert ids_new[0] == 3000
    q = np.rint(rng.uniform(0, 10, (20, 16))).astype(np.float32)
    ids, dist = idx.batch_search_flat(q, 20, 12)
    ref = oracle_mod.exact_knn(np.vstack([x, extra]), q, 12)
    assert np.array_equal(ids, ref["id"]) and np.array_equal(dist, ref["distance"])


def test_large_top_k_ivf_and_device_ptr(cuda):
    """test_bindings.py:123-138 (k=100, sorted, >= 90% filled) and
    e2e_search_test.rs:84-154 (device-pointer queries give the host answer)."""
    torch = cuda
    rng = np.random.default_rng(3)
    x = rng.standard_normal((1000, 64)).astype(np.float32)
    idx = make_index(x, 16, 8)
    q = rng.standard_normal((1, 64)).astype(np.float32)
    ids, dist = idx.batch_search_ivf_mode(q, 1, 100, 16, 0, "pq")
    assert (ids[0] != 0xFFFFFFFF).sum() >= 90
    assert np.all(dist[0, :-1] <= dist[0, 1:])
    dq = torch.from_numpy(x[:4]).cuda()
    h_ids, h_d = idx.batch_search_ivf_mode(x[:4], 4, 10, 8, 0, "pq")
    d_ids, d_d = idx.batch_search_ivf_device_ptr(dq, 4, 10, 8, 0, "pq")
    assert np.array_equal(h_ids, d_ids) and np.allclose(h_d, d_d, atol=1e-4)


def test_metrics_and_argument_errors(cuda):
    from fvgb300._lib import FvError

    x = gen_clustered(300, 32, 4, 7)
    idx = make_index(x, 4, 4)
    idx.batch_search_flat(x[:10], 10, 5)
    m = idx.metrics()
    assert m["count"] >= 10 and m["p50_us"] > 0 and m["qps"] > 0
    with pytest.raises(FvError):
        idx.batch_search_flat(x[:1], 1, 300)  # top_k > 256 (index.rs:322)
    with pytest.raises(ValueError):
        idx.build(np.zeros((0, 32), np.float32))  # test_bindings.py:79-86


def test_build_device_orders_after_the_producer(cuda):
    """Rows still being produced on the caller's stream when build_device is
    called are copied only once they are complete."""
    torch = cuda
    from fvgb300.index import BUILD_FP16, GpuVectorIndex, IndexConfig

    g = torch.Generator(device="cuda")
    g.manual_seed(3)
    x = torch.randn((2_000_000, 64), generator=g, device="cuda")
    for _ in range(20):  # more queued work on the producer's stream
        x = x * 1.0001 + 0.001
    idx = GpuVectorIndex(IndexConfig(dim=64, nlist=0, build_flags=BUILD_FP16))
    idx.build_device(x)
    q = x[[123, 1_999_999]].cpu().numpy()
    ids, _ = idx.batch_search_flat(q, 2, 1)
    assert ids[:, 0].tolist() == [123, 1_999_999]
