"""IVF-PQ / IVF-SQ8 scans through the C ABI against the oracle.

Every distance of the path (coarse L2, LUT entries, ADC sums, SQ8 decode,
warp-order rerank) is evaluated in the reference's operation order, so ids
and distances must be bit-identical to the oracle's restatement; results
are ordered by (distance, id)."""
from __future__ import annotations

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def gen_clustered(n, dim, clusters, seed, sigma=0.18):
    rng = np.random.default_rng(seed)
    centers = rng.uniform(-1, 1, size=(clusters, dim)).astype(np.float32)
    return (centers[np.arange(n) % clusters] + np.float32(sigma) * rng.standard_normal((n, dim))).astype(np.float32)


def res_np(res):
    r = res.cpu().numpy()
    return r[..., 0].view(np.uint32), r[..., 1].view(np.float32)


def assert_same(ids, dist, ref):
    bad = np.argwhere(ids != ref["id"])
    assert bad.size == 0, (bad[:5], ids[tuple(bad[0])], ref["id"][tuple(bad[0])])
    assert np.array_equal(dist.view(np.uint32), ref["distance"].view(np.uint32))


@pytest.fixture(scope="module")
def e2e_case(oracle_mod):
    """e2e_search_test.rs:231-288 parameters: d=96, N=1500, 12 clusters,
    nlist=24, M=12."""
    x = gen_clustered(1500, 96, 12, 202)
    t = oracle_mod.build_ivf(x, nlist=24, m_pq=12, iters=25, seed=5)
    return x, t


def run(cuda, t, x, q, mode, k, nprobe, rerank, metric="l2", mask=None, list_major=False, use_vectors=True):
    from fvgb300.ivf import IvfTable

    torch = cuda
    table = IvfTable(mode, t, vectors=x if use_vectors else None, list_major=list_major)
    qt = torch.from_numpy(np.ascontiguousarray(q)).cuda()
    m = None if mask is None else torch.from_numpy(mask.view(np.int32)).cuda()
    res = table.search(qt, k, nprobe, rerank, metric, mask=m)
    torch.cuda.synchronize()
    return res_np(res)


@pytest.mark.parametrize("mode", ["pq", "sq8"])
@pytest.mark.parametrize("rerank", [256, 512, 0, 1, 20])
def test_ivf_matches_oracle_e2e_params(cuda, oracle_mod, e2e_case, mode, rerank):
    x, t = e2e_case
    q = x[:8]
    ids, dist = run(cuda, t, x, q, mode, 10, 12, rerank)
    fn = oracle_mod.ivf_pq_search if mode == "pq" else oracle_mod.ivf_sq_search
    assert_same(ids, dist, fn(t, x, q, 10, 12, rerank))
    if rerank not in (0, 1):
        truth = oracle_mod.exact_knn(x, q, 10)
        assert oracle_mod.recall(ids, truth["id"]) >= 0.80


@pytest.mark.parametrize("mode", ["pq", "sq8"])
@pytest.mark.parametrize("metric", ["ip", "cosine"])
def test_ivf_rerank_metrics(cuda, oracle_mod, e2e_case, mode, metric):
    x, t = e2e_case
    q = x[100:140] + np.float32(0.01)
    ids, dist = run(cuda, t, x, q, mode, 16, 6, 64, metric)
    fn = oracle_mod.ivf_pq_search if mode == "pq" else oracle_mod.ivf_sq_search
    assert_same(ids, dist, fn(t, x, q, 16, 6, 64, metric))


@pytest.mark.parametrize("mode", ["pq", "sq8"])
def test_ivf_mask_and_list_major(cuda, oracle_mod, e2e_case, mode):
    """No masked-out id is returned (e2e_search_test.rs:322-433 window), and
    the list-major code layout gives the identical answer."""
    from fvgb300.datasets import pack_bools

    x, t = e2e_case
    allowed = np.zeros(x.shape[0], dtype=bool)
    allowed[10:200] = True
    words = pack_bools(allowed)
    q = x[:2]
    ids, dist = run(cuda, t, x, q, mode, 5, 8, 64, mask=words)
    fn = oracle_mod.ivf_pq_search if mode == "pq" else oracle_mod.ivf_sq_search
    assert_same(ids, dist, fn(t, x, q, 5, 8, 64, mask=words))
    valid = ids[ids != 0xFFFFFFFF]
    assert valid.size > 0 and np.all(allowed[valid])
    ids2, dist2 = run(cuda, t, x, q, mode, 5, 8, 64, mask=words, list_major=True)
    assert np.array_equal(ids, ids2) and np.array_equal(dist, dist2)


def test_ivf_large_k_sorted(cuda, oracle_mod):
    """python/tests/test_bindings.py:123-138: k=100 over N=1000, d=64,
    nlist=16, m_pq=8, nprobe=16 -> sorted, >= 90% filled."""
    rng = np.random.default_rng(3)
    x = rng.standard_normal((1000, 64), dtype=np.float32)
    t = oracle_mod.build_ivf(x, nlist=16, m_pq=8, iters=10, seed=1)
    q = rng.standard_normal((3, 64), dtype=np.float32)
    for mode in ("pq", "sq8"):
        ids, dist = run(cuda, t, x, q, mode, 100, 16, 0)
        fn = oracle_mod.ivf_pq_search if mode == "pq" else oracle_mod.ivf_sq_search
        assert_same(ids, dist, fn(t, x, q, 100, 16, 0))
        assert (ids[0] != 0xFFFFFFFF).sum() >= 90
        assert np.all(dist[:, :-1] <= dist[:, 1:])


@pytest.mark.parametrize("mode", ["pq", "sq8"])
def test_ivf_wide_batch_vector_loads(cuda, oracle_mod, mode):
    """d=128, M=32 (16-byte code loads), 300 queries, 400-candidate rerank,
    list-major and id-major layouts."""
    from fvgb300 import datasets

    mix = datasets.Mixture(dim=128, components=64, sigma=20.0, center_kind="uniform255", post="int255")
    x = datasets.sample_np(mix, 30000, seed=3, stream=0)
    q = datasets.sample_np(mix, 300, seed=3, stream=1)
    t = oracle_mod.build_ivf(x, nlist=128, m_pq=32, iters=8, seed=2)
    fn = oracle_mod.ivf_pq_search if mode == "pq" else oracle_mod.ivf_sq_search
    ref = fn(t, x, q, 10, 16, 400)
    for lm in (False, True):
        ids, dist = run(cuda, t, x, q, mode, 10, 16, 400, list_major=lm)
        assert_same(ids, dist, ref)


def test_ivf_clamps_and_noops(cuda, oracle_mod, e2e_case):
    """nprobe 0 -> 1, nprobe > nlist -> nlist, top_k > 256 -> 256, no fp32
    rows -> no rerank; zero queries is a no-op."""
    x, t = e2e_case
    q = x[:3]
    for k, nprobe, rerank in ((10, 0, 0), (10, 999, 32), (300, 24, 0)):
        ids, dist = run(cuda, t, x, q, "pq", k, nprobe, rerank)
        assert_same(ids, dist, oracle_mod.ivf_pq_search(t, x, q, k, nprobe, rerank))
    ids, dist = run(cuda, t, x, q, "pq", 10, 4, 50, use_vectors=False)
    assert_same(ids, dist, oracle_mod.ivf_pq_search(t, x, q, 10, 4, 50, use_vectors=False))
    from fvgb300 import _lib
    import ctypes as C
    from fvgb300.ivf import IvfTable

    table = IvfTable("pq", t, vectors=x)
    assert _lib.lib().cuda_ivf_pq_search_batch(C.byref(table.struct), C.c_void_p(1), 0, 10, 4, 0, 0, None,
                                               C.c_void_p(1), None) == 0
    assert _lib.lib().cuda_ivf_pq_search_batch(None, None, 1, 10, 4, 0, 0, None, None, None) == -1


@pytest.mark.parametrize("mode", ["pq", "sq8"])
@pytest.mark.parametrize("split", [0, 2, 7, 33])
def test_ivf_posting_ranges_give_the_same_answer(cuda, oracle_mod, mode, split):
    """A query's probed postings cut into G ranges (separate CTAs, merged
    shortlists) answer exactly as one CTA per query, and as the oracle; a
    skewed base puts most postings in one list, so ranges cut through it."""
    from fvgb300 import scan

    rng = np.random.default_rng(77)
    # one tight cluster of 5,000 rows (k-means leaves it in one list) and 40
    # small far-apart clusters
    big = (rng.standard_normal((1, 32)) + np.float32(0.01) * rng.standard_normal((5000, 32))).astype(np.float32)
    centers = rng.uniform(-10, 10, size=(40, 32)).astype(np.float32)
    rest = (centers[np.arange(1000) % 40] + np.float32(0.05) * rng.standard_normal((1000, 32))).astype(np.float32)
    x = np.vstack([big, rest]).astype(np.float32)
    x = x[rng.permutation(x.shape[0])]
    t = oracle_mod.build_ivf(x, nlist=16, m_pq=8, iters=10, seed=3)
    lens = np.diff(t["offsets"].astype(np.int64))
    assert lens.max() > 0.5 * x.shape[0]
    q = x[rng.integers(0, x.shape[0], 12)] + np.float32(0.001)
    words = (rng.random(x.shape[0]) < 0.7)
    from fvgb300.datasets import pack_bools

    mask = pack_bools(words)
    with scan.tuned(ivf_split=split):
        ids, dist = run(cuda, t, x, q, mode, 20, 6, 64, mask=mask, list_major=True)
    fn = oracle_mod.ivf_pq_search if mode == "pq" else oracle_mod.ivf_sq_search
    assert_same(ids, dist, fn(t, x, q, 20, 6, 64, mask=mask))
    assert np.all(words[ids[ids != 0xFFFFFFFF]])
