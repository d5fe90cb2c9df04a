"""IVF-PQ / IVF-SQ8 / IVF-RaBitQ scans through the C ABI against the oracle.

Every distance of the path (coarse L2, LUT entries, ADC sums, SQ8 decode,
RaBitQ rotation, 4-bit query code and popcount estimate, warp-order rerank)
is evaluated in the reference's operation order (the RaBitQ estimate in the
fixed order both sides restate), so ids and distances must be bit-identical
to the oracle's restatement; results are ordered by (distance, id)."""
from __future__ import annotations

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def gen_clustered(n, dim, clusters, seed, sigma=0.18):
    rng = np.random.default_rng(seed)
    centers = rng.uniform(-1, 1, size=(clusters, dim)).astype(np.float32)
    return (centers[np.arange(n) % clusters] + np.float32(sigma) * rng.standard_normal((n, dim))).astype(np.float32)


MODES = ["pq", "sq8", "rabitq"]


def oracle_fn(oracle_mod, mode):
    return {"pq": oracle_mod.ivf_pq_search, "sq8": oracle_mod.ivf_sq_search,
            "rabitq": oracle_mod.ivf_rabitq_search}[mode]


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


@pytest.mark.parametrize("mode", MODES)
@pytest.mark.parametrize("rerank", [256, 512, 0, 1, 20])
def test_ivf_matches_oracle_e2e_params(cuda, oracle_mod, e2e_case, mode, rerank):
    x, t = e2e_case
    q = x[:8]
    ids, dist = run(cuda, t, x, q, mode, 10, 12, rerank)
    fn = oracle_fn(oracle_mod, mode)
    assert_same(ids, dist, fn(t, x, q, 10, 12, rerank))
    if rerank not in (0, 1):
        truth = oracle_mod.exact_knn(x, q, 10)
        assert oracle_mod.recall(ids, truth["id"]) >= 0.80


@pytest.mark.parametrize("mode", MODES)
@pytest.mark.parametrize("metric", ["ip", "cosine"])
def test_ivf_rerank_metrics(cuda, oracle_mod, e2e_case, mode, metric):
    x, t = e2e_case
    q = x[100:140] + np.float32(0.01)
    ids, dist = run(cuda, t, x, q, mode, 16, 6, 64, metric)
    fn = oracle_fn(oracle_mod, mode)
    assert_same(ids, dist, fn(t, x, q, 16, 6, 64, metric))


@pytest.mark.parametrize("mode", MODES)
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
    fn = oracle_fn(oracle_mod, mode)
    assert_same(ids, dist, fn(t, x, q, 5, 8, 64, mask=words))
    valid = ids[ids != 0xFFFFFFFF]
    assert valid.size > 0 and np.all(allowed[valid])
    ids2, dist2 = run(cuda, t, x, q, mode, 5, 8, 64, mask=words, list_major=True)
    assert np.array_equal(ids, ids2) and np.array_equal(dist, dist2)


@pytest.mark.parametrize("mode", MODES)
def test_ivf_mask_with_an_id_space_beyond_the_lists(cuda, oracle_mod, e2e_case, mode):
    """num_vectors larger than the lists' posting count (an engine whose
    slots carry remapped ids reports its id space): the list-order mask pass
    reads ids only inside the lists, and the answer is the oracle's."""
    from fvgb300.datasets import pack_bools
    from fvgb300.ivf import IvfTable

    torch = cuda
    x, t = e2e_case
    allowed = np.zeros(x.shape[0] + 5000, dtype=bool)
    allowed[5:900] = True
    words = pack_bools(allowed)
    q = x[:4]
    table = IvfTable(mode, t, vectors=x)
    table.struct.num_vectors = table.n + 5000
    res = table.search(torch.from_numpy(np.ascontiguousarray(q)).cuda(), 5, 8, 64, "l2",
                       mask=torch.from_numpy(words.view(np.int32)).cuda())
    torch.cuda.synchronize()
    ids, dist = res_np(res)
    fn = oracle_fn(oracle_mod, mode)
    assert_same(ids, dist, fn(t, x, q, 5, 8, 64, mask=words[:(x.shape[0] + 31) // 32]))
    valid = ids[ids != 0xFFFFFFFF]
    assert valid.size > 0 and np.all(allowed[valid])


def test_ivf_large_k_sorted(cuda, oracle_mod):
    """python/tests/test_bindings.py:123-138: k=100 over N=1000, d=64,
    nlist=16, m_pq=8, nprobe=16 -> sorted, >= 90% filled."""
    rng = np.random.default_rng(3)
    x = rng.standard_normal((1000, 64), dtype=np.float32)
    t = oracle_mod.build_ivf(x, nlist=16, m_pq=8, iters=10, seed=1)
    q = rng.standard_normal((3, 64), dtype=np.float32)
    for mode in MODES:
        ids, dist = run(cuda, t, x, q, mode, 100, 16, 0)
        fn = oracle_fn(oracle_mod, mode)
        assert_same(ids, dist, fn(t, x, q, 100, 16, 0))
        assert (ids[0] != 0xFFFFFFFF).sum() >= 90
        assert np.all(dist[:, :-1] <= dist[:, 1:])


@pytest.mark.parametrize("mode", MODES)
def test_ivf_wide_batch_vector_loads(cuda, oracle_mod, mode):
    """d=128, M=32 (16-byte code loads), 300 queries, 400-candidate rerank,
    list-major and id-major layouts."""
    from fvgb300 import datasets

    mix = datasets.Mixture(dim=128, components=64, sigma=20.0, center_kind="uniform255", post="int255")
    x = datasets.sample_np(mix, 30000, seed=3, stream=0)
    q = datasets.sample_np(mix, 300, seed=3, stream=1)
    t = oracle_mod.build_ivf(x, nlist=128, m_pq=32, iters=8, seed=2)
    fn = oracle_fn(oracle_mod, mode)
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


@pytest.mark.parametrize("mode", MODES)
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
    fn = oracle_fn(oracle_mod, mode)
    assert_same(ids, dist, fn(t, x, q, 20, 6, 64, mask=mask))
    assert np.all(words[ids[ids != 0xFFFFFFFF]])


@pytest.mark.parametrize("dim", [20, 64, 200, 300, 1000])
@pytest.mark.parametrize("metric", ["l2", "ip"])
def test_rabitq_padded_dims(cuda, oracle_mod, dim, metric):
    """Every row width of the RaBitQ scan: P = 32 (one word, scalar path),
    256 / 512 / 1024 (2, 4, 8 sixteen-byte words in registers), both
    layouts, masks, against the oracle."""
    from fvgb300.datasets import pack_bools

    x = gen_clustered(3000, dim, 20, 9 + dim, sigma=0.3)
    t = oracle_mod.build_ivf(x, nlist=20, m_pq=None, iters=8, seed=4)
    assert t["padded_dim"] == oracle_mod.rabitq_padded_dim(dim)
    rng = np.random.default_rng(dim)
    q = (x[rng.integers(0, 3000, 24)] + np.float32(0.05) * rng.standard_normal((24, dim))).astype(np.float32)
    mask = pack_bools(rng.random(3000) < 0.8)
    ref = oracle_mod.ivf_rabitq_search(t, x, q, 10, 5, 100, metric, mask=mask)
    for lm in (False, True):
        ids, dist = run(cuda, t, x, q, "rabitq", 10, 5, 100, metric, mask=mask, list_major=lm)
        assert_same(ids, dist, ref)
    ids, dist = run(cuda, t, x, q, "rabitq", 10, 5, 1, metric)  # estimates themselves (no rerank)
    assert_same(ids, dist, oracle_mod.ivf_rabitq_search(t, x, q, 10, 5, 1, metric))


def test_rabitq_query_on_a_centroid(cuda, oracle_mod, e2e_case):
    """A query equal to a coarse centroid has a zero rotated residual to its
    own list: range 0, every 4-bit code 0 (ivf_quant_lookup.cu:409-424)."""
    x, t = e2e_case
    q = np.ascontiguousarray(t["centroids"][:6])
    for rerank in (1, 64):
        ids, dist = run(cuda, t, x, q, "rabitq", 10, 3, rerank)
        assert_same(ids, dist, oracle_mod.ivf_rabitq_search(t, x, q, 10, 3, rerank))


@pytest.mark.parametrize("dim", [96, 300])
def test_rabitq_gpu_encoder_matches_host_encoder(cuda, oracle_mod, dim):
    """fv_build_rabitq gives the host encoder's (quant.rs:156-234) rotated
    centroids, sign bits and meta bit for bit."""
    import torch

    from fvgb300.ivf import build_rabitq

    x = gen_clustered(2000, dim, 10, 31, sigma=0.4)
    t = oracle_mod.build_ivf(x, nlist=10, m_pq=None, iters=5, seed=6)
    enc = build_rabitq(torch.from_numpy(x).cuda(), torch.from_numpy(t["centroids"]).cuda(),
                       torch.from_numpy(t["assign"].astype(np.int32)).cuda())
    torch.cuda.synchronize()
    assert enc["padded_dim"] == t["padded_dim"]
    assert np.array_equal(enc["rot_signs"].cpu().numpy(), t["rot_signs"])
    assert np.array_equal(enc["rot_centroids"].cpu().numpy().view(np.uint32), t["rot_centroids"].view(np.uint32))
    assert np.array_equal(enc["rabitq_bits"].cpu().numpy().view(np.uint32), t["rabitq_bits"])
    assert np.array_equal(enc["rabitq_meta"].cpu().numpy().view(np.uint32), t["rabitq_meta"].view(np.uint32))


@pytest.mark.parametrize("name", ["ivf_e2e", "ivf_zipf"])
@pytest.mark.parametrize("mode", MODES)
@pytest.mark.parametrize("list_major", [False, True])
def test_ivf_matches_reference_kernels(cuda, name, mode, list_major):
    """The drop-in cuda_ivf_{pq,sq,rabitq}_search_batch (reference layout:
    codes by vector id) and the list-major fv_*_ex path against the
    reference's own kernels' recorded outputs (tests/golden/ivf_*.npz, made
    by tests/golden/make_ivf_golden.py on a GB300): every case of the
    e2e_search_test.rs:231-288 parameters and of the Zipf-skewed 64-list
    input. Tolerances and the tie rule: tests/ivf_golden.py."""
    import ivf_golden

    base, queries, mask, t, cases, ref = ivf_golden.load(name)
    for ci, c in enumerate(cases):
        ids, dist = run(cuda, t, base, queries, mode, c["k"], c["nprobe"], c["rerank"], c["metric"],
                        mask=mask if c["mask"] else None, list_major=list_major)
        bad = ivf_golden.compare(mode, c, ids, dist, *ref[(mode, ci)])
        assert not bad, (ci, c, bad[:3])


def given_centroid_tables(oracle_mod, x, nlist, m_pq, seed):
    """IVF tables around `nlist` rows picked as centroids (no k-means: large
    nlist stays quick on the CPU), in the reference's layout."""
    rng = np.random.default_rng(seed)
    cent = (x[rng.choice(x.shape[0], nlist, replace=False)]
            + np.float32(0.01) * rng.standard_normal((nlist, x.shape[1]))).astype(np.float32)
    assign = oracle_mod.coarse_probe(cent, x, 1)[0][:, 0].copy()
    res = oracle_mod.residuals(x, cent, assign)
    offsets, vec_ids = oracle_mod.ivf_lists(assign, nlist)
    cb = oracle_mod.pq_train(res, m_pq, 5, seed)
    mins, scales = oracle_mod.sq8_fit(res)
    t = {"centroids": cent, "offsets": offsets, "vec_ids": vec_ids, "nlist": nlist, "codebooks": cb,
         "pq_codes": oracle_mod.pq_encode(res, cb), "sq_mins": mins, "sq_scales": scales,
         "sq_codes": oracle_mod.sq8_encode(res, mins, scales)}
    t.update(oracle_mod.rabitq_encode(x, cent, assign))
    return t


@pytest.fixture(scope="module")
def wide_nlist_case(oracle_mod):
    x = gen_clustered(40000, 96, 64, 404)
    q = gen_clustered(300, 96, 64, 405)
    return x, q, given_centroid_tables(oracle_mod, x, 2048, 12, 7)


@pytest.mark.parametrize("mode", MODES)
def test_ivf_tensor_core_coarse_probe_is_exact(cuda, oracle_mod, wide_nlist_case, mode):
    """The tensor-core coarse probe (fp16 candidates of the centred queries and
    centroids, their exact distances, a proof that no other list can enter or
    the exact scan for that query) probes exactly the lists of the exact fp32
    scan: results bit-identical to the oracle with the path automatic (2,048
    lists, 300 queries), forced, forced with every query sent to the exact
    fallback, and off."""
    from fvgb300 import scan

    x, q, t = wide_nlist_case
    ref = oracle_fn(oracle_mod, mode)(t, x, q, 10, 32, 256)
    for knob in (-1, 1, 2, 0):
        with scan.tuned(ivf_tc_coarse=knob):
            ids, dist = run(cuda, t, x, q, mode, 10, 32, 256, list_major=True)
        assert_same(ids, dist, ref)
    assert scan.device_status() == 0
