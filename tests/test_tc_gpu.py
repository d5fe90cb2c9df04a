"""Tensor-core flat scans (fp16 / fp8) through the C ABI.

Reduced-precision forms are assessed the way the scan path's contract states
them: the candidate ranking must agree with an fp64 evaluation of the same
quantised products, the fp32-rescored results must reach recall@k >= 0.99
against the fp64 oracle, and every reported distance must be the fp32
rescore value (bit-identical to the oracle's restatement of the reference's
warp-order distance) or, inside the k-th boundary band, the fp64 value
rounded to fp32."""
from __future__ import annotations

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def unit_mixture(n, dim, comps, sigma, seed):
    rng = np.random.default_rng(seed)
    c = rng.standard_normal((comps, dim)).astype(np.float32)
    c /= np.linalg.norm(c, axis=1, keepdims=True)
    x = c[rng.integers(0, comps, n)] + np.float32(sigma) * rng.standard_normal((n, dim), dtype=np.float32)
    x /= np.linalg.norm(x, axis=1, keepdims=True)
    return x.astype(np.float32)


def res_np(res):
    r = res.cpu().numpy()
    return r[..., 0].view(np.uint32), r[..., 1].view(np.float32)


def check_rescored(oracle_mod, base, queries, ids, dist, metric, k):
    """recall vs fp64 and exactness of every reported distance."""
    truth, _ = oracle_mod.bruteforce_f64(base, queries, k, metric)
    rec = oracle_mod.recall(ids, truth)
    bad = 0
    for qi in range(queries.shape[0]):
        for r in range(k):
            i = ids[qi, r]
            if i == 0xFFFFFFFF:
                continue
            w = np.float32(oracle_mod.warp_distance(queries[qi], base[i], metric))
            if dist[qi, r] != w:
                x = base[i].astype(np.float64)
                q = queries[qi].astype(np.float64)
                if metric == "l2":
                    d64 = np.sum((q - x) ** 2)
                elif metric == "ip":
                    d64 = -np.dot(q, x)
                else:
                    d64 = 1 - np.dot(q, x) / (np.linalg.norm(q) * np.linalg.norm(x))
                if abs(np.float32(d64) - dist[qi, r]) > 1e-6 * max(1.0, abs(d64)):
                    bad += 1
    assert bad == 0, f"{bad} reported distances are neither the fp32 rescore nor the fp64 band value"
    # sorted ascending per query
    assert np.all(dist[:, :-1] <= dist[:, 1:])
    return rec


def test_encode_fp16_matches_oracle(cuda, oracle_mod):
    from fvgb300 import scan

    torch = cuda
    rng = np.random.default_rng(0)
    x = (rng.standard_normal((777, 70)) * np.logspace(-6, 4, 70)).astype(np.float32)
    x[0, :5] = [1.0 + 2 ** -11, 65519.0, 70000.0, 1e-9, -0.0]
    codes, norms = scan.encode_fp16(torch.from_numpy(x).cuda())
    ref_codes, ref_norms = oracle_mod.encode_fp16_padded(x)
    assert np.array_equal(codes.cpu().numpy().view(np.uint16), ref_codes)
    assert np.array_equal(norms.cpu().numpy().view(np.uint32), ref_norms.view(np.uint32))


def fp8_table_exponent(max_norm):
    """Smallest b with max_norm <= 896 * 4^b (0 for an all-zero table)."""
    if not max_norm > 0:
        return 0
    b = -62
    while b < 62 and np.ldexp(np.float32(896.0), 2 * b) < max_norm:
        b += 1
    return b


def fp8_query_exponent(q, b):
    """Smallest a with max|q| <= 448 * 2^a, at least b - 8."""
    amax = np.float32(np.abs(q).max())
    a = b - 8
    if amax > 0:
        ap = -200
        while np.ldexp(np.float32(448.0), ap) < amax:
            ap += 1
        a = max(a, ap)
    return a


def e4m3(torch, x):
    return torch.from_numpy(np.ascontiguousarray(x, dtype=np.float32)).cuda().to(torch.float8_e4m3fn)


def test_encode_fp8(cuda):
    """One power-of-two scale for the table, e4m3 codes at that scale, three
    norm digits summing to ||x||^2 / (2 s^2), zero padding."""
    from fvgb300 import scan

    torch = cuda
    rng = np.random.default_rng(1)
    x = rng.standard_normal((500, 96)).astype(np.float32)
    x[3] = 0.0
    x[7] *= np.float32(1e-3)
    x[8] *= np.float32(40.0)
    codes, scales, norms = scan.encode_fp8(torch.from_numpy(x).cuda())
    assert codes.shape == (500, scan.fp8_padded_dim(96)) == (500, 112)
    nrm = norms.cpu().numpy()
    assert np.allclose(nrm, (x.astype(np.float64) ** 2).sum(1), rtol=1e-6)
    b = fp8_table_exponent(nrm.max())
    assert np.ldexp(np.float32(896.0), 2 * b - 2) < nrm.max() <= np.ldexp(np.float32(896.0), 2 * b)
    assert np.all(scales.cpu().numpy() == np.ldexp(np.float32(1.0), b))
    ref = e4m3(torch, np.ldexp(x, -b)).view(torch.uint8)
    assert torch.equal(codes[:, :96], ref)
    r = np.ldexp(nrm, -1 - 2 * b).astype(np.float32)
    want = r.copy()
    for i in range(3):
        c = e4m3(torch, r)
        assert torch.equal(codes[:, 96 + i], c.view(torch.uint8))
        r = (r - c.float().cpu().numpy()).astype(np.float32)
    assert np.all(np.abs(r) <= want * 2.0 ** -11 + 2.0 ** -10)
    assert torch.all(codes[:, 99:] == 0)
    assert torch.all(codes[3] == 0)
    # the all-zero table: scale 1, zero codes
    z_codes, z_scales, _ = scan.encode_fp8(torch.zeros((4, 20), device="cuda"))
    assert torch.all(z_codes == 0) and torch.all(z_scales == 1.0)


def test_encode_fp8_per_vector(cuda):
    """The per-vector layout: scale max|x|/448 per row (1 for a zero row),
    codes e4m3(x / scale), zero padding, compensated ||x||^2."""
    from fvgb300 import scan

    torch = cuda
    rng = np.random.default_rng(1)
    x = rng.standard_normal((500, 96)).astype(np.float32)
    x[3] = 0.0
    codes, scales, norms = scan.encode_fp8_per_vector(torch.from_numpy(x).cuda())
    amax = np.abs(x).max(axis=1)
    exp_scale = np.where(amax > 0, amax / np.float32(448.0), 1.0).astype(np.float32)
    assert np.array_equal(scales.cpu().numpy(), exp_scale)
    ref = (torch.from_numpy(x).cuda() / scales[:, None]).to(torch.float8_e4m3fn).view(torch.uint8)
    assert torch.equal(codes[:, :96], ref)
    assert np.allclose(norms.cpu().numpy(), (x.astype(np.float64) ** 2).sum(1), rtol=1e-6)


@pytest.mark.parametrize("metric", ["ip", "l2", "cosine"])
@pytest.mark.parametrize("n,dim,nq,k", [(20000, 96, 200, 10), (5003, 70, 129, 16), (257, 253, 64, 10)])
def test_fp8_per_vector_ranking_without_rescore(cuda, metric, n, dim, nq, k):
    """Per-vector-scale table, no fp32 copy: results are the top-k of the fp8
    tensor-core distance with each row's scale and norm applied per value,
    checked against an fp64 evaluation of the same e4m3 products."""
    from fvgb300 import scan

    torch = cuda
    rng = np.random.default_rng(n + dim + 1)
    base = (rng.standard_normal((n, dim)) + rng.standard_normal((32, dim))[rng.integers(0, 32, n)]).astype(np.float32)
    base *= rng.uniform(0.5, 2.0, (n, 1)).astype(np.float32)
    queries = (rng.standard_normal((nq, dim)) * 1.3).astype(np.float32)
    table = scan.Fp8Table(torch.from_numpy(base).cuda(), keep_fp32=False, per_vector=True)
    res = scan.fp8_search(table, torch.from_numpy(queries).cuda(), k, metric, opts=scan.options(boundary_fp64=0))
    torch.cuda.synchronize()
    ids, dist = res_np(res)
    xs = table.scales.cpu().numpy().astype(np.float64)
    x8 = table.fp8.view(torch.float8_e4m3fn).double().cpu().numpy()[:, :dim]
    xn = table.norms.cpu().numpy().astype(np.float64)
    qn = (queries.astype(np.float64) ** 2).sum(1)
    amax = np.abs(queries).max(axis=1)
    qs = np.where(amax > 0, amax / np.float32(448.0), 1.0).astype(np.float32)
    q8 = (torch.from_numpy(queries).cuda() / torch.from_numpy(qs).cuda()[:, None]).to(torch.float8_e4m3fn)
    q8 = q8.double().cpu().numpy()
    dots = (q8 @ x8.T) * qs.astype(np.float64)[:, None] * xs[None, :]
    if metric == "ip":
        d64 = -dots
    elif metric == "l2":
        d64 = np.maximum(0, qn[:, None] + xn[None, :] - 2 * dots)
    else:
        d64 = 1 - dots / (np.sqrt(qn[:, None] * xn[None, :]) + 1e-8)
    order = np.argsort(d64, axis=1, kind="stable")[:, :k]
    hit = np.mean([len(set(ids[i]) & set(order[i])) / k for i in range(nq)])
    assert hit >= 0.995, hit
    got = np.take_along_axis(d64, ids.astype(np.int64), axis=1)
    scale = np.abs(d64).max(axis=1, keepdims=True)
    assert np.all(np.abs(dist - got) <= 2e-5 * np.maximum(scale, 1.0)), np.abs(dist - got).max()
    assert np.all(dist[:, :-1] <= dist[:, 1:])
    assert scan.device_status() == 0


@pytest.mark.parametrize("metric", ["ip", "l2", "cosine"])
@pytest.mark.parametrize("n,dim,nq,k", [(20000, 96, 200, 10), (5003, 70, 129, 16), (1000, 128, 1, 5),
                                        (257, 253, 64, 10)])
def test_fp8_scan_ranking_without_rescore(cuda, metric, n, dim, nq, k):
    """No fp32 copy: results are the top-k of the fp8 tensor-core distance
    (L2 through the norm digits). Checked against an fp64 evaluation of the
    same e4m3 products."""
    from fvgb300 import scan

    torch = cuda
    rng = np.random.default_rng(n + dim)
    base = (rng.standard_normal((n, dim)) + rng.standard_normal((32, dim))[rng.integers(0, 32, n)]).astype(np.float32)
    base *= rng.uniform(0.5, 2.0, (n, 1)).astype(np.float32)
    queries = (rng.standard_normal((nq, dim)) * 1.3).astype(np.float32)
    table = scan.Fp8Table(torch.from_numpy(base).cuda(), keep_fp32=False)
    res = scan.fp8_search(table, torch.from_numpy(queries).cuda(), k, metric, opts=scan.options(boundary_fp64=0))
    torch.cuda.synchronize()
    ids, dist = res_np(res)
    s = np.float64(table.scales[0].item())
    b = int(np.log2(s))
    x8 = table.fp8.view(torch.float8_e4m3fn).double().cpu().numpy()
    xn = table.norms.cpu().numpy().astype(np.float64)
    qn = (queries.astype(np.float64) ** 2).sum(1)
    a = np.array([fp8_query_exponent(q, b) for q in queries])
    q8 = np.stack([e4m3(torch, np.ldexp(q, -int(ai))).double().cpu().numpy() for q, ai in zip(queries, a)])
    dots = q8 @ x8[:, :dim].T
    qs = np.ldexp(1.0, a)
    if metric == "l2":
        c = np.where(b - a >= -9, -np.ldexp(1.0, b - a), 0.0)
        acc = dots + c[:, None] * x8[:, dim:dim + 3].sum(1)[None, :]
        d64 = np.maximum(0, qn[:, None] - 2 * (qs * s)[:, None] * acc)
    elif metric == "ip":
        d64 = -(qs * s)[:, None] * dots
    else:
        d64 = 1 - (qs * s)[:, None] * dots / (np.sqrt(qn[:, None] * xn[None, :]) + 1e-8)
    order = np.argsort(d64, axis=1, kind="stable")[:, :k]
    hit = np.mean([len(set(ids[i]) & set(order[i])) / k for i in range(nq)])
    assert hit >= 0.995, hit
    got = np.take_along_axis(d64, ids.astype(np.int64), axis=1)
    scale = np.abs(d64).max(axis=1, keepdims=True)
    assert np.all(np.abs(dist - got) <= 2e-5 * np.maximum(scale, 1.0)), np.abs(dist - got).max()
    assert np.all(dist[:, :-1] <= dist[:, 1:])
    assert scan.device_status() == 0


@pytest.mark.parametrize("metric", ["ip", "l2", "cosine"])
@pytest.mark.parametrize("n,dim,nq,k", [(30000, 768, 200, 10), (5003, 70, 129, 16), (1000, 128, 1, 5),
                                        (257, 64, 64, 10)])
def test_fp16_scan_ranking_without_rescore(cuda, metric, n, dim, nq, k):
    """No fp32 copy: results are the top-k of the fp16 tensor-core distance.
    Checked against an fp64 evaluation of the same fp16 products."""
    from fvgb300 import scan

    torch = cuda
    base = unit_mixture(n, dim, 64, 0.4, n + dim)
    queries = unit_mixture(nq, dim, 64, 0.4, 7 + nq)
    bt = torch.from_numpy(base).cuda()
    table = scan.Fp16Table(bt, keep_fp32=False)
    res = scan.fp16_search(table, torch.from_numpy(queries).cuda(), k, metric, opts=scan.options(boundary_fp64=0))
    torch.cuda.synchronize()
    ids, dist = res_np(res)
    x16 = table.fp16.cpu().numpy().view(np.float16).astype(np.float64)[:, :dim]
    q16 = queries.astype(np.float16).astype(np.float64)
    dots = q16 @ x16.T
    xn = table.norms.cpu().numpy().astype(np.float64)
    qn = (queries.astype(np.float64) ** 2).sum(1)
    if metric == "ip":
        d64 = -dots
    elif metric == "l2":
        d64 = np.maximum(0, qn[:, None] + xn[None, :] - 2 * dots)
    else:
        d64 = 1 - dots / (np.sqrt(qn[:, None] * xn[None, :]) + 1e-8)
    order = np.argsort(d64, axis=1, kind="stable")[:, :k]
    hit = np.mean([len(set(ids[i]) & set(order[i])) / k for i in range(nq)])
    assert hit >= 0.995, hit
    got = np.take_along_axis(d64, ids.astype(np.int64), axis=1)
    assert np.allclose(dist, got, rtol=2e-5, atol=2e-5)
    assert np.all(dist[:, :-1] <= dist[:, 1:])
    assert scan.device_status() == 0


@pytest.mark.parametrize("metric", ["ip", "l2"])
@pytest.mark.parametrize("k", [10, 100])
def test_fp16_rescored_recall(cuda, oracle_mod, metric, k):
    from fvgb300 import scan

    torch = cuda
    base = unit_mixture(40000, 768, 256, 0.3, 11)
    queries = unit_mixture(64, 768, 256, 0.3, 12)
    table = scan.Fp16Table(torch.from_numpy(base).cuda())
    res = scan.fp16_search(table, torch.from_numpy(queries).cuda(), k, metric)
    torch.cuda.synchronize()
    ids, dist = res_np(res)
    rec = check_rescored(oracle_mod, base, queries, ids, dist, metric, k)
    assert rec >= 0.99, rec
    assert scan.device_status() == 0


def test_fp16_masked_and_dropin(cuda, oracle_mod):
    """Bernoulli(0.5) slot mask; no masked id comes back; the drop-in entry
    point gives the same answer as the extension with default options."""
    from fvgb300 import scan
    from fvgb300.datasets import bernoulli_mask_words, unpack_words

    torch = cuda
    base = unit_mixture(20000, 256, 128, 0.3, 21)
    queries = unit_mixture(100, 256, 128, 0.3, 22)
    words = bernoulli_mask_words(base.shape[0], 0.5, 1)
    allowed = unpack_words(words, base.shape[0])
    table = scan.Fp16Table(torch.from_numpy(base).cuda())
    m = torch.from_numpy(words.view(np.int32)).cuda()
    q = torch.from_numpy(queries).cuda()
    a = scan.fp16_search(table, q, 10, "ip", mask=m)
    b = scan.fp16_search(table, q, 10, "ip", mask=m, dropin=True)
    torch.cuda.synchronize()
    ids, dist = res_np(a)
    assert torch.equal(a, b)
    assert np.all(allowed[ids])
    truth, _ = oracle_mod.bruteforce_f64(base, queries, 10, "ip", mask=words)
    assert oracle_mod.recall(ids, truth) >= 0.99


@pytest.mark.parametrize("splits", [1, 2, 7, 0])
def test_fp16_split_invariance(cuda, splits):
    """The answer does not depend on how the base range is split over CTAs."""
    from fvgb300 import scan

    torch = cuda
    base = unit_mixture(9000, 128, 32, 0.3, 31)
    queries = unit_mixture(300, 128, 32, 0.3, 32)
    table = scan.Fp16Table(torch.from_numpy(base).cuda())
    q = torch.from_numpy(queries).cuda()
    ref = scan.fp16_search(table, q, 16, "l2", opts=scan.options(splits=1))
    got = scan.fp16_search(table, q, 16, "l2", opts=scan.options(splits=splits))
    torch.cuda.synchronize()
    assert torch.equal(ref, got)


def gen_clustered(n, dim, clusters, seed):
    rng = np.random.default_rng(seed)
    centers = rng.uniform(-1, 1, size=(clusters, dim)).astype(np.float32)
    return (centers[np.arange(n) % clusters] + np.float32(0.18) * rng.standard_normal((n, dim))).astype(np.float32)


@pytest.mark.parametrize("metric", ["l2", "cosine"])
def test_fp16_self_query(cuda, metric):
    """e2e_search_test.rs:291-319: gen_clustered(512, 64, 8, 303), the first
    4 rows as queries; the nearest neighbour of row 0 is row 0."""
    from fvgb300 import scan

    torch = cuda
    x = gen_clustered(512, 64, 8, 303)
    if metric == "cosine":  # the engine normalises for cosine (index.rs:338-345)
        x /= np.linalg.norm(x, axis=1, keepdims=True)
    table = scan.Fp16Table(torch.from_numpy(x).cuda())
    res = scan.fp16_search(table, torch.from_numpy(x[:4]).cuda(), 10, metric, dropin=True)
    ids, _ = res_np(res)
    assert ids[0, 0] == 0
    assert np.array_equal(ids[:, 0], [0, 1, 2, 3])


def test_fp16_filter_window(cuda):
    """python/tests/test_bindings.py:142-169: mask = ids in [10, 200); every
    returned id lies in the window."""
    from fvgb300 import scan
    from fvgb300.datasets import pack_bools

    torch = cuda
    rng = np.random.default_rng(7)
    data = rng.standard_normal((400, 64)).astype(np.float32)
    mask = np.zeros(400, dtype=bool)
    mask[10:200] = True
    table = scan.Fp16Table(torch.from_numpy(data).cuda())
    m = torch.from_numpy(pack_bools(mask).view(np.int32)).cuda()
    res = scan.fp16_search(table, torch.from_numpy(data[:2]).cuda(), 5, "l2", mask=m, dropin=True)
    ids, _ = res_np(res)
    valid = ids[ids != 0xFFFFFFFF]
    assert valid.size > 0 and np.all((valid >= 10) & (valid < 200))


def test_fp16_tiny_and_empty(cuda):
    from fvgb300 import scan

    torch = cuda
    x = torch.randn(3, 32, device="cuda")
    table = scan.Fp16Table(x)
    res = scan.fp16_search(table, x[:2].contiguous(), 8, "l2")
    ids, dist = res_np(res)
    assert np.all(ids[:, 3:] == 0xFFFFFFFF) and np.all(dist[:, 3:] == np.float32(1e30))
    assert sorted(ids[0, :3].tolist()) == [0, 1, 2]
    empty = scan.Fp16Table(torch.zeros((0, 32), device="cuda"))
    ids, dist = res_np(scan.fp16_search(empty, x[:2].contiguous(), 4, "ip"))
    assert np.all(ids == 0xFFFFFFFF)
    assert scan.device_status() == 0


@pytest.mark.parametrize("per_vector", [False, True])
@pytest.mark.parametrize("k", [10, 100])
def test_fp8_rescored_recall(cuda, oracle_mod, k, per_vector):
    """fp8 E4M3 (table scale + norm digits, or per-vector scales), fp32
    rescore, fp64 boundary band, on data shaped like the 10M x 96 workload
    (N(0,1) component means, sigma 0.5), scaled down."""
    from fvgb300 import datasets, scan

    torch = cuda
    base = datasets.sample_np(datasets.FP8_L2, 60000, seed=2, stream=0)
    queries = datasets.sample_np(datasets.FP8_L2, 96, seed=2, stream=1)
    table = scan.Fp8Table(torch.from_numpy(base).cuda(), per_vector=per_vector)
    res = scan.fp8_search(table, torch.from_numpy(queries).cuda(), k, "l2")
    torch.cuda.synchronize()
    ids, dist = res_np(res)
    rec = check_rescored(oracle_mod, base, queries, ids, dist, "l2", k)
    assert rec >= 0.99, rec
    assert scan.device_status() == 0


def test_fp8_extreme_query_scales(cuda, oracle_mod):
    """Queries 2 x 10^5 times longer than the rows: the norm-digit factor
    -2^(b-a) falls below e4m3's range and is dropped, the rows' norms then
    weighing little against the dot. Each query is a scaled row, whose own
    row must come first (the gap to any other row is 4 x 10^5 (1 - cos),
    far above fp32's resolution at ||q||^2 = 4e10). Queries 10^4 times shorter:
    the query scale is held at 2^(b - 8) and small codes lose precision; the
    rescored distances stay exact. A zero query returns rows; an all-zero
    table ties every row at ||q||^2 (lower slots first)."""
    from fvgb300 import scan

    torch = cuda
    base = unit_mixture(20000, 96, 64, 0.4, 21)
    table = scan.Fp8Table(torch.from_numpy(base).cuda())
    src = np.random.default_rng(23).choice(20000, 32, replace=False)
    big = (base[src] * np.float32(2e5)).astype(np.float32)
    ids, dist = res_np(scan.fp8_search(table, torch.from_numpy(big).cuda(), 1, "l2"))
    torch.cuda.synchronize()
    assert np.array_equal(ids[:, 0], src.astype(np.uint32))
    small = (unit_mixture(32, 96, 64, 0.4, 22) * np.float32(1e-4)).astype(np.float32)
    small[0] = 0.0
    ids, dist = res_np(scan.fp8_search(table, torch.from_numpy(small).cuda(), 10, "l2"))
    torch.cuda.synchronize()
    rec = check_rescored(oracle_mod, base, small, ids, dist, "l2", 10)
    assert rec >= 0.9, rec
    assert np.all(ids[0] != 0xFFFFFFFF)
    zero = scan.Fp8Table(torch.zeros((300, 40), device="cuda"))
    q = torch.from_numpy(np.full((2, 40), 0.5, np.float32)).cuda()
    ids, dist = res_np(scan.fp8_search(zero, q, 5, "l2"))
    torch.cuda.synchronize()
    assert np.array_equal(ids, np.tile(np.arange(5, dtype=np.uint32), (2, 1)))
    assert np.all(dist == np.float32(10.0))
    assert scan.device_status() == 0


@pytest.mark.parametrize("fp8", [False, True])
def test_sampled_prepass_gives_the_unbounded_answer(cuda, oracle_mod, fp8):
    """k = 100 (a 400-entry shortlist, above the 64-entry range heap): the
    scan bounded by the sampled pre-pass returns exactly what the unbounded
    scan returns, also when the bound is made too tight on purpose (stride
    64, margin 1: many queries fall back to the device-side re-scan)."""
    from fvgb300 import scan

    torch = cuda
    base = unit_mixture(300_000, 96, 512, 0.5, 21)
    queries = unit_mixture(300, 96, 512, 0.5, 22)
    t = (scan.Fp8Table if fp8 else scan.Fp16Table)(torch.from_numpy(base).cuda())
    q = torch.from_numpy(queries).cuda()
    search = scan.fp8_search if fp8 else scan.fp16_search
    with scan.tuned(tc_prepass=0):
        ref = res_np(search(t, q, 100, "l2"))
    for knobs in ({"tc_prepass": 1}, {"tc_prepass": 1, "tc_prepass_stride": 64, "tc_prepass_margin": 1}):
        with scan.tuned(**knobs):
            got = res_np(search(t, q, 100, "l2"))
        assert np.array_equal(got[0], ref[0]) and np.array_equal(got[1], ref[1]), knobs
    assert scan.device_status() == 0
    rec = check_rescored(oracle_mod, base, queries[:40], ref[0][:40], ref[1][:40], "l2", 100)
    assert rec >= 0.99



@pytest.mark.parametrize("fp8", [False, True])
@pytest.mark.parametrize("n,dim,nq,k", [(70_001, 768, 300, 10), (20_000, 384, 129, 100), (5_000, 200, 1, 16)])
def test_cta_pair_scan_matches_single_cta(cuda, fp8, n, dim, nq, k):
    """The cta_group::2 pair variant (two SMs per 256-row tile) returns
    exactly what the one-SM kernel returns: odd query-block counts, partial
    last tiles, the pre-pass path (k = 100) and a single query."""
    from fvgb300 import scan

    torch = cuda
    base = unit_mixture(n, dim, 128, 0.4, n + dim)
    queries = unit_mixture(nq, dim, 128, 0.4, nq + 1)
    t = (scan.Fp8Table if fp8 else scan.Fp16Table)(torch.from_numpy(base).cuda())
    q = torch.from_numpy(queries).cuda()
    search = scan.fp8_search if fp8 else scan.fp16_search
    with scan.tuned(tc_pair=0):
        ref = res_np(search(t, q, k, "l2"))
    with scan.tuned(tc_pair=1, tc_prepass=1 if k == 100 else -1):
        got = res_np(search(t, q, k, "l2"))
    assert scan.device_status() == 0
    assert np.array_equal(got[0], ref[0]) and np.array_equal(got[1], ref[1])


@pytest.mark.parametrize("metric", ["l2", "ip"])
@pytest.mark.parametrize(
    "n,dim,nq,k,prepass,masked",
    [(100_001, 96, 300, 100, -1, False), (60_000, 96, 257, 100, 1, False), (40_000, 112, 129, 64, 1, True),
     (70_000, 70, 200, 100, 0, True), (3_000, 96, 1, 16, -1, False)],
)
def test_fp8_four_group_epilogue_matches_two_groups(cuda, metric, n, dim, nq, k, prepass, masked):
    """Table-scale fp8 rows of one K block: four epilogue groups (16 warps,
    interleaved 32-column chunks, heaps of <= 32 keys, more ranges) give the
    same answers as two groups bit for bit -- partial last tiles, odd query
    blocks, the sampled pre-pass on and off, a packed mask, a single query."""
    from fvgb300 import datasets, scan

    torch = cuda
    base = unit_mixture(n, dim, 256, 0.4, n + dim)
    queries = unit_mixture(nq, dim, 256, 0.4, nq + 5)
    t = scan.Fp8Table(torch.from_numpy(base).cuda())
    assert t.pd <= 128
    q = torch.from_numpy(queries).cuda()
    mask = torch.from_numpy(datasets.bernoulli_mask_words(n, 0.5, 11).view(np.int32)).cuda() if masked else None
    with scan.tuned(tc_groups=2, tc_prepass=prepass):
        ref = res_np(scan.fp8_search(t, q, k, metric, mask=mask))
    with scan.tuned(tc_groups=4, tc_prepass=prepass):
        got = res_np(scan.fp8_search(t, q, k, metric, mask=mask))
    assert scan.device_status() == 0
    assert np.array_equal(got[0], ref[0]) and np.array_equal(got[1], ref[1])


def test_scan_wait_timeout_is_reported_and_the_next_call_is_exact(cuda):
    """A pipeline wait that runs out ends the scan early without faulting: a
    test-only 1 ns limit on the tensor-core scan's waits (its tile copies
    cannot land that fast) makes the kernel abort, drain its copies in
    flight, free its accumulators and return; the device status word reports
    the timeout, the context stays usable, and the next call on the same
    stream, with the normal limit, returns exactly the answer of a call
    before it. One-CTA scans (short rows: no CTA pairs)."""
    from fvgb300 import scan

    torch = cuda
    x = unit_mixture(20000, 64, 32, 0.3, 21)
    q = unit_mixture(256, 64, 32, 0.3, 22)
    table = scan.Fp16Table(torch.from_numpy(x).cuda())
    qt = torch.from_numpy(q).cuda()
    scan.device_status()  # read and clear
    with scan.tuned(tc_pair=0):
        ref = scan.fp16_search(table, qt, 10, "ip", dropin=True).clone()
        torch.cuda.synchronize()
        assert scan.device_status() == 0
        with scan.tuned(tc_wait_limit_ns=1):
            scan.fp16_search(table, qt, 10, "ip", dropin=True)
            torch.cuda.synchronize()
        assert scan.device_status() & 1  # the timeout bit
        again = scan.fp16_search(table, qt, 10, "ip", dropin=True)
        torch.cuda.synchronize()
        assert scan.device_status() == 0
    assert torch.equal(ref, again)
