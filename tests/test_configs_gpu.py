"""Parity at the benchmark configurations' shapes (GPU, through the C ABI).

* exact flat L2, 100,000 x 128 integer-valued rows (1,024 components,
  centres U[0,255], sigma 20), 1,000 queries, k = 10: ids and distance bits
  equal to the oracle's restatement of the reference's exact search
  (metrics.rs:103-135, ties to the lower id);
* fp16 tensor-core inner product with fp32 rescore, d = 768 unit vectors
  (4,096 components, sigma 0.3), 200,000 rows, 1,024 queries, k = 10 and
  100, a Bernoulli(0.5) mask: recall@k >= 0.99 against an fp64 evaluation
  and every reported distance the fp32 warp-order rescore (or, in the k-th
  boundary band, the fp64 value rounded to fp32);
* fp8 e4m3 L2 with fp32 rescore, 1,000,000 x 96 rows (16,384 components,
  N(0,1) means, sigma 0.5), 1,000 queries, k = 100, both fp8 layouts (table
  scale with norm digits; per-vector max|x|/448 scales): recall@10 and
  recall@100 >= 0.99 against fp64, rescored distances as above;
* IVF-PQ, 1,000,000 x 128 integer-valued rows in 4,096 lists whose sizes
  follow Zipf(1.1) (floor 64), m_pq 32, nprobe 32, rerank 400, a 10% mask,
  200 queries: the drop-in's ids and distances bit-identical to the oracle's
  IVF-PQ restatement over the same (GPU-built) tables, recall reported.
"""
from __future__ import annotations

import dataclasses

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def res_np(res):
    r = res.cpu().numpy()
    return r[..., 0].view(np.uint32), r[..., 1].view(np.float32)


def fp64_truth(torch, base, queries, k, metric, allowed=None, chunk=250_000):
    """Exact top-k ids by an fp64 evaluation on the device."""
    q = queries.double()
    best_d = best_i = None
    for c in range(0, base.shape[0], chunk):
        x = base[c:c + chunk].double()
        d = ((q * q).sum(1, keepdim=True) + (x * x).sum(1)[None, :] - 2.0 * (q @ x.T)) if metric == "l2" \
            else -(q @ x.T)
        if allowed is not None:
            d = d.masked_fill(~allowed[None, c:c + chunk], float("inf"))
        tv, ti = torch.topk(d, min(k, d.shape[1]), dim=1, largest=False)
        ti = ti + c
        if best_d is None:
            best_d, best_i = tv, ti
        else:
            best_d, o = torch.topk(torch.cat([best_d, tv], 1), k, dim=1, largest=False)
            best_i = torch.cat([best_i, ti], 1).gather(1, o)
    return best_i.cpu().numpy()


def recall(ids, truth):
    k = truth.shape[1]
    return sum(len(set(ids[i, :k].tolist()) & set(truth[i].tolist())) for i in range(truth.shape[0])) / truth.size


def check_distances(oracle_mod, base_np, q_np, ids, dist, metric, rows):
    """Every reported distance is the oracle's fp32 warp-order distance or,
    inside the boundary band, the fp64 value rounded to fp32."""
    bad = 0
    for qi in rows:
        for r in range(ids.shape[1]):
            i = ids[qi, r]
            if i == 0xFFFFFFFF:
                continue
            w = np.float32(oracle_mod.warp_distance(q_np[qi], base_np[i], metric))
            if dist[qi, r] != w:
                x, q = base_np[i].astype(np.float64), q_np[qi].astype(np.float64)
                d64 = np.sum((q - x) ** 2) if metric == "l2" else -np.dot(q, x)
                if abs(np.float32(d64) - dist[qi, r]) > 1e-6 * max(1.0, abs(d64)):
                    bad += 1
    assert bad == 0, f"{bad} distances are neither the fp32 rescore nor the fp64 band value"
    assert np.all(dist[:, :-1] <= dist[:, 1:])


def test_exact_flat_l2_100k_x_128(cuda, oracle_mod):
    from fvgb300 import datasets, scan

    torch = cuda
    base = datasets.sample_np(datasets.FLAT_L2_INT, 100_000, seed=0, stream=0)
    queries = datasets.sample_np(datasets.FLAT_L2_INT, 1000, seed=0, stream=1)
    res = scan.flat_scan(torch.from_numpy(base).cuda(), torch.from_numpy(queries).cuda(), 10, "l2")
    torch.cuda.synchronize()
    ids, dist = res_np(res)
    ref = oracle_mod.exact_knn(base, queries, 10, "l2")
    assert np.array_equal(ids, ref["id"])
    assert np.array_equal(dist.view(np.uint32), ref["distance"].view(np.uint32))


@pytest.fixture(scope="module")
def fp16_ip_200k(cuda):
    from fvgb300 import datasets

    torch = cuda
    base = datasets.sample_torch(datasets.FP16_IP_UNIT, 200_000, seed=1, stream=0)
    queries = datasets.sample_torch(datasets.FP16_IP_UNIT, 1024, seed=1, stream=1)
    words = datasets.bernoulli_mask_words(200_000, 0.5, seed=1)
    return base, queries, words


@pytest.mark.parametrize("k", [10, 100])
def test_fp16_ip_768_1024_queries_masked(cuda, oracle_mod, fp16_ip_200k, k):
    from fvgb300 import datasets, scan

    torch = cuda
    base, queries, words = fp16_ip_200k
    mask = torch.from_numpy(words.view(np.int32)).cuda()
    table = scan.Fp16Table(base)
    res = scan.fp16_search(table, queries, k, "ip", mask=mask, dropin=True)
    torch.cuda.synchronize()
    ids, dist = res_np(res)
    allowed = torch.from_numpy(datasets.unpack_words(words, base.shape[0])).cuda()
    truth = fp64_truth(torch, base, queries, k, "ip", allowed=allowed)
    assert recall(ids, truth) >= 0.99
    assert datasets.unpack_words(words, base.shape[0])[ids.astype(np.int64)].all()
    check_distances(oracle_mod, base.cpu().numpy(), queries.cpu().numpy(), ids, dist, "ip", range(0, 1024, 8))


@pytest.mark.parametrize("per_vector", [False, True])
def test_fp8_l2_1m_x_96_k100(cuda, oracle_mod, per_vector):
    from fvgb300 import datasets, scan

    torch = cuda
    base = datasets.sample_torch(datasets.FP8_L2, 1_000_000, seed=2, stream=0)
    queries = datasets.sample_torch(datasets.FP8_L2, 1000, seed=2, stream=1)
    table = scan.Fp8Table(base, per_vector=per_vector)
    res = scan.fp8_search(table, queries, 100, "l2", opts=scan.options(overfetch=0, boundary_fp64=1))
    torch.cuda.synchronize()
    ids, dist = res_np(res)
    truth = fp64_truth(torch, base, queries, 100, "l2")
    assert recall(ids[:, :10], truth[:, :10]) >= 0.99
    assert recall(ids, truth) >= 0.99
    check_distances(oracle_mod, base.cpu().numpy(), queries.cpu().numpy(), ids, dist, "l2", range(0, 1000, 20))


def test_ivf_pq_zipf_1m_x_128(cuda, oracle_mod):
    import bench
    from fvgb300 import datasets
    from fvgb300.index import BUILD_IVF_PQ, GpuVectorIndex, IndexConfig
    from fvgb300.ivf import IvfTable

    torch = cuda
    n, dim, nlist = 1_000_000, 128, 4096
    rows, centres, qgen, sizes = bench.zipf_ivf_data(n, dim, nlist, 3, torch.device("cuda"))
    assert sizes.max() > 40 * 64 and sizes.min() == 64
    idx = GpuVectorIndex(IndexConfig(dim=dim, nlist=nlist, m_pq=32, metric="l2", build_flags=BUILD_IVF_PQ,
                                     kmeans_iters_given=2, train_rows=262_144, pq_iters=10, seed=3))
    idx.build_device(rows, centres)
    torch.cuda.synchronize()
    t = idx.export_ivf()
    q = qgen(200, 4242).contiguous()
    words = datasets.bernoulli_mask_words(n, 0.10, seed=3)
    mask = torch.from_numpy(words.view(np.int32)).cuda()
    table = IvfTable("pq", t, vectors=rows)
    res = table.search(q, 10, 32, 400, "l2", mask=mask)
    torch.cuda.synchronize()
    ids, dist = res_np(res)
    rows_np, q_np = rows.cpu().numpy(), q.cpu().numpy()
    ref = oracle_mod.ivf_pq_search(t, rows_np, q_np, 10, 32, 400, "l2", mask=words)
    assert np.array_equal(ids, ref["id"])
    assert np.array_equal(dist.view(np.uint32), ref["distance"].view(np.uint32))
    allowed = torch.from_numpy(datasets.unpack_words(words, n)).cuda()
    truth = fp64_truth(torch, rows, q, 10, "l2", allowed=allowed)
    assert recall(ids, truth) >= 0.9
