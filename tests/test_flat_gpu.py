"""Parity of the exact fp32 flat scan (cuda_flat_scan_batch) with the oracle.

The kernel sums in the same order as the reference's exact search, so ids
and distances must be bit-identical to the oracle's (ties -> lower slot),
and to the reference backend's golden outputs on integer data."""
from __future__ import annotations

import numpy as np
import pytest

from conftest import load_golden

pytestmark = pytest.mark.gpu


def run_flat(torch, base, queries, k, metric="l2", mask=None, vec_ids=None):
    from fvgb300 import scan

    dev = torch.device("cuda")
    b = torch.from_numpy(np.ascontiguousarray(base)).to(dev) if base is not None and base.size else None
    q = torch.from_numpy(np.ascontiguousarray(queries)).to(dev)
    m = torch.from_numpy(np.ascontiguousarray(mask, dtype=np.uint32).view(np.int32)).to(dev) if mask is not None else None
    v = torch.from_numpy(np.ascontiguousarray(vec_ids, dtype=np.uint32).view(np.int32)).to(dev) if vec_ids is not None else None
    res = scan.flat_scan(b, q, k, metric, mask=m, vec_ids=v)
    torch.cuda.synchronize()
    r = res.cpu().numpy()
    return r[..., 0].view(np.uint32), r[..., 1].view(np.float32)


def assert_same(ids, dist, ref):
    assert np.array_equal(ids, ref["id"]), np.argwhere(ids != ref["id"])[:5]
    assert np.array_equal(dist.view(np.uint32), ref["distance"].view(np.uint32))


@pytest.mark.parametrize("name", ["flat_l2_int", "flat_l2_int_k100", "flat_ip_unit", "flat_cos"])
def test_flat_golden(cuda, oracle_mod, name):
    from fvgb300.datasets import pack_bools

    g = load_golden(name)
    k = int(g["k"])
    metric = str(g["metric"])
    ids, dist = run_flat(cuda, g["base"], g["queries"], k, metric)
    assert_same(ids, dist, oracle_mod.exact_knn(g["base"], g["queries"], k, metric))
    if metric == "l2":
        assert np.array_equal(ids, g["labels"])
        assert np.array_equal(dist, g["dists"])
    words = pack_bools(g["mask"])
    ids, dist = run_flat(cuda, g["base"], g["queries"], k, metric, mask=words)
    assert_same(ids, dist, oracle_mod.exact_knn(g["base"], g["queries"], k, metric, mask=words))
    if metric == "l2":
        assert np.array_equal(ids, g["labels_masked"])


@pytest.mark.parametrize("metric", ["l2", "ip", "cosine"])
@pytest.mark.parametrize("n,dim,nq,k", [(5000, 128, 70, 10), (4099, 33, 5, 1), (777, 97, 130, 256),
                                        (3000, 64, 64, 300), (20, 8, 3, 50), (100000, 16, 2, 7)])
def test_flat_random_shapes(cuda, oracle_mod, metric, n, dim, nq, k):
    rng = np.random.default_rng(n + dim + k)
    base = rng.standard_normal((n, dim), dtype=np.float32)
    queries = rng.standard_normal((nq, dim), dtype=np.float32)
    ids, dist = run_flat(cuda, base, queries, k, metric)
    assert ids.shape == (nq, min(k, 256))
    assert_same(ids, dist, oracle_mod.exact_knn(base, queries, min(k, 256), metric))


def test_flat_mask_and_vec_ids(cuda, oracle_mod):
    rng = np.random.default_rng(9)
    n, dim = 6000, 48
    base = np.rint(rng.uniform(0, 20, (n, dim))).astype(np.float32)
    queries = np.rint(rng.uniform(0, 20, (40, dim))).astype(np.float32)
    from fvgb300.datasets import bernoulli_mask_words

    mask = bernoulli_mask_words(n, 0.1, 4)
    vec_ids = rng.permutation(10 * n)[:n].astype(np.uint32)
    ids, dist = run_flat(cuda, base, queries, 20, "l2", mask=mask, vec_ids=vec_ids)
    ref = oracle_mod.exact_knn(base, queries, 20, "l2", mask=mask, vec_ids=vec_ids)
    assert_same(ids, dist, ref)


def test_flat_edge_cases(cuda):
    from fvgb300 import scan
    from fvgb300._lib import FvError

    torch = cuda
    q = torch.zeros((3, 8), device="cuda")
    # N == 0: the reference memsets the outputs to 0xFF
    out = scan.flat_scan(None, q, 4)
    torch.cuda.synchronize()
    assert np.all(out.cpu().numpy().view(np.uint32) == 0xFFFFFFFF)
    # fewer rows than k: sentinels {0xFFFFFFFF, 1e30} fill the tail
    ids, dist = run_flat(torch, np.ones((3, 8), np.float32), np.zeros((2, 8), np.float32), 5)
    assert np.all(ids[:, 3:] == 0xFFFFFFFF) and np.all(dist[:, 3:] == np.float32(1e30))
    assert np.array_equal(ids[:, :3], [[0, 1, 2], [0, 1, 2]])  # all tie -> lower slot first
    # every row masked out
    ids, _ = run_flat(torch, np.ones((40, 8), np.float32), np.zeros((1, 8), np.float32), 3,
                      mask=np.zeros(2, np.uint32))
    assert np.all(ids == 0xFFFFFFFF)
    # zero queries / zero k are no-ops that succeed
    from fvgb300._lib import lib
    import ctypes

    assert lib().cuda_flat_scan_batch(None, None, 0, 8, ctypes.c_void_p(q.data_ptr()), 0, 5, 0, None,
                                      ctypes.c_void_p(q.data_ptr()), None) == 0
    # null queries -> -1
    assert lib().cuda_flat_scan_batch(None, None, 0, 8, None, 1, 5, 0, None, None, None) == -1
    # the wrapper raises on a non-zero return
    from fvgb300._lib import call

    with pytest.raises(FvError):
        call("cuda_flat_scan_batch", None, None, 4, 8, None, 1, 5, 0, None, None, None)
    assert scan.device_status() == 0


def test_warp_distance_fixture(cuda, oracle_mod):
    """tests/cuda_sanity_test.rs:45-113 ramp fixture through
    cuda_compute_distances_warp: bit-identical to the oracle's restatement of
    the reference's warp-order distance."""
    from fvgb300 import scan

    torch = cuda
    dim = 128
    q = (np.arange(4 * dim, dtype=np.float32) * np.float32(0.01)).reshape(4, dim)
    x = (np.arange(8 * dim, dtype=np.float32) * np.float32(0.02)).reshape(8, dim)
    for metric in ("l2", "ip", "cosine"):
        got = scan.distance_matrix(torch.from_numpy(q).cuda(), torch.from_numpy(x).cuda(), metric).cpu().numpy()
        ref = oracle_mod.distance_matrix(q, x, metric)
        assert np.array_equal(got.view(np.uint32), ref.view(np.uint32)), metric


def test_bitonic_fixture(cuda):
    """tests/cuda_sanity_test.rs:116-159 keys, plus a 1000-element case."""
    from fvgb300 import scan

    torch = cuda
    for keys in ([45.2, 1.2, 99.0, 3.15, 0.5, 12.8, 88.3, 7.7],
                 list(np.random.default_rng(1).standard_normal(1000))):
        k = torch.tensor(keys, dtype=torch.float32, device="cuda")
        v = torch.arange(len(keys), dtype=torch.int32, device="cuda")
        ko, vo = scan.bitonic_sort(k, v)
        ko, vo = ko.cpu().numpy(), vo.cpu().numpy()
        assert np.all(ko[1:] >= ko[:-1])
        assert np.array_equal(np.asarray(keys, np.float32)[vo], ko)
