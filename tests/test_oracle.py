"""Pins the CPU oracle against the reference's known-answer tests and against
golden fixtures produced by the reference's own Python brute force
(tests/golden/make_golden.py). CPU only."""
from __future__ import annotations

import numpy as np
import pytest

from conftest import load_golden


def seq_l2(q, x):
    s = np.float32(0.0)
    for a, b in zip(q, x):
        t = np.float32(a) - np.float32(b)
        s = np.float32(s + np.float32(t * t))
    return s


def test_ramp_fixture_warp_vs_sequential(oracle_mod):
    """tests/cuda_sanity_test.rs:45-113: q = i*0.01, x = i*0.02, d = 128,
    4 x 8; the warp-order distance agrees with the sequential CPU sum to a
    relative 1e-4 (denominator max(cpu, 1))."""
    dim, nq, n = 128, 4, 8
    q = (np.arange(nq * dim, dtype=np.float32) * np.float32(0.01)).reshape(nq, dim)
    x = (np.arange(n * dim, dtype=np.float32) * np.float32(0.02)).reshape(n, dim)
    warp = oracle_mod.distance_matrix(q, x, "l2")
    exact = oracle_mod.exact_knn(x, q, n)
    for i in range(nq):
        for j in range(n):
            cpu = seq_l2(q[i], x[j])
            assert abs(cpu - warp[i, j]) / max(cpu, 1.0) < 1e-4
        # exact_knn returns sequential-order distances exactly
        for r in range(n):
            sid = exact[i, r]["id"]
            assert exact[i, r]["distance"] == seq_l2(q[i], x[sid])


def test_packed_mask_kat():
    """crates/engine/src/filter.rs:491-515: ids 4096 and 70000 packed into
    ceil(70005/32) words, bit id&31 of word id>>5."""
    from fvgb300.datasets import pack_bools, unpack_words

    bits = np.zeros(70005, dtype=bool)
    bits[[4096, 70000]] = True
    words = pack_bools(bits)
    assert words.shape[0] == (70005 + 31) // 32
    assert words[4096 // 32] & (1 << (4096 & 31))
    assert words[70000 // 32] & (1 << (70000 & 31))
    assert words[0] == 0
    assert np.array_equal(unpack_words(words, 70005), bits)


def test_sq8_roundtrip_kat(oracle_mod):
    """crates/engine/src/quant.rs:349-359."""
    res = np.array([-2.0, 0.0, 2.0, 4.0, -1.0, 0.5, 1.0, 2.0], dtype=np.float32).reshape(2, 4)
    mins, scales = oracle_mod.sq8_fit(res)
    codes = oracle_mod.sq8_encode(res, mins, scales)
    rec = mins + scales * codes[0].astype(np.float32)
    assert np.all(np.abs(rec - res[0]) < 0.03)


def test_fp16_roundtrip_and_rounding_kat(oracle_mod):
    """crates/engine/src/quant.rs:361-368 plus the converter's rounding rule
    (quant.rs:264: half-way mantissas round up, unlike IEEE round-to-even)."""
    for v in (0.0, 1.0, -1.5, 0.125, 42.25, -100.5):
        assert abs(oracle_mod.f16_bits_to_f32(oracle_mod.f32_to_f16_bits(v)) - v) < 1e-2
    halfway = float(np.float32(1.0) + np.float32(2.0 ** -11))
    assert oracle_mod.f32_to_f16_bits(halfway) == 0x3C01
    assert int(np.float16(halfway).view(np.uint16)) == 0x3C00  # RNE differs
    assert oracle_mod.f32_to_f16_bits(1e6) == 0x7C00
    assert oracle_mod.f32_to_f16_bits(float("nan")) == 0x7E00
    assert oracle_mod.f32_to_f16_bits(1e-9) == 0


@pytest.mark.parametrize("name", ["flat_l2_int", "flat_l2_int_k100"])
def test_exact_knn_matches_reference_backend_on_integer_data(oracle_mod, name):
    """On integer-valued data every summation order is exact, so the fp32
    restatement must reproduce the reference backend's ids and distances
    bit for bit, lower id first on ties (duplicates are planted)."""
    g = load_golden(name)
    k = int(g["k"])
    got = oracle_mod.exact_knn(g["base"], g["queries"], k)
    assert np.array_equal(got["id"], g["labels"])
    assert np.array_equal(got["distance"], g["dists"])
    from fvgb300.datasets import pack_bools

    got_m = oracle_mod.exact_knn(g["base"], g["queries"], k, mask=pack_bools(g["mask"]))
    assert np.array_equal(got_m["id"], g["labels_masked"])
    valid = g["labels_masked"] != 0xFFFFFFFF
    assert np.array_equal(got_m["distance"][valid], g["dists_masked"][valid])


@pytest.mark.parametrize("name,metric", [("flat_ip_unit", "ip"), ("flat_cos", "cosine")])
def test_fp64_oracle_matches_reference_backend(oracle_mod, name, metric):
    g = load_golden(name)
    k = int(g["k"])
    ids, dist = oracle_mod.bruteforce_f64(g["base"], g["queries"], k, metric)
    assert np.array_equal(ids, g["labels"])
    assert np.allclose(dist, g["dists"], rtol=1e-6, atol=1e-6)
    from fvgb300.datasets import pack_bools

    ids_m, _ = oracle_mod.bruteforce_f64(g["base"], g["queries"], k, metric, mask=pack_bools(g["mask"]))
    assert np.array_equal(ids_m, g["labels_masked"])
    # the fp32 restatement agrees with the float64 backend up to fp32 rounding
    got = oracle_mod.exact_knn(g["base"], g["queries"], k, metric)
    agree = (got["id"] == g["labels"]).mean()
    assert agree > 0.98
    assert np.allclose(got["distance"], g["dists"], rtol=1e-5, atol=1e-5)


def gen_clustered(n, dim, clusters, seed):
    """Shape of the reference's e2e generator (e2e_search_test.rs:156-177):
    centres U(-1, 1), sigma 0.18, row i in cluster i % clusters."""
    rng = np.random.default_rng(seed)
    centers = rng.uniform(-1, 1, size=(clusters, dim)).astype(np.float32)
    x = centers[np.arange(n) % clusters] + np.float32(0.18) * rng.standard_normal((n, dim), dtype=np.float32)
    return x.astype(np.float32)


@pytest.fixture(scope="module")
def ivf_case(oracle_mod):
    x = gen_clustered(1500, 96, 12, 202)
    t = oracle_mod.build_ivf(x, nlist=24, m_pq=12, iters=25, seed=5)
    return x, t


@pytest.mark.parametrize("mode", ["pq", "sq8"])
@pytest.mark.parametrize("rerank", [256, 512, 0, 1])
def test_ivf_oracle_recall_at_reference_params(oracle_mod, ivf_case, mode, rerank):
    """e2e_search_test.rs:231-277: d=96, N=1500, nlist=24, M=12, nprobe=12,
    rerank 256 (and the 2-stage 512), queries = the first 8 rows; recall@10
    >= 0.80 against exact search."""
    x, t = ivf_case
    q = x[:8]
    fn = oracle_mod.ivf_pq_search if mode == "pq" else oracle_mod.ivf_sq_search
    res = fn(t, x, q, 10, 12, rerank)
    truth = oracle_mod.exact_knn(x, q, 10)
    r = oracle_mod.recall(res["id"], truth["id"])
    floor = 0.80 if rerank not in (0, 1) or mode == "sq8" else 0.3
    assert r >= floor, (mode, rerank, r)
    d = res["distance"]
    assert np.all(d[:, :-1] <= d[:, 1:])


def test_ivf_oracle_large_k_sorted_and_filled(oracle_mod):
    """python/tests/test_bindings.py:123-138: k=100 over N=1000, d=64,
    nlist=16, m_pq=8, nprobe=16 -> sorted and >= 90% valid."""
    rng = np.random.default_rng(3)
    x = rng.standard_normal((1000, 64), dtype=np.float32)
    t = oracle_mod.build_ivf(x, nlist=16, m_pq=8, iters=10, seed=1)
    res = oracle_mod.ivf_pq_search(t, x, rng.standard_normal((1, 64), dtype=np.float32), 100, 16, 0)
    assert (res["id"] != 0xFFFFFFFF).sum() >= 90
    assert np.all(res["distance"][0, :-1] <= res["distance"][0, 1:])


def test_ivf_oracle_respects_mask(oracle_mod, ivf_case):
    """e2e_search_test.rs:322-433: no masked-out id is returned."""
    from fvgb300.datasets import pack_bools

    x, t = ivf_case
    allowed = np.zeros(x.shape[0], dtype=bool)
    allowed[10:200] = True
    words = pack_bools(allowed)
    for fn in (oracle_mod.ivf_pq_search, oracle_mod.ivf_sq_search):
        res = fn(t, x, x[:2], 5, 8, 64, mask=words)
        ids = res["id"][res["id"] != 0xFFFFFFFF]
        assert ids.size > 0 and np.all(allowed[ids])
