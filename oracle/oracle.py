"""ctypes front end of the CPU oracle (liboracle.so).

TEST INFRASTRUCTURE ONLY: imported by tests/, by __graft_entry__.smoke() as
the checker, and by bench.py's CPU-baseline / reference legs. The product
never imports this module.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB_PATH = HERE / "liboracle.so"

L2, COSINE, IP = 0, 1, 2
METRICS = {"l2": L2, "cosine": COSINE, "ip": IP}
RESULT_DTYPE = np.dtype([("id", "<u4"), ("distance", "<f4")])

_lib = None


def build(force: bool = False) -> Path:
    if force or not LIB_PATH.exists() or LIB_PATH.stat().st_mtime < max(
        (HERE / "oracle.c").stat().st_mtime, (HERE / "oracle.h").stat().st_mtime
    ):
        subprocess.run(["make", "-s", "-B" if force else "all"], cwd=HERE, check=True)
    return LIB_PATH


def lib():
    global _lib
    if _lib is None:
        build()
        _lib = C.CDLL(str(LIB_PATH))
        P = C.c_void_p
        u32 = C.c_uint32
        i32 = C.c_int
        sig = {
            "fvo_exact_knn_f32": (None, [P, P, u32, u32, P, u32, u32, i32, P, P, i32]),
            "fvo_bruteforce_f64": (None, [P, u32, u32, P, u32, u32, i32, P, P, P, i32]),
            "fvo_warp_distance": (C.c_float, [P, P, u32, i32]),
            "fvo_distance_matrix": (None, [P, P, u32, u32, u32, i32, P]),
            "fvo_f32_to_f16": (C.c_uint16, [C.c_float]),
            "fvo_f16_to_f32": (C.c_float, [C.c_uint16]),
            "fvo_encode_fp16_padded": (None, [P, u32, u32, P, P]),
            "fvo_sq8_fit": (None, [P, u32, u32, P, P]),
            "fvo_sq8_encode": (None, [P, u32, u32, P, P, P]),
            "fvo_kmeans": (None, [P, u32, u32, u32, u32, C.c_uint64, P, P, i32]),
            "fvo_pq_train": (None, [P, u32, u32, u32, u32, C.c_uint64, P, i32]),
            "fvo_pq_encode": (None, [P, u32, u32, u32, P, P, i32]),
            "fvo_ivf_lists": (None, [P, u32, u32, P, P]),
            "fvo_residuals": (None, [P, u32, u32, P, P, P]),
            "fvo_ivf_pq_search": (u32, [P, P, P, P, P, P, u32, u32, u32, u32, u32, P, u32, u32, u32, u32, i32, P, P, i32]),
            "fvo_ivf_sq_search": (u32, [P, P, P, P, P, P, P, u32, u32, u32, P, u32, u32, u32, u32, i32, P, P, i32]),
            "fvo_coarse_probe": (None, [P, u32, u32, P, u32, u32, P, P, i32]),
            "fvo_recall": (C.c_double, [P, u32, P, u32, u32, u32]),
            "fvo_rabitq_padded_dim": (u32, [u32]),
            "fvo_rabitq_rot_signs": (None, [u32, C.c_uint64, P]),
            "fvo_rabitq_inv_sqrt": (C.c_float, [u32]),
            "fvo_rabitq_rotate": (None, [P, u32, P, u32, P]),
            "fvo_rabitq_encode": (None, [P, u32, u32, P, u32, P, P, u32, P, P, P, i32]),
            "fvo_ivf_rabitq_search": (u32, [P, P, P, P, P, P, P, P, u32, u32, u32, u32, P, u32, u32, u32, u32, i32, P,
                                            P, i32]),
        }
        for name, (res, args) in sig.items():
            f = getattr(_lib, name)
            f.restype = res
            f.argtypes = args
    return _lib


def _p(a):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


def _f32(a):
    return np.ascontiguousarray(a, dtype=np.float32)


def _metric(m):
    return METRICS[m] if isinstance(m, str) else int(m)


def threads_default() -> int:
    return os.cpu_count() or 1


def exact_knn(base, queries, k, metric="l2", mask=None, vec_ids=None, threads=None):
    """Reference-order exact fp32 search; returns structured (Q, k) results."""
    base, queries = _f32(base), _f32(queries)
    n, dim = base.shape if base.size else (0, queries.shape[1])
    nq = queries.shape[0]
    out = np.zeros((nq, k), dtype=RESULT_DTYPE)
    mask = None if mask is None else np.ascontiguousarray(mask, dtype=np.uint32)
    vec_ids = None if vec_ids is None else np.ascontiguousarray(vec_ids, dtype=np.uint32)
    lib().fvo_exact_knn_f32(_p(base), _p(vec_ids), n, dim, _p(queries), nq, k, _metric(metric), _p(mask), _p(out),
                            threads or threads_default())
    return out


def bruteforce_f64(base, queries, k, metric="l2", mask=None, threads=None):
    base, queries = _f32(base), _f32(queries)
    n, dim = base.shape
    nq = queries.shape[0]
    ids = np.zeros((nq, k), dtype=np.uint32)
    dist = np.zeros((nq, k), dtype=np.float64)
    mask = None if mask is None else np.ascontiguousarray(mask, dtype=np.uint32)
    lib().fvo_bruteforce_f64(_p(base), n, dim, _p(queries), nq, k, _metric(metric), _p(mask), _p(ids), _p(dist),
                             threads or threads_default())
    return ids, dist


def warp_distance(q, x, metric="l2") -> float:
    q, x = _f32(q), _f32(x)
    return float(lib().fvo_warp_distance(_p(q), _p(x), q.shape[0], _metric(metric)))


def distance_matrix(queries, base, metric="l2"):
    queries, base = _f32(queries), _f32(base)
    out = np.zeros((queries.shape[0], base.shape[0]), dtype=np.float32)
    lib().fvo_distance_matrix(_p(queries), _p(base), queries.shape[0], base.shape[0], queries.shape[1],
                              _metric(metric), _p(out))
    return out


def f32_to_f16_bits(x) -> int:
    return int(lib().fvo_f32_to_f16(float(x)))


def f16_bits_to_f32(h) -> float:
    return float(lib().fvo_f16_to_f32(int(h)))


def encode_fp16_padded(x):
    x = _f32(x)
    n, dim = x.shape
    pd = (dim + 15) // 16 * 16
    out = np.zeros((n, pd), dtype=np.uint16)
    norms = np.zeros(n, dtype=np.float32)
    lib().fvo_encode_fp16_padded(_p(x), n, dim, _p(out), _p(norms))
    return out, norms


def sq8_fit(res):
    res = _f32(res)
    n, dim = res.shape
    mins = np.zeros(dim, dtype=np.float32)
    scales = np.zeros(dim, dtype=np.float32)
    lib().fvo_sq8_fit(_p(res), n, dim, _p(mins), _p(scales))
    return mins, scales


def sq8_encode(res, mins, scales):
    res = _f32(res)
    n, dim = res.shape
    codes = np.zeros((n, dim), dtype=np.uint8)
    lib().fvo_sq8_encode(_p(res), n, dim, _p(_f32(mins)), _p(_f32(scales)), _p(codes))
    return codes


def kmeans(x, k, iters=25, seed=0, threads=None):
    x = _f32(x)
    n, dim = x.shape
    cent = np.zeros((k, dim), dtype=np.float32)
    assign = np.zeros(n, dtype=np.uint32)
    lib().fvo_kmeans(_p(x), n, dim, k, iters, seed, _p(cent), _p(assign), threads or threads_default())
    return cent, assign


def pq_train(x, m_pq, iters=25, seed=0, threads=None):
    x = _f32(x)
    n, dim = x.shape
    sub = dim // m_pq
    cb = np.zeros((m_pq, 256, sub), dtype=np.float32)
    lib().fvo_pq_train(_p(x), n, dim, m_pq, iters, seed, _p(cb), threads or threads_default())
    return cb


def pq_encode(x, codebooks, threads=None):
    x = _f32(x)
    n, dim = x.shape
    m_pq = codebooks.shape[0]
    codes = np.zeros((n, m_pq), dtype=np.uint8)
    lib().fvo_pq_encode(_p(x), n, dim, m_pq, _p(_f32(codebooks)), _p(codes), threads or threads_default())
    return codes


def ivf_lists(assign, nlist):
    assign = np.ascontiguousarray(assign, dtype=np.uint32)
    offsets = np.zeros(nlist + 1, dtype=np.uint32)
    vec_ids = np.zeros(assign.shape[0], dtype=np.uint32)
    lib().fvo_ivf_lists(_p(assign), assign.shape[0], nlist, _p(offsets), _p(vec_ids))
    return offsets, vec_ids


def residuals(x, centroids, assign):
    x = _f32(x)
    out = np.zeros_like(x)
    lib().fvo_residuals(_p(x), x.shape[0], x.shape[1], _p(_f32(centroids)),
                        _p(np.ascontiguousarray(assign, dtype=np.uint32)), _p(out))
    return out


def build_ivf(x, nlist, m_pq=None, iters=25, seed=0, threads=None):
    """IVF build as index.rs:405-458: k-means, residuals, PQ / SQ8 on residuals, lists."""
    x = _f32(x)
    n, dim = x.shape
    nlist = max(1, min(nlist, n))
    cent, assign = kmeans(x, nlist, iters, seed, threads)
    res = residuals(x, cent, assign)
    offsets, vec_ids = ivf_lists(assign, nlist)
    t = {"centroids": cent, "assign": assign, "offsets": offsets, "vec_ids": vec_ids, "nlist": nlist}
    if m_pq:
        cb = pq_train(res, m_pq, iters, seed + 7, threads)
        t["codebooks"] = cb
        t["pq_codes"] = pq_encode(res, cb, threads)
    mins, scales = sq8_fit(res)
    t["sq_mins"], t["sq_scales"] = mins, scales
    t["sq_codes"] = sq8_encode(res, mins, scales)
    t.update(rabitq_encode(x, cent, assign, RABITQ_SEED, threads))
    return t


# the engine's RaBitQ rotation seed (index.rs:435-441)
RABITQ_SEED = 0x5F37_59DF_CAFE_BABE


def rabitq_padded_dim(dim) -> int:
    return int(lib().fvo_rabitq_padded_dim(dim))


def rabitq_rot_signs(padded_dim, seed=RABITQ_SEED):
    out = np.zeros(3 * padded_dim, dtype=np.float32)
    lib().fvo_rabitq_rot_signs(padded_dim, seed, _p(out))
    return out


def rabitq_rotate(v, signs, padded_dim):
    v = _f32(v)
    out = np.zeros(padded_dim, dtype=np.float32)
    lib().fvo_rabitq_rotate(_p(v), v.shape[0], _p(_f32(signs)), padded_dim, _p(out))
    return out


def rabitq_encode(x, centroids, assign, seed=RABITQ_SEED, threads=None):
    """RabitqEncoder::encode (quant.rs:156-234): rot_signs, rot_centroids,
    rabitq_bits [n][P/32] u32, rabitq_meta [n][4] f32."""
    x, centroids = _f32(x), _f32(centroids)
    n, dim = x.shape
    nlist = centroids.shape[0]
    P = rabitq_padded_dim(dim)
    signs = rabitq_rot_signs(P, seed)
    rot_c = np.zeros((nlist, P), dtype=np.float32)
    bits = np.zeros((n, P // 32), dtype=np.uint32)
    meta = np.zeros((n, 4), dtype=np.float32)
    lib().fvo_rabitq_encode(_p(x), n, dim, _p(centroids), nlist, _p(np.ascontiguousarray(assign, dtype=np.uint32)),
                            _p(signs), P, _p(rot_c), _p(bits), _p(meta), threads or threads_default())
    return {"padded_dim": P, "rot_signs": signs, "rot_centroids": rot_c, "rabitq_bits": bits, "rabitq_meta": meta}


def ivf_pq_search(t, vectors, queries, top_k, nprobe, rerank_k, metric="l2", mask=None, use_vectors=True,
                  threads=None):
    queries = _f32(queries)
    vectors = _f32(vectors)
    n, dim = vectors.shape
    nq = queries.shape[0]
    k = min(top_k, 256)
    out = np.zeros((nq, k), dtype=RESULT_DTYPE)
    cb = _f32(t["codebooks"])
    m_pq = cb.shape[0]
    mask = None if mask is None else np.ascontiguousarray(mask, dtype=np.uint32)
    lib().fvo_ivf_pq_search(_p(_f32(t["centroids"])), _p(cb), _p(t["pq_codes"]), _p(t["offsets"]), _p(t["vec_ids"]),
                            _p(vectors) if use_vectors else None, n, dim, t["nlist"], m_pq, dim // m_pq,
                            _p(queries), nq, top_k, nprobe, rerank_k, _metric(metric), _p(mask), _p(out),
                            threads or threads_default())
    return out


def ivf_sq_search(t, vectors, queries, top_k, nprobe, rerank_k, metric="l2", mask=None, use_vectors=True,
                  threads=None):
    queries = _f32(queries)
    vectors = _f32(vectors)
    n, dim = vectors.shape
    nq = queries.shape[0]
    k = min(top_k, 256)
    out = np.zeros((nq, k), dtype=RESULT_DTYPE)
    mask = None if mask is None else np.ascontiguousarray(mask, dtype=np.uint32)
    lib().fvo_ivf_sq_search(_p(_f32(t["centroids"])), _p(_f32(t["sq_mins"])), _p(_f32(t["sq_scales"])),
                            _p(t["sq_codes"]), _p(t["offsets"]), _p(t["vec_ids"]),
                            _p(vectors) if use_vectors else None, n, dim, t["nlist"], _p(queries), nq, top_k, nprobe,
                            rerank_k, _metric(metric), _p(mask), _p(out), threads or threads_default())
    return out


def ivf_rabitq_search(t, vectors, queries, top_k, nprobe, rerank_k, metric="l2", mask=None, use_vectors=True,
                      threads=None):
    queries = _f32(queries)
    vectors = _f32(vectors)
    n, dim = vectors.shape
    nq = queries.shape[0]
    k = min(top_k, 256)
    out = np.zeros((nq, k), dtype=RESULT_DTYPE)
    mask = None if mask is None else np.ascontiguousarray(mask, dtype=np.uint32)
    lib().fvo_ivf_rabitq_search(_p(_f32(t["centroids"])), _p(_f32(t["rot_centroids"])), _p(t["rabitq_bits"]),
                                _p(_f32(t["rabitq_meta"])), _p(_f32(t["rot_signs"])), _p(t["offsets"]),
                                _p(t["vec_ids"]), _p(vectors) if use_vectors else None, n, dim, t["padded_dim"],
                                t["nlist"], _p(queries), nq, top_k, nprobe, rerank_k, _metric(metric), _p(mask),
                                _p(out), threads or threads_default())
    return out


def coarse_probe(centroids, queries, nprobe, threads=None):
    centroids, queries = _f32(centroids), _f32(queries)
    nq = queries.shape[0]
    lists = np.zeros((nq, nprobe), dtype=np.uint32)
    dist = np.zeros((nq, nprobe), dtype=np.float32)
    lib().fvo_coarse_probe(_p(centroids), centroids.shape[0], centroids.shape[1], _p(queries), nq, nprobe, _p(lists),
                           _p(dist), threads or threads_default())
    return lists, dist


def recall(approx_ids, truth_ids) -> float:
    a = np.ascontiguousarray(approx_ids, dtype=np.uint32)
    t = np.ascontiguousarray(truth_ids, dtype=np.uint32)
    k = t.shape[1]
    return float(lib().fvo_recall(_p(a), a.shape[1], _p(t), t.shape[1], t.shape[0], min(k, a.shape[1])))
