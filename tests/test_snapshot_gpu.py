"""FLSHVEC1 snapshots on the GPU: an engine saved and loaded answers every
engine's queries exactly as before; a file laid out as the reference writes
it (slots whose logical ids are not their indices, tombstones, the
reference's id-ordered IVF codes) loads into tables whose answers equal the
oracle's on the same data, ids mapped to logical ids."""
from __future__ import annotations

import numpy as np
import pytest

from flshvec1 import EMPTY_GRAPH_SECTIONS, write_snapshot

pytestmark = pytest.mark.gpu


def gen(n, dim, clusters, seed, sigma=0.2):
    rng = np.random.default_rng(seed)
    c = rng.uniform(-1, 1, size=(clusters, dim)).astype(np.float32)
    return (c[rng.integers(0, clusters, n)] + np.float32(sigma) * rng.standard_normal((n, dim))).astype(np.float32)


def all_engines(idx, q, k=10):
    return {"flat": idx.batch_search_flat(q, len(q), k), "fp16": idx.batch_search_fp16_tc(q, len(q), k),
            "pq": idx.batch_search_ivf_mode(q, len(q), k, 6, 64, "pq"),
            "sq8": idx.batch_search_ivf_mode(q, len(q), k, 6, 64, "sq8"),
            "rabitq": idx.batch_search_ivf_mode(q, len(q), k, 6, 64, "rabitq")}


@pytest.mark.parametrize("metric", ["l2", "ip"])
def test_save_load_round_trip(cuda, tmp_path, metric):
    from fvgb300.index import BUILD_FP8, BUILD_FP16, BUILD_IVF_PQ, BUILD_IVF_RABITQ, BUILD_IVF_SQ8, GpuVectorIndex, \
        IndexConfig, snapshot_manifest

    x = gen(3000, 48, 16, 1)
    flags = BUILD_FP16 | BUILD_IVF_PQ | BUILD_IVF_SQ8 | BUILD_IVF_RABITQ
    idx = GpuVectorIndex(IndexConfig(dim=48, nlist=24, m_pq=8, metric=metric, build_flags=flags))
    idx.build(x)
    idx.add_vectors(gen(40, 48, 16, 2))
    idx.delete_ids([5, 17, 3001])
    q = gen(20, 48, 16, 3)
    before = all_engines(idx, q)
    p = tmp_path / "idx.flshvec1"
    idx.save_snapshot(p)
    m = snapshot_manifest(p)
    for name in ("vectors", "logical_ids", "main_valid_words", "hnsw_adjacency", "cagra_adjacency", "ivf_centroids",
                 "pq_codebooks", "pq_codes", "ivf_offsets", "ivf_vec_ids", "sq_mins", "sq_scales", "sq_codes",
                 "rabitq_signs", "rabitq_bits", "vectors_fp16", "vec_norms_sq", "tombstones", "delta_vectors",
                 "delta_ids"):
        assert name in m["sections"], name
    assert m["num_vectors"] == 3000 and m["next_logical_id"] == 3040 and m["fp16_padded_dim"] == 48
    assert m["rabitq_padded_dim"] == 64 and m["sections"]["rabitq_bits"]["byte_len"] == 3000 * 2 * 4
    loaded = GpuVectorIndex.load_snapshot(p, IndexConfig(dim=48, build_flags=flags | BUILD_FP8))
    inf0, inf1 = idx.info(), loaded.info()
    for key in ("num_vectors", "delta_len", "tombstones", "dim", "nlist", "m_pq", "metric", "next_id"):
        assert inf0[key] == inf1[key], key
    after = all_engines(loaded, q)
    for name in before:
        assert np.array_equal(before[name][0], after[name][0]), name
        assert np.array_equal(before[name][1], after[name][1]), name
    ids, _ = loaded.batch_search_fp8(q, len(q), 10)
    assert not np.isin(ids, [5, 17, 3001]).any()
    t0, t1 = idx.export_ivf(), loaded.export_ivf()
    for key in ("centroids", "offsets", "vec_ids", "codebooks", "pq_codes", "sq_codes", "rot_signs", "rot_centroids",
                "rabitq_bits", "rabitq_meta"):
        assert np.array_equal(t0[key], t1[key]), key
    assert loaded.add_vectors(gen(1, 48, 16, 9)).tolist() == [3040]


@pytest.mark.parametrize("rabitq_in_file", [True, False])
def test_reference_layout_with_remapped_ids(cuda, oracle_mod, tmp_path, rabitq_in_file):
    """Slots carry logical ids 3 s + 1 (gaps between them), a few slots are
    tombstoned; codes are indexed by slot, as the reference stores them.
    RaBitQ tables come from the file, or (sections empty) are encoded on the
    GPU from the file's rows and lists -- the same tables either way."""
    from fvgb300.index import BUILD_FP16, BUILD_IVF_PQ, BUILD_IVF_RABITQ, BUILD_IVF_SQ8, GpuVectorIndex, IndexConfig

    n, dim = 2000, 32
    x = gen(n, dim, 10, 4)
    t = oracle_mod.build_ivf(x, nlist=12, m_pq=8, iters=10, seed=2)
    lid = (3 * np.arange(n) + 1).astype(np.uint32)
    dead_slots = np.array([0, 7, 99, 1500])
    valid = np.ones(n, bool)
    valid[dead_slots] = False
    words = np.zeros((n + 31) // 32, np.uint32)
    for s in np.nonzero(valid)[0]:
        words[s >> 5] |= np.uint32(1 << (s & 31))
    f16, norms = oracle_mod.encode_fp16_padded(x)
    cfg = {"dim": dim, "max_elements": n, "m": 32, "ef_construction": 128, "nlist": 12, "m_pq": 8, "metric": 0}
    sections = [("vectors", x), ("logical_ids", lid), ("main_valid_words", words)] + EMPTY_GRAPH_SECTIONS[:3] + [
        ("ivf_centroids", t["centroids"]), ("pq_codebooks", t["codebooks"]), ("pq_codes", t["pq_codes"]),
        ("ivf_offsets", t["offsets"]), ("ivf_vec_ids", t["vec_ids"]), ("sq_mins", t["sq_mins"]),
        ("sq_scales", t["sq_scales"]), ("sq_codes", t["sq_codes"])]
    rq = [("rabitq_signs", t["rot_signs"]), ("rabitq_centroids", t["rot_centroids"]),
          ("rabitq_bits", t["rabitq_bits"]), ("rabitq_meta", t["rabitq_meta"])]
    sections += (rq if rabitq_in_file else EMPTY_GRAPH_SECTIONS[3:]) + [
        ("vectors_fp16", f16), ("vec_norms_sq", norms), ("tombstones", lid[dead_slots])]
    p = tmp_path / "ref.flshvec1"
    write_snapshot(p, cfg, n, sections, next_logical_id=int(lid.max()) + 1, fp16_padded_dim=f16.shape[1],
                   rabitq_padded_dim=t["padded_dim"] if rabitq_in_file else 0)
    idx = GpuVectorIndex.load_snapshot(p, IndexConfig(dim=dim, build_flags=BUILD_FP16 | BUILD_IVF_PQ | BUILD_IVF_SQ8 |
                                                      BUILD_IVF_RABITQ))
    inf = idx.info()
    assert inf["num_vectors"] == int(lid.max()) + 1 and inf["tombstones"] == len(dead_slots)
    q = gen(16, dim, 10, 5)
    slot_mask = words
    for mode, fn in (("pq", oracle_mod.ivf_pq_search), ("sq8", oracle_mod.ivf_sq_search),
                     ("rabitq", oracle_mod.ivf_rabitq_search)):
        ids, dist = idx.batch_search_ivf_mode(q, 16, 10, 5, 64, mode)
        ref = fn(t, x, q, 10, 5, 64, mask=slot_mask)
        want = np.where(ref["id"] == 0xFFFFFFFF, 0xFFFFFFFF, lid[np.minimum(ref["id"], n - 1)])
        assert np.array_equal(ids, want), mode
        assert np.array_equal(dist, ref["distance"]), mode
    ids, dist = idx.batch_search_flat(q, 16, 10)
    ref = oracle_mod.exact_knn(x, q, 10, "l2", mask=slot_mask)
    assert np.array_equal(ids, lid[ref["id"]]) and np.array_equal(dist, ref["distance"])
    # a user filter over logical ids is honoured on the remapped slots
    allow = np.zeros(int(lid.max()) + 1, bool)
    allow[lid[::2]] = True
    from fvgb300.datasets import pack_bools

    ids, _ = idx.batch_search_fp16_tc(q, 16, 10, pack_bools(allow))
    assert np.all(allow[ids[ids != 0xFFFFFFFF]])
