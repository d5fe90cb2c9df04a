"""Loading and comparing the reference's recorded IVF outputs
(tests/golden/ivf_*.npz, written by tests/golden/make_ivf_golden.py from the
reference's own kernels, kernels/src/ivf_pq_lookup.cu and
kernels/src/ivf_quant_lookup.cu, built with its -O3 --use_fast_math flags).

Parity rule, per query row (both rows sorted ascending by distance):

* distances: position by position within `tol` of the reference's:
  - IVF-PQ / IVF-SQ8, and any exact rerank, with L2 or inner product: 0
    (bit-equal: their arithmetic is written out as fmaf / adds, which
    --use_fast_math leaves alone);
  - cosine rerank: 1e-6 absolute (fast-math division and square root in
    1 - dot / (|q| |x| + 1e-8), distance_metrics.cuh);
  - IVF-RaBitQ estimates (rerank_k = 1): 1e-6 + 4e-6 x the row's largest
    |distance| (the reference rotates with rsqrtf and quantises the query
    with fast-math divisions, ivf_quant_lookup.cu:347, :409-410; this build
    uses the correctly rounded forms);
* ids: equal, except inside a tie group (entries whose reference distances
  lie within `tol` of each other): there the members must be the same set,
  in any order (the reference's bitonic sorts are not stable,
  bitonic_topk.cuh:71-95), and a tie group that reaches the k-th position
  may hold different members of the tie (each with a distance in the group).
"""
from __future__ import annotations

import json
from pathlib import Path

import numpy as np

GOLDEN = Path(__file__).resolve().parent / "golden"
TABLE_KEYS = ("centroids", "offsets", "vec_ids", "codebooks", "pq_codes", "sq_mins", "sq_scales", "sq_codes",
              "rot_signs", "rot_centroids", "rabitq_bits", "rabitq_meta")
NAMES = ("ivf_e2e", "ivf_zipf")
MODES = ("pq", "sq8", "rabitq")


def load(name):
    """-> (base f32, queries f32, mask words, tables dict, cases, reference
    results {(mode, case index): (ids, distances)})."""
    z = np.load(GOLDEN / f"{name}.npz")
    meta = json.loads(str(z["meta"]))
    if "base_f16" in z:
        base, queries = z["base_f16"].astype(np.float32), z["queries_f16"].astype(np.float32)
    else:
        base, queries = z["base_u8"].astype(np.float32), z["queries_u8"].astype(np.float32)
    t = {k: z[k] for k in TABLE_KEYS}
    t["nlist"] = int(z["nlist"])
    t["padded_dim"] = int(z["padded_dim"])
    ref = {}
    for mode in MODES:
        for ci in range(len(meta["cases"])):
            ref[(mode, ci)] = (z[f"{mode}_{ci}_id"], z[f"{mode}_{ci}_distance"])
    return base, queries, z["mask"], t, meta["cases"], ref


def tolerance(mode, case, d_ref_row):
    if mode == "rabitq" and case["rerank"] == 1:
        return 1e-6 + 4e-6 * float(np.max(np.abs(d_ref_row[d_ref_row < 1e29]), initial=0.0))
    if case["metric"] == "cosine":
        return 1e-6
    return 0.0


def compare(mode, case, ids, dist, ref_ids, ref_dist):
    """Returns a list of mismatch descriptions (empty: parity holds)."""
    bad = []
    ids = np.asarray(ids, dtype=np.uint32)
    dist = np.asarray(dist, dtype=np.float32)
    if ids.shape != ref_ids.shape:
        return [f"shape {ids.shape} != {ref_ids.shape}"]
    k = ids.shape[1]
    for q in range(ids.shape[0]):
        dr, dm = ref_dist[q].astype(np.float64), dist[q].astype(np.float64)
        tol = tolerance(mode, case, ref_dist[q])
        if np.any(np.abs(dm - dr) > tol):
            j = int(np.argmax(np.abs(dm - dr)))
            bad.append(f"q{q} pos {j}: distance {dm[j]!r} vs reference {dr[j]!r} (tol {tol:g})")
            continue
        if np.array_equal(ids[q], ref_ids[q]):
            continue
        j = 0
        while j < k:
            e = j
            while e + 1 < k and abs(dr[e + 1] - dr[j]) <= tol:
                e += 1
            if not np.array_equal(ids[q, j:e + 1], ref_ids[q, j:e + 1]):
                same = set(ids[q, j:e + 1].tolist()) == set(ref_ids[q, j:e + 1].tolist())
                at_boundary = e == k - 1
                if not (same or at_boundary):
                    bad.append(f"q{q} pos {j}..{e}: ids {ids[q, j:e + 1].tolist()} vs reference "
                               f"{ref_ids[q, j:e + 1].tolist()} (distances {dr[j]!r}..{dr[e]!r})")
                    break
            j = e + 1
    return bad
