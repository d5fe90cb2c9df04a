"""Records the reference's own IVF-PQ / IVF-SQ8 / IVF-RaBitQ kernels' outputs
as committed fixtures (tests/golden/ivf_*.npz).

The reference's CUDA kernels for this path (kernels/src/ivf_pq_lookup.cu,
ivf_quant_lookup.cu) are compiled unchanged for sm_103a into
oracle/_ref/libfvref.so (oracle/Makefile, targets ref-stage and ref) and
driven through their C ABI (kernels/include/cuda_bridge.h:96-135) on a GPU.
Inputs are seeded and built on the CPU with the oracle's encoders (k-means,
PQ, SQ8, RaBitQ, posting lists in the reference's layout: code rows indexed
by vector id). Each fixture stores the inputs, the tables, the search
parameters and the reference's (id, distance) results, so the tests need
neither the reference nor its library.

Two inputs:
  ivf_e2e   the parameters of the reference's own IVF test
            (tests/e2e_search_test.rs:231-288): 1,500 rows of d = 96 from 12
            clusters, nlist 24, m_pq 12, k 10, nprobe 12 / 16, rerank 256 /
            512, plus single-pass (rerank <= 32), no-rerank, inner-product,
            cosine, k = 100 and 50%-mask searches; rows are rounded to
            half-precision values (stored exactly as float16);
  ivf_zipf  a small version of the 10M-row IVF-PQ benchmark: 12,000
            integer-valued rows of d = 128 in 64 lists whose sizes follow
            Zipf(1.1), m_pq 32, k 10, rerank 400, nprobe 8 / 32, a 10%
            Bernoulli mask.

Shortlists of 33..128 are left out on purpose: there the reference's stage-1
buffer (2 x next_pow2(shortlist) entries, filled by up to 256 appends per
round after a flush to `shortlist`, ivf_rerank.cuh:134-160 with
ivf_pq_lookup.cu:297-305) drops candidates in atomic order, so its output
is not a function of its inputs.

    make -C oracle ref-stage              # where the reference checkout is
    python tests/golden/make_ivf_golden.py [out_dir]   # on a GPU host
"""
from __future__ import annotations

import json
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent.parent
sys.path.insert(0, str(ROOT / "oracle"))

import oracle  # noqa: E402

RESULT = np.dtype([("id", "<u4"), ("distance", "<f4")])


def pack(bits):
    bits = np.asarray(bits, dtype=bool)
    pad = (-bits.shape[0]) % 32
    bits = np.concatenate([bits, np.zeros(pad, dtype=bool)])
    return np.packbits(bits.reshape(-1, 32), axis=1, bitorder="little").view("<u4").reshape(-1).copy()


def e2e_input():
    rng = np.random.default_rng([202, 1])
    n, dim, comps = 1500, 96, 12
    centres = rng.standard_normal((comps, dim)).astype(np.float32)
    x = centres[rng.integers(0, comps, n)] + np.float32(0.35) * rng.standard_normal((n, dim), dtype=np.float32)
    base = x.astype(np.float16)
    fresh = (centres[rng.integers(0, comps, 24)]
             + np.float32(0.35) * rng.standard_normal((24, dim), dtype=np.float32)).astype(np.float16)
    queries = np.concatenate([base[:8], fresh])  # the e2e test queries its own first 8 rows
    xf = base.astype(np.float32)
    t = oracle.build_ivf(xf, nlist=24, m_pq=12, iters=25, seed=5)
    mask = pack(rng.random(n) < 0.5)
    cases = []
    for c in ({"k": 10, "nprobe": 12, "rerank": 256, "metric": "l2", "mask": 0},    # e2e_search_test.rs:251
              {"k": 10, "nprobe": 16, "rerank": 512, "metric": "l2", "mask": 0},    # e2e_search_test.rs:271-274
              {"k": 10, "nprobe": 8, "rerank": 20, "metric": "l2", "mask": 1},      # single-pass path
              {"k": 10, "nprobe": 12, "rerank": 1, "metric": "l2", "mask": 0},      # no rerank: ADC / estimates
              {"k": 10, "nprobe": 12, "rerank": 0, "metric": "ip", "mask": 1},      # shortlist = k
              {"k": 16, "nprobe": 12, "rerank": 256, "metric": "ip", "mask": 0},
              {"k": 10, "nprobe": 12, "rerank": 256, "metric": "cosine", "mask": 0},
              {"k": 100, "nprobe": 24, "rerank": 256, "metric": "l2", "mask": 1}):
        cases.append(c)
    return {"base_f16": base, "queries_f16": queries, "mask": mask}, xf, queries.astype(np.float32), t, cases


def zipf_input():
    rng = np.random.default_rng([3, 11])
    n, dim, nlist, floor = 12000, 128, 64, 16
    comps = rng.uniform(0, 255, size=(256, dim)).astype(np.float32)
    centres = comps[rng.integers(0, 256, nlist)] + np.float32(20.0) * rng.standard_normal((nlist, dim),
                                                                                           dtype=np.float32)
    w = np.arange(1, nlist + 1, dtype=np.float64) ** -1.1
    sizes = np.maximum(floor, np.floor(n * w / w.sum())).astype(np.int64)
    sizes[0] += n - sizes.sum()
    sizes = sizes[rng.permutation(nlist)]
    lists = np.repeat(np.arange(nlist), sizes)
    x = centres[lists] + np.float32(8.0) * rng.standard_normal((n, dim), dtype=np.float32)
    base = np.clip(np.rint(x), 0, 255).astype(np.uint8)[rng.permutation(n)]
    li = rng.choice(nlist, size=48, p=sizes / sizes.sum())
    q = centres[li] + np.float32(8.0) * rng.standard_normal((48, dim), dtype=np.float32)
    queries = np.clip(np.rint(q), 0, 255).astype(np.uint8)
    xf = base.astype(np.float32)
    assign = oracle.coarse_probe(centres, xf, 1)[0][:, 0].copy()
    res = oracle.residuals(xf, centres, assign)
    offsets, vec_ids = oracle.ivf_lists(assign, nlist)
    cb = oracle.pq_train(res, 32, 10, 9)
    mins, scales = oracle.sq8_fit(res)
    t = {"centroids": centres, "assign": assign, "offsets": offsets, "vec_ids": vec_ids, "nlist": nlist,
         "codebooks": cb, "pq_codes": oracle.pq_encode(res, cb), "sq_mins": mins, "sq_scales": scales,
         "sq_codes": oracle.sq8_encode(res, mins, scales)}
    t.update(oracle.rabitq_encode(xf, centres, assign))
    mask = pack(rng.random(n) < 0.10)
    cases = [{"k": 10, "nprobe": 8, "rerank": 400, "metric": "l2", "mask": 1},
             {"k": 10, "nprobe": 32, "rerank": 400, "metric": "l2", "mask": 1},
             {"k": 10, "nprobe": 32, "rerank": 400, "metric": "l2", "mask": 0},
             {"k": 10, "nprobe": 8, "rerank": 1, "metric": "l2", "mask": 1},
             {"k": 100, "nprobe": 16, "rerank": 400, "metric": "l2", "mask": 0}]
    return {"base_u8": base, "queries_u8": queries, "mask": mask}, xf, queries.astype(np.float32), t, cases


TABLE_KEYS = ("centroids", "offsets", "vec_ids", "codebooks", "pq_codes", "sq_mins", "sq_scales", "sq_codes",
              "rot_signs", "rot_centroids", "rabitq_bits", "rabitq_meta")


def record(name, make, out_dir):
    import torch

    import refgpu

    stored, xf, qf, t, cases = make()
    q = torch.from_numpy(qf).cuda()
    mask = torch.from_numpy(stored["mask"].view(np.int32)).cuda()
    arrays = dict(stored)
    for key in TABLE_KEYS:
        arrays[key] = np.asarray(t[key])
    arrays["nlist"] = np.int32(t["nlist"])
    arrays["padded_dim"] = np.int32(t["padded_dim"])
    for mode in ("pq", "sq8", "rabitq"):
        tab = refgpu.IvfTables(mode, t, xf)
        for ci, c in enumerate(cases):
            out = torch.empty((qf.shape[0], c["k"], 2), dtype=torch.int32, device="cuda")
            rc = tab.search(q, c["k"], c["nprobe"], c["rerank"], c["metric"], mask if c["mask"] else None, out)
            torch.cuda.synchronize()
            assert rc == 0, f"reference {mode} case {ci} returned {rc}"
            r = out.cpu().numpy()
            arrays[f"{mode}_{ci}_id"] = r[..., 0].view(np.uint32).copy()
            arrays[f"{mode}_{ci}_distance"] = r[..., 1].view(np.float32).copy()
    lens = np.diff(np.asarray(t["offsets"], dtype=np.int64))
    meta = {"cases": cases, "list_len_max": int(lens.max()), "list_len_min": int(lens.min()),
            "reference_kernels": "kernels/src/ivf_pq_lookup.cu, kernels/src/ivf_quant_lookup.cu "
                                 "(-O3 --use_fast_math, sm_103a)",
            "gpu": torch.cuda.get_device_name(0)}
    arrays["meta"] = np.array(json.dumps(meta))
    out_dir.mkdir(parents=True, exist_ok=True)
    np.savez_compressed(out_dir / f"{name}.npz", **arrays)
    print(name, "cases", len(cases), "lists", meta["list_len_min"], "..", meta["list_len_max"])


def main(argv):
    out_dir = Path(argv[1]) if len(argv) > 1 else HERE
    record("ivf_e2e", e2e_input, out_dir)
    record("ivf_zipf", zipf_input, out_dir)


if __name__ == "__main__":
    main(sys.argv)
