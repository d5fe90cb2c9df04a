"""Autotuner of the tensor-core scans and the IVF list scans; its results are
committed to flashvector-gpu_gb300/tuning/gb300.json and compiled into
libfvgb300 by build.py, where launch_tc_scan and launch_ivf_search consult
them for calls of a matching shape.

For each benchmark shape it sweeps
  * tc.pair          one-SM CTAs or cta_group::2 pairs (long rows only),
  * tc.prepass       sampled pre-pass bound on / off, and its stride,
  * over-fetch       the fp32-rescored shortlist = over-fetch x k,
times each configuration (CUDA events around the whole search call, median
of several runs, after warm-up) and measures recall@10 and recall@k against
an fp64 exact search on a query subsample. The chosen configuration is the
fastest whose recall@10 and recall@k are both >= the target (0.99); the
pair / pre-pass / stride knobs never change the answer (the tests check
this), the over-fetch can.

For each IVF benchmark shape (the 10M-row IVF-PQ / IVF-RaBitQ list scans over
Zipf-skewed lists at nprobe 8 / 32 / 128, the serving configuration's
IVF-SQ8 at nprobe 16 / 64) it sweeps
  * ivf.pipeline     the PQ list scan's plain or software-pipelined loop,
  * ivf.split        the work items of the persistent list scan: each
                     query's probed postings as one item (0), cut into 2 or
                     4 equal (query, posting-range) items merged per query
                     afterwards (2, 4), or the automatic rule (-1: ranges
                     only for batches of fewer than 4 queries per SM),
  * ivf.tc_coarse    the exact fp32 coarse probe or the tensor-core one
                     (candidates, exact rescore, proof or exact fallback),
all of which give the same answer (the tests check it), and keeps the
fastest. The tile shape of the tensor-core scans is fixed by the hardware
layout (128 TMEM lanes of queries per CTA, 256 base rows per MMA, two
accumulator buffers in the 512 TMEM columns); the CTA-pair knob is the
queries-per-tile choice (128 or 256).

    python -m fvgb300.autotune [--shapes all|fp16|fp8|ivf] [--out tuning/gb300.json]

Data: the seeded synthetic mixtures of the benchmark configurations
(fvgb300.datasets), queries fresh draws from the same mixture.
"""
from __future__ import annotations

import argparse
import dataclasses
import json
import statistics
import time
from pathlib import Path

import numpy as np

PKG = Path(__file__).resolve().parents[1]
DEFAULT_OUT = PKG / "tuning" / "gb300.json"

# precision, metric, N, dim, queries, k, mixture name, mask fraction (0 = no
# mask), over-fetch values to try: the fp16 inner-product configuration fixes
# a 4k over-fetch, the fp8 one tunes it
SHAPES = {
    "fp16_ip_1M_q1024_k10": ("fp16", "ip", 1_000_000, 768, 1024, 10, "FP16_IP_UNIT", 0.5, (4,)),
    "fp16_ip_1M_q1024_k100": ("fp16", "ip", 1_000_000, 768, 1024, 100, "FP16_IP_UNIT", 0.5, (4,)),
    "fp16_ip_1M_q64_k10": ("fp16", "ip", 1_000_000, 768, 64, 10, "FP16_IP_UNIT", 0.5, (4,)),
    "fp16_ip_1M_q1_k10": ("fp16", "ip", 1_000_000, 768, 1, 10, "FP16_IP_UNIT", 0.5, (4,)),
    "fp16_ip_1M_q64_k100": ("fp16", "ip", 1_000_000, 768, 64, 100, "FP16_IP_UNIT", 0.5, (4,)),
    "fp16_ip_1M_q1_k100": ("fp16", "ip", 1_000_000, 768, 1, 100, "FP16_IP_UNIT", 0.5, (4,)),
    "fp8_l2_10M_q10000_k100": ("fp8", "l2", 10_000_000, 96, 10_000, 100, "FP8_L2", 0.0, (4, 3, 2)),
}


# mode, N, dim, nlist, m_pq (PQ), queries, k, nprobe, rerank_k, mask fraction, rows
IVF_SHAPES = {
    f"ivf_{mode}_10M_nprobe{npb}": (mode, 10_000_000, 128, 16384, 32, 10_000, 10, npb, 400, 0.10, "zipf")
    for mode in ("pq", "rabitq") for npb in (8, 32, 128)
}
IVF_SHAPES.update({
    f"ivf_sq8_1M_768_nprobe{npb}": ("sq8", 1_000_000, 768, 4096, 0, 1024, 10, npb, 0, 0.0, "FP16_IP_UNIT_RAWMEANS")
    for npb in (16, 64)
})


def _ivf_ranges(n, dim, nlist, nq, nprobe):
    """The shape range an IVF entry applies to: base within 4x, nlist within
    2x, dimension within 1.5x, batch within 2x (batches of 1-64 form one
    range), nprobe halfway to the neighbouring tuned values."""
    nq_range = [1, 64] if nq <= 64 else [nq // 2, nq * 2]
    np_range = [max(1, (nprobe * 2) // 3), min(256, nprobe + nprobe // 2)]
    return {"dim": [max(1, int(dim / 1.5)), int(dim * 1.5)], "n": [max(1, n // 4), n * 4],
            "nlist": [max(1, nlist // 2), nlist * 2], "nq": nq_range, "nprobe": np_range}


def tune_ivf_shape(name, spec, runs=3, nsub=100, log=print):
    import ctypes as C

    import torch

    from . import _lib, datasets, scan
    from .index import BUILD_IVF_PQ, BUILD_IVF_RABITQ, BUILD_IVF_SQ8, GpuVectorIndex, IndexConfig

    mode, n, dim, nlist, m_pq, nq, k, nprobe, rerank, mask_frac, rows_kind = spec
    dev = torch.device("cuda", 0)
    metric = "l2" if rows_kind == "zipf" else "ip"
    if rows_kind == "zipf":
        rows, centers, qgen, _ = datasets.zipf_ivf_data(n, dim, nlist, 3, dev)
        queries = qgen(nq, 4242).contiguous()
        flags = {"pq": BUILD_IVF_PQ, "rabitq": BUILD_IVF_RABITQ}[mode]
        idx = GpuVectorIndex(IndexConfig(dim=dim, nlist=nlist, m_pq=m_pq, metric=metric, build_flags=flags,
                                         kmeans_iters_given=2, train_rows=min(n, 4 * nlist * 64), pq_iters=10,
                                         seed=3))
        idx.build_device(rows, centers)
    else:
        mix = getattr(datasets, rows_kind)
        rows = datasets.sample_torch(mix, n, seed=1, stream=0, device=dev)
        queries = datasets.sample_torch(mix, nq, seed=1, stream=1, device=dev).contiguous()
        idx = GpuVectorIndex(IndexConfig(dim=dim, nlist=nlist, metric=metric, build_flags=BUILD_IVF_SQ8,
                                         kmeans_iters=6, train_rows=min(n, 262144), seed=4))
        idx.build_device(rows)
    torch.cuda.synchronize()
    if mode == "rabitq":
        tab, opt = idx.rabitq_tables()
    else:
        pq_t, sq_t, opt = idx.ivf_tables()
        tab = pq_t if mode == "pq" else sq_t
    fn = {"pq": "fv_ivf_pq_search_ex", "sq8": "fv_ivf_sq_search_ex", "rabitq": "fv_ivf_rabitq_search_ex"}[mode]
    mask = allowed = None
    if mask_frac > 0:
        words = datasets.bernoulli_mask_words(n, mask_frac, seed=3)
        mask = torch.from_numpy(words.view(np.int32)).to(dev)
        allowed = torch.from_numpy(datasets.unpack_words(words, n)).to(dev)
    truth = _fp64_topk(rows, queries[:nsub], k, metric, allowed)
    out = scan.empty_results(nq, k, dev)
    stream = torch.cuda.current_stream()

    def search():
        _lib.call(fn, C.byref(tab), C.byref(opt), C.c_void_p(queries.data_ptr()), nq, k, nprobe, rerank,
                  {"l2": 0, "ip": 2}[metric], None if mask is None else C.c_void_p(mask.data_ptr()),
                  C.c_void_p(out.data_ptr()), C.c_void_p(stream.cuda_stream))

    results, answer = [], None
    for pipeline in ((0, 1) if mode == "pq" else (0,)):
        for split in (-1, 0, 2, 4):
            for tcc in (0, 1):
                with scan.tuned(tc_table=0, ivf_pipeline=pipeline, ivf_split=split, ivf_tc_coarse=tcc):
                    for _ in range(2):
                        search()
                    torch.cuda.synchronize()
                    times = []
                    for _ in range(runs):
                        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                        e0.record(stream)
                        search()
                        e1.record(stream)
                        e1.synchronize()
                        times.append(e0.elapsed_time(e1))
                res = out.clone()
                same = answer is None or torch.equal(res, answer)
                answer = res if answer is None else answer
                ms = statistics.median(times)
                results.append({"pipeline": pipeline, "split": split, "tc_coarse": tcc, "ms": ms, "same_answer": same})
                log(f"{name} pipeline {pipeline} split {split} tc_coarse {tcc}: {ms:.3f} ms same {same}")
    ids = answer.cpu().numpy()[..., 0].view(np.uint32)
    best = min(results, key=lambda r: r["ms"])
    default = next(r for r in results if r["pipeline"] == 0 and r["split"] == -1 and r["tc_coarse"] == 0)
    del idx
    torch.cuda.empty_cache()
    return {"name": name, "mode": mode, **_ivf_ranges(n, dim, nlist, nq, nprobe),
            "shape": {"n": n, "dim": dim, "nlist": nlist, "m_pq": m_pq, "nq": nq, "k": k, "nprobe": nprobe,
                      "rerank_k": rerank, "mask_fraction": mask_frac, "rows": rows_kind},
            "knobs": {"pipeline": best["pipeline"], "split": best["split"], "tc_coarse": best["tc_coarse"]},
            "measured": {"ms": best["ms"], "qps": nq / (best["ms"] / 1e3), "untuned_ms": default["ms"],
                         "recall_at_k": _recall(ids[:nsub], truth), "all_answers_equal":
                             all(r["same_answer"] for r in results), "candidates": len(results)}}


def _ranges(n, dim, nq, k):
    """The shape range an entry applies to: dimension within 1.5x, base size
    within 4x, batch within 2x (batches of 1-16 queries form one range),
    k within 2x."""
    nq_range = [1, 16] if nq <= 16 else [nq // 2, nq * 2]
    return {"dim": [max(1, int(dim / 1.5)), int(dim * 1.5)], "n": [max(1, n // 4), n * 4],
            "nq": nq_range, "k": [max(1, k // 2), min(256, k * 2)]}


def _candidates(precision, dim, overfetches):
    long_rows = (dim + (127 if precision == "fp8" else 63)) // (128 if precision == "fp8" else 64) > 2
    pairs = [1, 0] if long_rows else [0]
    prepasses = [(0, 0), (1, 16), (1, 32), (1, 64)]
    for overfetch in overfetches:
        for pair in pairs:
            for prepass, stride in prepasses:
                yield {"pair": pair, "prepass": prepass, "stride": stride, "overfetch": overfetch}


def tune_shape(name, spec, runs=5, nsub=100, target=0.99, log=print):
    import torch

    from . import datasets, scan

    precision, metric, n, dim, nq, k, mix_name, mask_frac, overfetches = spec
    dev = torch.device("cuda", 0)
    mix = dataclasses.replace(getattr(datasets, mix_name), dim=dim)
    base = datasets.sample_torch(mix, n, seed=11, stream=0, device=dev)
    queries = datasets.sample_torch(mix, nq, seed=11, stream=1, device=dev).contiguous()
    table = (scan.Fp8Table if precision == "fp8" else scan.Fp16Table)(base)
    search = scan.fp8_search if precision == "fp8" else scan.fp16_search
    mask = allowed = None
    if mask_frac > 0:
        words = datasets.bernoulli_mask_words(n, mask_frac, seed=1)
        mask = torch.from_numpy(words.view(np.int32)).to(dev)
        allowed = torch.from_numpy(datasets.unpack_words(words, n)).to(dev)
    truth = _fp64_topk(base, queries[:nsub], k, metric, allowed)
    out = scan.empty_results(nq, k, dev)
    stream = torch.cuda.current_stream()
    results = []
    for cand in _candidates(precision, dim, overfetches):
        knobs = {"tc_table": 0, "tc_pair": cand["pair"], "tc_prepass": cand["prepass"],
                 "tc_prepass_stride": cand["stride"] or 32}
        opts = scan.options(overfetch=cand["overfetch"], boundary_fp64=1)
        with scan.tuned(**knobs):
            for _ in range(2):
                search(table, queries, k, metric, mask=mask, opts=opts, out=out)
            torch.cuda.synchronize()
            times = []
            for _ in range(runs):
                e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                e0.record(stream)
                search(table, queries, k, metric, mask=mask, opts=opts, out=out)
                e1.record(stream)
                e1.synchronize()
                times.append(e0.elapsed_time(e1))
        res = out.cpu().numpy()
        ids = res[..., 0].view(np.uint32)
        r10 = _recall(ids[:nsub, :10], truth[:, :10])
        rk = _recall(ids[:nsub], truth)
        ms = statistics.median(times)
        results.append({**cand, "ms": ms, "qps": nq / (ms / 1e3), "recall_at_10": r10, "recall_at_k": rk})
        log(f"{name} {cand} {ms:.3f} ms recall@10 {r10:.4f} recall@{k} {rk:.4f}")
    ok = [r for r in results if r["recall_at_10"] >= target and r["recall_at_k"] >= target]
    best = min(ok or results, key=lambda r: r["ms"])
    default = next(r for r in results if r["overfetch"] == 4 and r["prepass"] == 0 and r["pair"] == 0)
    return {"name": name, "precision": precision, "metric": metric, **_ranges(n, dim, nq, k),
            "shape": {"n": n, "dim": dim, "nq": nq, "k": k, "mask_fraction": mask_frac},
            "knobs": {"pair": best["pair"], "prepass": best["prepass"], "stride": best["stride"],
                      "overfetch": best["overfetch"]},
            "measured": {"ms": best["ms"], "qps": best["qps"], "recall_at_10": best["recall_at_10"],
                         "recall_at_k": best["recall_at_k"], "untuned_ms": default["ms"],
                         "recall_target": target, "candidates": len(results)}}


def _fp64_topk(base, queries, k, metric, allowed, chunk=500_000):
    import torch

    q64 = queries.double()
    best_d = best_i = None
    for c in range(0, base.shape[0], chunk):
        x = base[c:c + chunk].double()
        if metric == "l2":
            d = (q64 * q64).sum(1, keepdim=True) + (x * x).sum(1)[None, :] - 2.0 * (q64 @ x.T)
        else:
            d = -(q64 @ x.T)
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


def _recall(ids, truth):
    k = truth.shape[1]
    return float(sum(len(set(ids[i, :k].tolist()) & set(truth[i].tolist())) for i in range(truth.shape[0]))
                 / (truth.shape[0] * k))


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__, formatter_class=argparse.RawDescriptionHelpFormatter)
    ap.add_argument("--shapes", default="all", help="all, fp16, fp8 or a comma-separated list of shape names")
    ap.add_argument("--out", default=str(DEFAULT_OUT))
    ap.add_argument("--runs", type=int, default=5)
    a = ap.parse_args(argv)
    import torch

    every = list(SHAPES) + list(IVF_SHAPES)
    if a.shapes == "all":
        names = every
    elif a.shapes in ("fp16", "fp8", "ivf"):
        names = [s for s in every if s.startswith(a.shapes)]
    else:
        names = a.shapes.split(",")
    entries = [tune_shape(nm, SHAPES[nm], runs=a.runs) for nm in names if nm in SHAPES]
    ivf_entries = [tune_ivf_shape(nm, IVF_SHAPES[nm]) for nm in names if nm in IVF_SHAPES]
    out = Path(a.out)
    prev = json.loads(out.read_text()) if out.exists() else {"entries": []}
    keep = [e for e in prev.get("entries", []) if e.get("name") not in {x["name"] for x in entries}]
    keep_ivf = [e for e in prev.get("ivf_entries", []) if e.get("name") not in {x["name"] for x in ivf_entries}]
    doc = {"device": torch.cuda.get_device_name(0), "date": time.strftime("%Y-%m-%d"),
           "method": "fastest configuration with recall@10 and recall@k >= target vs fp64 exact search "
                     "(median of CUDA-event times around the whole search call)",
           "entries": keep + entries,
           "ivf_method": "fastest of the knob settings, all of which return the same answer (median of CUDA-event "
                         "times around the whole search call)",
           "ivf_entries": keep_ivf + ivf_entries}
    out.parent.mkdir(parents=True, exist_ok=True)
    out.write_text(json.dumps(doc, indent=1) + "\n")
    print(f"wrote {len(doc['entries'])} entries to {out}")


if __name__ == "__main__":
    main()
