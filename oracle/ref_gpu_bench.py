"""Times the reference's own CUDA kernels for this path on the local GPU (a
same-box baseline; TEST AND MEASUREMENT INFRASTRUCTURE, never the product).

The kernels are the reference's, compiled unchanged by `make -C oracle ref`
(oracle/Makefile) and called through their C ABI (oracle/refgpu.py) on
device-resident synthetic inputs of the benchmark shapes:

  flat_f32   cuda_flat_scan_batch (kernels/src/sparse_hybrid.cu:13-107):
             100,000 x 128 integer-valued rows (1,024-component mixture,
             centres U[0,255], sigma 20), 1,000 queries, k = 10, L2; its ids
             are compared with the oracle's exact search (exact_knn order);
  fp16_ip    cuda_fp16_tc_search_batch (kernels/src/ivf_quant_lookup.cu:
             894-1058): 1,000,000 x 768 unit vectors (4,096 components,
             sigma 0.3) as binary16, batches of 1, 64 and 1,024 queries,
             k = 10 (and k = 100 at 1,024), a Bernoulli(0.5) mask, inner
             product; recall@k against an fp64 evaluation is reported.

Each line: kernel time per call (CUDA events on the calling stream, after
one warm-up call), QPS = queries / time.

    make -C oracle ref-stage     # where the reference checkout exists
    python oracle/ref_gpu_bench.py [flat_f32] [fp16_ip]
"""
from __future__ import annotations

import json
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent
sys.path.insert(0, str(HERE))
sys.path.insert(0, str(ROOT / "flashvector-gpu_gb300"))


def _time(fn, reps):
    import torch

    fn()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(reps):
        rc = fn()
        assert rc == 0, f"reference call returned {rc}"
    e1.record()
    torch.cuda.synchronize()
    return e0.elapsed_time(e1) / reps


def bench_flat(out_lines):
    import numpy as np
    import torch

    import oracle
    import refgpu
    from fvgb300 import datasets

    n, dim, nq, k = 100_000, 128, 1000, 10
    base = datasets.sample_np(datasets.FLAT_L2_INT, n, seed=0, stream=0)
    queries = datasets.sample_np(datasets.FLAT_L2_INT, nq, seed=0, stream=1)
    b, q = torch.from_numpy(base).cuda(), torch.from_numpy(queries).cuda()
    out = torch.empty((nq, k, 2), dtype=torch.int32, device="cuda")
    ms = _time(lambda: refgpu.flat_scan(b, None, q, k, "l2", None, out), 3)
    r = out.cpu().numpy()
    ref = oracle.exact_knn(base, queries, k, "l2")
    same_ids = float((r[..., 0].view(np.uint32) == ref["id"]).mean())
    same_dist = float((r[..., 1].view(np.float32) == ref["distance"]).mean())
    out_lines.append({"kernel": "flat_scan_kernel (reference)", "workload": "flat_f32 100k x 128, Q 1000, k 10, L2",
                      "ms_per_call": ms, "qps": nq / (ms / 1e3), "ids_equal_to_exact_knn": same_ids,
                      "distances_equal_to_exact_knn": same_dist})


def bench_fp16(out_lines):
    import numpy as np
    import torch

    import refgpu
    from fvgb300 import datasets

    n, dim = 1_000_000, 768
    base = datasets.sample_torch(datasets.FP16_IP_UNIT, n, seed=1, stream=0)
    qpool = datasets.sample_torch(datasets.FP16_IP_UNIT, 1024, seed=1, stream=1)
    table = base.half().contiguous()
    norms = (base * base).sum(1).contiguous()
    words = datasets.bernoulli_mask_words(n, 0.5, seed=1)
    mask = torch.from_numpy(words.view(np.int32)).cuda()
    allowed = torch.from_numpy(datasets.unpack_words(words, n)).cuda()
    base64 = base.double()
    for nq, k, reps in ((1, 10, 2), (64, 10, 2), (1024, 10, 2), (1024, 100, 1)):
        q = qpool[:nq].contiguous()
        out = torch.empty((nq, k, 2), dtype=torch.int32, device="cuda")
        ms = _time(lambda: refgpu.fp16_search(table, norms, n, dim, dim, q, k, "ip", mask, out), reps)
        ids = out.cpu().numpy()[..., 0].view(np.uint32).astype(np.int64)
        hits = 0
        for s in range(0, nq, 256):
            d = -(q[s:s + 256].double() @ base64.T)
            d = d.masked_fill(~allowed[None, :], float("inf"))
            ti = torch.topk(d, k, dim=1, largest=False)[1].cpu().numpy()
            hits += sum(len(set(ti[r].tolist()) & set(ids[s + r].tolist())) for r in range(ti.shape[0]))
            del d
        out_lines.append({"kernel": "fp16_tc_wmma_search_kernel (reference)",
                          "workload": f"fp16_ip 1M x 768, Q {nq}, k {k}, 50% mask, IP", "ms_per_call": ms,
                          "qps": nq / (ms / 1e3), "recall_at_k_vs_fp64": hits / (nq * k)})


def main(argv):
    import torch

    which = argv[1:] or ["flat_f32", "fp16_ip"]
    lines = []
    if "flat_f32" in which:
        bench_flat(lines)
    if "fp16_ip" in which:
        bench_fp16(lines)
    for ln in lines:
        ln["gpu"] = torch.cuda.get_device_name(0)
        print(json.dumps(ln), flush=True)


if __name__ == "__main__":
    main(sys.argv)
