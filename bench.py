#!/usr/bin/env python3
"""Benchmark of the GB300 distance-scan path (one JSON line on rank 0).

Workload (the configuration the headline metric is quoted on): FP16
tensor-core flat inner-product scan with fp32 rescore of a 4k over-fetched
shortlist and fp64 boundary re-rank; N = 1,000,000 unit-normalised vectors
of d = 768 from a 4,096-component Gaussian mixture (sigma 0.3), 1,024-query
batches from the same mixture, k = 10, a Bernoulli(0.5) slot bitmask.
Synthetic data of that shape stands in for the benchmark corpus.

A step is one call of the drop-in entry point cuda_fp16_tc_search_batch over
one batch. `value` times K steps with the queries already in HBM (CUDA
events on the call's stream); `e2e` times K steps that each copy the batch
from pinned host memory, search, and copy the results back. The base set
(1.54 GB fp16 + 3.07 GB fp32) is far larger than L2, so no flush is needed.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]
"""
from __future__ import annotations

import argparse
import dataclasses
import json
import os
import statistics
import subprocess
import sys
import threading
import time
from pathlib import Path

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT / "flashvector-gpu_gb300"))

METRIC = "QPS at recall@10>=0.99 vs FP64 exact, FP8/FP16+rescore vs FP32 scan; p99 ms"
UNIT = "QPS"
WORKLOAD = "fp16 tensor-core flat IP scan + fp32 rescore (4k over-fetch) + fp64 boundary, 50% bitmask"


def parse_args():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--n", type=int, default=1_000_000)
    ap.add_argument("--dim", type=int, default=768)
    ap.add_argument("--batch", type=int, default=1024)
    ap.add_argument("--k", type=int, default=10)
    ap.add_argument("--overfetch", type=int, default=4)
    ap.add_argument("--cpu-seconds", type=float, default=12.0, help="budget of the CPU baseline sample")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    return ap.parse_args()


def config(a, extra=None):
    c = {"workload": WORKLOAD, "N": a.n, "dim": a.dim, "batch": a.batch, "k": a.k, "overfetch": a.overfetch,
         "mask_valid_fraction": 0.5, "metric": "inner_product", "mixture": "4096 comps, sigma 0.3, unit norm",
         "l2": "inputs larger than L2 (fp16 base 1.54 GB streamed per step)", "parallelism": "replicas"}
    if extra:
        c.update(extra)
    return c


# --------------------------------------------------------------- clocks
class ClockSampler:
    FIELDS = ["clocks.sm", "clocks.max.sm", "clocks_event_reasons.active", "clocks_event_reasons.hw_slowdown",
              "clocks_event_reasons.hw_thermal_slowdown", "clocks_event_reasons.sw_thermal_slowdown",
              "clocks_event_reasons.sw_power_cap"]

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.lines: list[str] = []
        self.thread = None

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), f"--query-gpu={','.join(self.FIELDS)}",
                 "--format=csv,noheader,nounits", "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL,
                text=True)
        except OSError:
            self.proc = None
            return
        self.thread = threading.Thread(target=self._read, daemon=True)
        self.thread.start()

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self) -> dict:
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        if self.thread:
            self.thread.join(timeout=2)
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 7:
                continue
            try:
                sm.append(float(parts[0]))
                mx.append(float(parts[1]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[3:7]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(sm)}


# --------------------------------------------------------- distributed
def dist_setup():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


def measured_peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        try:
            return json.loads(p.read_text()), "measured"
        except ValueError:
            pass
    return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0, "bf16_tflops_sustained": 1700.0}, "fallback"


def profile_traffic():
    """dram bytes per launch of the scan kernel from the committed ncu
    summary (null when no capture has been summarised yet)."""
    p = ROOT / "profiles" / "tc_scan_fp16_traffic.json"
    if p.exists():
        try:
            return json.loads(p.read_text())
        except ValueError:
            return None
    return None


# ------------------------------------------------------------ CPU legs
def cpu_exact_sample(base_np, queries_np, mask_words, k, budget_s, threads):
    """The reference's exact search restated on the host (oracle port, IP in
    metrics.rs:103-135's summation order), on a bounded query sample."""
    sys.path.insert(0, str(ROOT / "oracle"))
    import oracle

    oracle.build()
    t0 = time.perf_counter()
    oracle.exact_knn(base_np, queries_np[:threads], k, "ip", mask=mask_words, threads=threads)
    per = (time.perf_counter() - t0) / threads
    nq = int(max(threads, min(queries_np.shape[0], budget_s / max(per, 1e-9))))
    nq = max(threads, nq // threads * threads)
    t0 = time.perf_counter()
    oracle.exact_knn(base_np, queries_np[:nq], k, "ip", mask=mask_words, threads=threads)
    dt = time.perf_counter() - t0
    return nq / dt, nq, dt


def run_reference(a, world, rank):
    if rank != 0:
        return
    import numpy as np

    from fvgb300 import datasets

    threads = os.cpu_count() or 1
    mix = dataclasses.replace(datasets.FP16_IP_UNIT, dim=a.dim)
    base = datasets.sample_np(mix, a.n, seed=1, stream=0)
    queries = datasets.sample_np(mix, a.batch, seed=1, stream=1)
    words = datasets.bernoulli_mask_words(a.n, 0.5, seed=1)
    sys.path.insert(0, str(ROOT / "oracle"))
    import oracle

    oracle.build()
    per_step = threads
    for w in range(max(a.warmup, 0)):
        if w >= 1:
            break  # one untimed call warms caches; more would only burn CPU
        oracle.exact_knn(base, queries[:per_step], a.k, "ip", mask=words, threads=threads)
    t0 = time.perf_counter()
    done = 0
    for s in range(a.steps):
        lo = (s * per_step) % max(1, a.batch - per_step + 1)
        oracle.exact_knn(base, queries[lo:lo + per_step], a.k, "ip", mask=words, threads=threads)
        done += per_step
    dt = time.perf_counter() - t0
    qps = done / dt
    line = {"impl": "reference", "metric": METRIC, "value": qps, "unit": UNIT, "n_gpus": world, "steps": a.steps,
            "warmup": a.warmup, "ms_per_step": dt / a.steps * 1e3, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": config(a, {"reference_sample": f"{per_step} queries per step against the full base"}),
            "cpu_baseline": {"value": qps, "unit": UNIT, "cores": threads, "kind": "port",
                             "sample": f"{done} queries ({per_step} per step x {a.steps} steps), exact fp32 "
                                       f"search of the full {a.n} x {a.dim} base on {threads} host threads"},
            "e2e": {"value": qps, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


# ---------------------------------------------------------------- ours
def run_ours(a, world, rank, local):
    import numpy as np
    import torch

    import build as fv_build

    fv_build.build()
    from fvgb300 import datasets, scan

    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl", device_id=dev)
    stream = torch.cuda.current_stream()

    mix = dataclasses.replace(datasets.FP16_IP_UNIT, dim=a.dim)
    base = datasets.sample_torch(mix, a.n, seed=1, stream=0, device=dev)
    nbatches = 4
    qpool = datasets.sample_torch(mix, a.batch * nbatches, seed=1, stream=1, device=dev)
    batches = [qpool[i * a.batch:(i + 1) * a.batch].contiguous() for i in range(nbatches)]
    words = datasets.bernoulli_mask_words(a.n, 0.5, seed=1)
    mask = torch.from_numpy(words.view(np.int32)).to(dev)
    table = scan.Fp16Table(base)
    opts = scan.options(overfetch=a.overfetch, boundary_fp64=1)
    out = scan.empty_results(a.batch, a.k, dev)

    def step(i, q=None):
        scan.fp16_search(table, batches[i % nbatches] if q is None else q, a.k, "ip", mask=mask, opts=opts, out=out,
                         dropin=(a.overfetch == 4))

    for i in range(max(a.warmup, 3)):
        step(i)
    torch.cuda.synchronize()

    def barrier():
        if world > 1:
            import torch.distributed as dist

            dist.barrier()

    # ---- device-resident timed region
    clocks = ClockSampler(local)
    clocks.start()
    time.sleep(0.3)
    barrier()
    torch.cuda.synchronize()
    scan.profile_summary()
    scan.profile_enable(True)
    l0 = scan.launch_count()
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    ev0.record(stream)
    for i in range(a.steps):
        step(i)
    ev1.record(stream)
    torch.cuda.synchronize()
    launches = scan.launch_count() - l0
    scan.profile_enable(False)
    prof = scan.profile_summary()
    barrier()
    clk = clocks.stop()
    dev_ms = ev0.elapsed_time(ev1)

    # ---- end-to-end through the C ABI with host buffers
    host_q = [b.cpu().pin_memory() for b in batches]
    host_out = torch.empty(out.shape, dtype=out.dtype).pin_memory()
    dq = torch.empty_like(batches[0])
    for i in range(2):
        dq.copy_(host_q[i % nbatches], non_blocking=True)
        step(i, dq)
        host_out.copy_(out, non_blocking=True)
    torch.cuda.synchronize()
    barrier()
    t0 = time.perf_counter()
    for i in range(a.steps):
        dq.copy_(host_q[i % nbatches], non_blocking=True)
        step(i, dq)
        host_out.copy_(out, non_blocking=True)
    torch.cuda.synchronize()
    e2e_s = time.perf_counter() - t0
    barrier()

    # ---- max over ranks
    times = torch.tensor([dev_ms / 1e3, e2e_s], dtype=torch.float64, device=dev)
    if world > 1:
        import torch.distributed as dist

        dist.all_reduce(times, op=dist.ReduceOp.MAX)
    dev_s, e2e_s = times.tolist()
    total_q = a.batch * a.steps * world
    qps = total_q / dev_s
    e2e_qps = total_q / e2e_s

    # ---- recall@10 and distance error against an fp64 evaluation on device
    step(0)
    torch.cuda.synchronize()
    res = out.cpu().numpy()
    ids = res[..., 0].view(np.uint32).astype(np.int64)
    dist32 = res[..., 1].view(np.float32)
    allowed = torch.from_numpy(datasets.unpack_words(words, a.n)).to(dev)
    q64 = batches[0].double()
    hits, maxerr = 0, 0.0
    for s in range(0, a.batch, 128):
        dots = q64[s:s + 128] @ base.double().T if a.n <= 200_000 else torch.cat(
            [q64[s:s + 128] @ base[c:c + 200_000].double().T for c in range(0, a.n, 200_000)], dim=1)
        d = (-dots).masked_fill(~allowed[None, :], float("inf"))
        tv, ti = torch.topk(d, a.k, dim=1, largest=False)
        ti = ti.cpu().numpy()
        for r in range(ti.shape[0]):
            hits += len(set(ti[r].tolist()) & set(ids[s + r].tolist()))
        got = d.gather(1, torch.from_numpy(ids[s:s + 128]).to(dev).clamp_max(a.n - 1))
        maxerr = max(maxerr, float((got - torch.from_numpy(dist32[s:s + 128]).to(dev).double()).abs().max()))
        del dots, d
    recall = hits / (a.batch * a.k)

    if rank != 0:
        return
    peaks, peak_kind = measured_peaks()
    scan_name = "tc_scan_fp16"
    scan_ms = prof.get(scan_name, {}).get("ms", 0.0) / max(1, prof.get(scan_name, {}).get("launches", 1))
    flops = 2.0 * a.n * a.dim * a.batch
    achieved = flops / (scan_ms / 1e3) / 1e12 if scan_ms > 0 else None
    peak = peaks.get("bf16_tflops")
    traffic = profile_traffic()
    roof = {"bound": "tensor", "achieved": achieved, "peak": peak, "unit": "TFLOP/s",
            "frac": (achieved / peak) if achieved and peak else None,
            "traffic": traffic.get("bytes_per_launch") if traffic else None,
            "kernel": scan_name, "kernel_ms": scan_ms, "algorithmic_flops_per_launch": flops,
            "peak_source": f"{peak_kind} dense bf16 burst (fp16 dense rate is the same)"}
    kernels = {k: {"launches": v["launches"], "ms_per_launch": v["ms"] / max(1, v["launches"])} for k, v in prof.items()}

    cpu = None
    if not a.no_cpu_baseline:
        threads = os.cpu_count() or 1
        base_np = base.cpu().numpy()
        q_np = batches[0].cpu().numpy()
        cqps, cnq, cdt = cpu_exact_sample(base_np, q_np, words, a.k, a.cpu_seconds, threads)
        cpu = {"value": cqps, "unit": UNIT, "cores": threads, "kind": "port",
               "sample": f"{cnq} of the {a.batch} queries, exact fp32 search of the full base, {cdt:.1f} s"}

    line = {"metric": METRIC, "value": qps, "unit": UNIT, "n_gpus": world, "steps": a.steps, "warmup": a.warmup,
            "ms_per_step": dev_s / a.steps * 1e3, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f16", "data": "synthetic", "config": config(a),
            "recall_at_k": recall, "max_dist_err_vs_fp64": maxerr,
            "e2e": {"value": e2e_qps, "unit": UNIT, "h2d_bytes_per_step": a.batch * a.dim * 4,
                    "d2h_bytes_per_step": a.batch * a.k * 8, "ms_per_step": e2e_s / a.steps * 1e3},
            "gpu_launches": launches, "roofline": roof, "kernels": kernels, "clocks": clk, "cpu_baseline": cpu}
    print(json.dumps(line), flush=True)
    if world > 1:
        import torch.distributed as dist

        dist.destroy_process_group()


def main():
    a = parse_args()
    world, rank, local = dist_setup()
    if a.impl == "reference":
        run_reference(a, world, rank)
    else:
        run_ours(a, world, rank, local)


if __name__ == "__main__":
    main()
