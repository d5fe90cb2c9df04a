"""Generates the golden search fixtures of tests/golden/ from the reference's
own Python brute-force backend.

The reference ships no golden files; its python/tests_adapters/fake_backend.py
(FakeBackend: float64 brute force, stable argsort so ties go to the lower
id, boolean filter mask) is the one piece of its search semantics that runs
here. This script imports it from a reference checkout, runs it on small
seeded inputs and stores inputs and outputs as .npz fixtures. The tests then
pin the oracle and the CUDA path against those files; the reference checkout
is not needed after the fixtures exist.

    python tests/golden/make_golden.py /path/to/FlashVector-GPU
"""
from __future__ import annotations

import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent


def load_fake_backend(ref_root: Path):
    sys.path.insert(0, str(ref_root / "python" / "tests_adapters"))
    import fake_backend  # noqa: E402

    return fake_backend.FakeBackend


def mixture(rng, n, dim, comps, sigma, kind):
    if kind == "int255":
        c = rng.uniform(0, 255, size=(comps, dim))
    else:
        c = rng.standard_normal((comps, dim))
    x = c[rng.integers(0, comps, size=n)] + sigma * rng.standard_normal((n, dim))
    if kind == "int255":
        x = np.clip(np.rint(x), 0, 255)
    elif kind == "unit":
        x /= np.linalg.norm(x, axis=1, keepdims=True)
    return x.astype(np.float32)


def make_case(FB, name, seed, n, nq, dim, k, metric, kind, comps, sigma, p_valid):
    rng = np.random.default_rng(seed)
    base = mixture(rng, n, dim, comps, sigma, kind)
    queries = mixture(rng, nq, dim, comps, sigma, kind)
    if kind == "int255":
        # force exact duplicates so the lower-id tie rule is exercised
        base[n // 2: n // 2 + 8] = base[n // 3]
    mask = rng.random(n) < p_valid
    fb = FB(dim, metric=metric)
    fb.build(base)
    labels, dists = fb.search(queries, top_k=k)
    labels_m, dists_m = fb.search(queries, top_k=k, filter_mask=mask)
    np.savez_compressed(HERE / f"{name}.npz", base=base, queries=queries, k=np.int32(k),
                        metric=np.array(metric), mask=mask, labels=labels, dists=dists, labels_masked=labels_m,
                        dists_masked=dists_m)
    print(name, base.shape, queries.shape, k, metric)


def main(argv):
    if len(argv) != 2:
        sys.exit("usage: python tests/golden/make_golden.py /path/to/FlashVector-GPU")
    FB = load_fake_backend(Path(argv[1]))
    make_case(FB, "flat_l2_int", 11, 2500, 32, 128, 10, "l2", "int255", 64, 20.0, 0.5)
    make_case(FB, "flat_l2_int_k100", 12, 2500, 16, 33, 100, "l2", "int255", 16, 8.0, 0.3)
    make_case(FB, "flat_ip_unit", 13, 2000, 32, 96, 16, "ip", "unit", 64, 0.3, 0.5)
    make_case(FB, "flat_cos", 14, 2000, 24, 64, 12, "cosine", "normal", 32, 0.4, 0.7)


if __name__ == "__main__":
    main(sys.argv)
