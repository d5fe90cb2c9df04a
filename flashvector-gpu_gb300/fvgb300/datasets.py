"""Seeded synthetic workloads with the shapes and value distributions of the
scan path's benchmark configurations (no public dataset is used).

Each generator draws a Gaussian mixture: component centres first (from the
seed), then for every row an independently drawn component id plus isotropic
noise, so rows of one component are scattered through the base set the way
a real corpus is. Queries are fresh draws from the same mixture (never
copies of base rows).

Two backends: numpy (CPU, any size that fits in host memory) and torch on a
CUDA device (for the multi-GB benchmark sets). They use different random
streams, so the same seed gives the same distribution, not the same bits.
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np


@dataclass(frozen=True)
class Mixture:
    dim: int
    components: int
    sigma: float
    center_kind: str   # "uniform255" | "normal"
    post: str          # "int255" (round+clip to [0,255]) | "unit" (L2-normalise) | "none"
    center_norm: bool = False  # normalise the component means


# Plain exact flat L2: integers in [0, 255] from 1,024 components, sigma 20.
FLAT_L2_INT = Mixture(dim=128, components=1024, sigma=20.0, center_kind="uniform255", post="int255")
# FP16 flat inner product: unit vectors from 4,096 components, sigma 0.3.
FP16_IP_UNIT = Mixture(dim=768, components=4096, sigma=0.3, center_kind="normal", post="unit", center_norm=True)
# The same shape with the component means left un-normalised (N(0, I),
# norm ~ sqrt(768)): the configuration's text leaves the means unspecified;
# against these means the sigma 0.3 noise is small, so rows cluster tightly
# (the convention of the fp8 configuration's mixture).
FP16_IP_UNIT_RAWMEANS = Mixture(dim=768, components=4096, sigma=0.3, center_kind="normal", post="unit")
# FP8 flat L2: 16,384 components with N(0,1) means, sigma 0.5.
FP8_L2 = Mixture(dim=96, components=16384, sigma=0.5, center_kind="normal", post="none")


def _centers_np(m: Mixture, rng: np.random.Generator) -> np.ndarray:
    if m.center_kind == "uniform255":
        c = rng.uniform(0.0, 255.0, size=(m.components, m.dim)).astype(np.float32)
    else:
        c = rng.standard_normal((m.components, m.dim), dtype=np.float32)
    if m.center_norm:
        c /= np.maximum(np.linalg.norm(c, axis=1, keepdims=True), 1e-12)
    return c


def _post_np(x: np.ndarray, m: Mixture) -> np.ndarray:
    if m.post == "int255":
        np.rint(x, out=x)
        np.clip(x, 0.0, 255.0, out=x)
    elif m.post == "unit":
        x /= np.maximum(np.linalg.norm(x, axis=1, keepdims=True), 1e-12)
    return x


def sample_np(m: Mixture, n: int, seed: int, stream: int = 0, chunk: int = 1 << 18) -> np.ndarray:
    """n rows of mixture m (numpy). stream 0 = base set, 1 = queries."""
    centers = _centers_np(m, np.random.default_rng([seed, 0]))
    rng = np.random.default_rng([seed, 1 + stream])
    out = np.empty((n, m.dim), dtype=np.float32)
    for s in range(0, n, chunk):
        e = min(n, s + chunk)
        comp = rng.integers(0, m.components, size=e - s)
        x = centers[comp] + np.float32(m.sigma) * rng.standard_normal((e - s, m.dim), dtype=np.float32)
        out[s:e] = _post_np(x, m)
    return out


def sample_torch(m: Mixture, n: int, seed: int, stream: int = 0, device="cuda", chunk: int = 1 << 20):
    """n rows of mixture m generated on a torch device (fp32, row-major)."""
    import torch

    g = torch.Generator(device=device)
    g.manual_seed(seed * 1000003 + 17)
    if m.center_kind == "uniform255":
        centers = torch.rand((m.components, m.dim), generator=g, device=device) * 255.0
    else:
        centers = torch.randn((m.components, m.dim), generator=g, device=device)
    if m.center_norm:
        centers = centers / centers.norm(dim=1, keepdim=True).clamp_min(1e-12)
    g.manual_seed(seed * 1000003 + 101 + stream)
    out = torch.empty((n, m.dim), dtype=torch.float32, device=device)
    for s in range(0, n, chunk):
        e = min(n, s + chunk)
        comp = torch.randint(0, m.components, (e - s,), generator=g, device=device)
        x = centers[comp] + m.sigma * torch.randn((e - s, m.dim), generator=g, device=device)
        if m.post == "int255":
            x = x.round_().clamp_(0.0, 255.0)
        elif m.post == "unit":
            x = x / x.norm(dim=1, keepdim=True).clamp_min(1e-12)
        out[s:e] = x
    return out


def bernoulli_mask_words(n: int, p_valid: float, seed: int) -> np.ndarray:
    """Packed LSB-first validity words with each slot valid with prob p_valid."""
    rng = np.random.default_rng([seed, 77])
    bits = rng.random(n) < p_valid
    return pack_bools(bits)


def pack_bools(bits) -> np.ndarray:
    """bool[n] -> uint32[ceil(n/32)], bit i&31 of word i>>5 (py_index.rs:73-81)."""
    bits = np.asarray(bits, dtype=bool)
    n = bits.shape[0]
    pad = (-n) % 32
    if pad:
        bits = np.concatenate([bits, np.zeros(pad, dtype=bool)])
    return np.packbits(bits.reshape(-1, 32), axis=1, bitorder="little").view("<u4").reshape(-1).copy()


def unpack_words(words, n: int) -> np.ndarray:
    w = np.ascontiguousarray(words, dtype="<u4")
    return np.unpackbits(w.view(np.uint8), bitorder="little")[:n].astype(bool)


def zipf_ivf_data(n, dim, nlist, seed, device):
    """Rows around 16,384 list centres whose sizes follow Zipf(1.1) with a
    floor of 64; list centres scattered around the 1,024 components of the
    integer-valued mixture (centres U[0,255], sigma 20); rows rounded and
    clipped to [0, 255]. Returns (rows, list centres, queries sampler)."""
    import torch

    rng = np.random.default_rng([seed, 3])
    comps = rng.uniform(0, 255, size=(1024, dim)).astype(np.float32)
    centers = comps[rng.integers(0, 1024, size=nlist)] + np.float32(20.0) * rng.standard_normal((nlist, dim),
                                                                                              dtype=np.float32)
    w = np.arange(1, nlist + 1, dtype=np.float64) ** -1.1
    sizes = np.maximum(64, np.floor(n * w / w.sum())).astype(np.int64)
    excess = int(sizes.sum() - n)
    order = np.argsort(-sizes)
    i = 0
    while excess != 0:  # take the excess from (or give the deficit to) the largest lists
        j = order[i % 8]
        d = min(excess, sizes[j] - 64) if excess > 0 else excess
        sizes[j] -= d
        excess -= d
        i += 1
    sizes = sizes[rng.permutation(nlist)]
    c_dev = torch.from_numpy(centers).to(device)
    lists = torch.repeat_interleave(torch.arange(nlist, device=device), torch.from_numpy(sizes).to(device))
    g = torch.Generator(device=device)
    g.manual_seed(seed * 7919 + 11)
    rows = torch.empty((n, dim), dtype=torch.float32, device=device)
    for s in range(0, n, 1 << 20):
        e = min(n, s + (1 << 20))
        x = c_dev[lists[s:e]] + 8.0 * torch.randn((e - s, dim), generator=g, device=device)
        rows[s:e] = x.round_().clamp_(0.0, 255.0)
    perm = torch.randperm(n, generator=g, device=device)
    rows = rows[perm].contiguous()
    probs = torch.from_numpy(sizes.astype(np.float64) / sizes.sum()).to(device)

    def queries(count, qseed):
        gq = torch.Generator(device=device)
        gq.manual_seed(qseed)
        li = torch.multinomial(probs, count, replacement=True, generator=gq)
        return (c_dev[li] + 8.0 * torch.randn((count, dim), generator=gq, device=device)).round_().clamp_(0.0, 255.0)

    return rows, c_dev, queries, sizes
