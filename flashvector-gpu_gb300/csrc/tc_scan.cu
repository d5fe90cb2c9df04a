// tc_scan.cu -- tensor-core flat scan (FP16 and FP8-E4M3) fused with top-k,
// followed by an exact fp32 rescore of an over-fetched shortlist and an
// fp64 re-rank of the candidates that straddle the k-th distance.
//
// Replaces the reference's fp16_tc_wmma_search_kernel / launch_fp16_tc_search
// (ivf_quant_lookup.cu:894-1058): same inputs (Fp16GpuTables) and result
// layout; the reference scores 16 queries x 64 rows per step with wmma and
// re-streams the whole fp16 base set once per 16 queries.
//
// The scan kernel itself (tc_scan_kernel.cuh) is instantiated per precision
// in tc_scan_fp16.cu / tc_scan_fp8.cu. Machine mapping (one CTA per SM,
// 64 + 128 G threads for G epilogue groups):
//   warp 0    TMA producer: per K block, a 128-query tile (A) and a 256-row
//             base tile (B), 128-byte-swizzled, into a STAGES-deep ring;
//   warp 1    TMEM owner + single-thread tcgen05.mma issuer (M=128, N=256,
//             fp32 accumulators, two 256-column buffers so the epilogue of
//             tile i overlaps the MMAs of tile i+1);
//   warps 2.. epilogue, 4 warps per group: thread r of a group owns query r
//             of the block (TMEM lane r),
//             turns dot products into distances, applies the slot mask and
//             keeps that query's best KL (distance, slot) keys in a shared-
//             memory max-heap. No distance matrix ever reaches HBM.
// A CTA scans a contiguous range of base tiles; the per-(query, range)
// heaps are merged by tc_select_kernel, which also rescores them in fp32.
#include <cmath>
#include <cuda_fp16.h>
#include <cuda_fp8.h>
#include <cudaTypedefs.h>

#include "../../include/fv_bridge.h"
#include "tc_scan_kernel.cuh"

namespace fv {

namespace {

// ---------------------------------------------------------------------------
// Query preparation: fp32 -> fp16 (round to nearest even, as the reference
// converts queries: ivf_quant_lookup.cu:953) or fp32 -> e4m3 with a per-query
// power-of-two scale s_q = 2^a: the smallest with max|q| <= 448 s_q, raised
// where needed to 2^(b - 8) (s = 2^b the table's scale) so that the L2
// norm-digit factor -s / s_q = -2^(b - a) is an e4m3 value; it goes into
// columns dim..dim+2 against the table's norm digits (0 there for inner
// product and cosine, and for L2 where b - a < -9: a query so much larger
// than every row that the rows' norms no longer order the candidates);
// ||q||^2 of the fp32 query (the reference's :922-928, here summed across
// the warp: it only enters the scan's approximate distance). One warp per
// query.
// ---------------------------------------------------------------------------
template <bool FP8>
__global__ void __launch_bounds__(256) tc_prep_queries_kernel(const float* __restrict__ q, uint32_t nq, uint32_t dim,
                                                              uint32_t pd, void* __restrict__ out,
                                                              float* __restrict__ qnorm, float* __restrict__ qscale,
                                                              uint32_t* __restrict__ tslot, uint32_t kl,
                                                              uint32_t stride, const float* __restrict__ xscale,
                                                              int metric, uint32_t nq_rows, bool table_scale) {
  const uint32_t qi = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (qi >= nq_rows) return;
  if (qi >= nq) {
    // padding rows up to a whole query block: zero codes, so that every TMA
    // load of a query tile is in bounds (an out-of-bounds fill of most of a
    // 128-row tile, reloaded per K block, slowed a one-query scan by 40%)
    const size_t row_bytes = (size_t)pd * (FP8 ? 1 : 2);
    uint8_t* o = static_cast<uint8_t*>(out) + (size_t)qi * row_bytes;
    for (size_t b = (size_t)lane * 16; b < row_bytes; b += 32 * 16) *reinterpret_cast<uint4*>(o + b) = make_uint4(0, 0, 0, 0);
    return;
  }
  const float* src = q + (size_t)qi * dim;
  // shared-bound slots: empty (all ones) for the kl used, 0 for the padding
  for (uint32_t s = lane; s < stride; s += 32) tslot[(size_t)qi * stride + s] = s < kl ? 0xFFFFFFFFu : 0u;
  {
    // ||q||^2 of the scan's approximate distance (L2 and cosine); the exact
    // fp32 rescore recomputes distances in the reference's order
    float s = 0.f;
    for (uint32_t d = lane; d < dim; d += 32) s = fmaf(src[d], src[d], s);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if (lane == 0) qnorm[qi] = s;
  }
  if (FP8) {
    float amax = 0.f;
    for (uint32_t d = lane; d < dim; d += 32) amax = fmaxf(amax, fabsf(src[d]));
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) amax = fmaxf(amax, __shfl_xor_sync(0xffffffffu, amax, o));
    if (!table_scale) {
      // per-row-scale table: the query's scale amax / 448, no norm digits
      const float scale = amax > 0.f ? amax / 448.0f : 1.0f;
      if (lane == 0) qscale[qi] = scale;
      uint8_t* o8 = static_cast<uint8_t*>(out) + (size_t)qi * pd;
      for (uint32_t d = lane; d < pd; d += 32)
        o8[d] = d < dim ? (uint8_t)__nv_cvt_float_to_fp8(src[d] / scale, __NV_SATFINITE, __NV_E4M3) : (uint8_t)0;
      return;
    }
    const int b = ilogbf(__ldg(xscale));
    int a = b - 8;
    if (amax > 0.f) {
      int ap = ilogbf(amax) - 8;
      for (int it = 0; it < 4 && ldexpf(448.0f, ap) < amax; ++it) ++ap;
      for (int it = 0; it < 4 && ldexpf(448.0f, ap - 1) >= amax; ++it) --ap;
      a = max(a, ap);
    }
    if (lane == 0) qscale[qi] = ldexpf(1.0f, a);
    const float digit = (metric == METRIC_L2 && b - a >= -9) ? -ldexpf(1.0f, b - a) : 0.f;
    uint8_t* o8 = static_cast<uint8_t*>(out) + (size_t)qi * pd;
    for (uint32_t d = lane; d < pd; d += 32) {
      const float v = d < dim ? ldexpf(src[d], -a) : (d < dim + 3 ? digit : 0.f);
      o8[d] = (uint8_t)__nv_cvt_float_to_fp8(v, __NV_SATFINITE, __NV_E4M3);
    }
  } else {
    __half* o16 = static_cast<__half*>(out) + (size_t)qi * pd;
    for (uint32_t d = lane; d < pd; d += 32) o16[d] = d < dim ? __float2half_rn(src[d]) : __float2half_rn(0.f);
  }
}

// fp64 distance in the warp's lane-strided order (only the candidates at the
// k-th boundary go through here).
__device__ double warp_distance_f64(const float* __restrict__ q, const float* __restrict__ x, uint32_t dim, int lane,
                                    int metric) {
  double a = 0.0, b = 0.0, c = 0.0;
  constexpr int B = 8;  // loads in flight ahead of the (ordered) accumulation
  for (uint32_t d0 = lane; d0 < dim; d0 += 32 * B) {
    float qa[B], xa[B];
#pragma unroll
    for (int i = 0; i < B; ++i) {
      const uint32_t d = d0 + 32 * i;
      qa[i] = d < dim ? q[d] : 0.f;
      xa[i] = d < dim ? __ldg(x + d) : 0.f;
    }
#pragma unroll
    for (int i = 0; i < B; ++i) {
      if (d0 + 32 * i >= dim) break;
      const double u = qa[i], w = xa[i];
      if (metric == METRIC_L2) {
        const double t = u - w;
        a += t * t;
      } else {
        a += u * w;
        b += u * u;
        c += w * w;
      }
    }
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    a += __shfl_xor_sync(0xffffffffu, a, o);
    b += __shfl_xor_sync(0xffffffffu, b, o);
    c += __shfl_xor_sync(0xffffffffu, c, o);
  }
  if (metric == METRIC_L2) return a;
  if (metric == METRIC_INNER_PRODUCT) return -a;
  return 1.0 - a / (sqrt(b) * sqrt(c) + 1e-300);
}

struct SelectArgs {
  const uint64_t* partial;   // [nq][lists][KL]
  uint32_t lists, kl, pow2, shortlist, k;
  const float* queries;      // fp32 queries (rescore)
  const float* vectors;      // fp32 rows (null: no rescore)
  uint32_t dim;
  int metric;
  uint32_t boundary;
  float eps;
  GpuSearchResult* out;
  uint32_t* status;
  const float* tau;          // per-query admission bound of the scan (null: none)
  uint32_t* redo;            // set for a bounded query whose shortlist came up short
  const uint32_t* only;      // process only the flagged queries (null: all)
  uint32_t* incomplete_q;    // per-query flag set when a range heap may have dropped keys (or null)
};

constexpr int SEL_THREADS = 256;
constexpr int BAND_MAX = 64;

// One CTA per query: merge the per-range heaps, keep the best `shortlist`
// keys, rescore them in fp32 (the reference's warp-order distance), sort,
// re-rank the band |d - d_k| <= eps * scale in fp64, write the top k.
__global__ void __launch_bounds__(SEL_THREADS) tc_select_kernel(SelectArgs s) {
  extern __shared__ uint64_t keys[];
  __shared__ double band_d[BAND_MAX];
  __shared__ int band_lo, band_hi;
  __shared__ int incomplete;
  const uint32_t q = blockIdx.x;
  if (s.only && s.only[q] == 0u) return;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const uint32_t total = s.lists * s.kl;
  const uint64_t* src = s.partial + (size_t)q * total;
  __shared__ uint32_t n_live;
  if (threadIdx.x == 0) incomplete = 0;
  // only the kept keys are sorted (lists that stayed partly empty hold
  // sentinels); sorted they are the same sequence as the whole table sorted
  const uint32_t kp = min(s.shortlist, total);
  const uint32_t live = block_compact_keys(src, total, keys, &n_live);
  const uint32_t sp2 = next_pow2_dev(max(max(live, kp), 2u));
  for (uint32_t i = live + threadIdx.x; i < sp2; i += SEL_THREADS) keys[i] = kSentinelKey;
  __syncthreads();
  block_bitonic_sort(keys, sp2);
  if (s.kl < kp) {
    // a range whose heap stayed full and whose worst kept key still beats the
    // kp-th merged key may have dropped keys that belong in the shortlist
    const uint64_t cut = keys[kp - 1];
    for (uint32_t l = threadIdx.x; l < s.lists; l += SEL_THREADS) {
      const uint64_t root = src[(size_t)l * s.kl];
      if (root != kSentinelKey && root < cut) incomplete = 1;
    }
  }
  __syncthreads();
  if (incomplete && threadIdx.x == 0) {
    set_status(s.status, kStatusOverflow);
    if (s.incomplete_q) s.incomplete_q[q] = 1u;
  }
  // a bounded scan admitted fewer than kp rows: the bound from the sample was
  // below the query's kp-th distance, so the query is scanned again unbounded
  if (s.redo && threadIdx.x == 0 && keys[kp - 1] == kSentinelKey && s.tau[q] < kSentinelDist) s.redo[q] = 1u;

  const float* qv = s.queries + (size_t)q * s.dim;
  if (s.vectors) {
    for (uint32_t c = warp; c < kp; c += SEL_THREADS / 32) {
      const uint64_t key = keys[c];
      if (key == kSentinelKey) continue;
      const uint32_t slot = key_slot(key);
      const float d = warp_metric_distance(qv, s.vectors + (size_t)slot * s.dim, s.dim, lane, (MetricType)s.metric);
      if (lane == 0) keys[c] = d < kSentinelDist ? make_key(d, slot) : kSentinelKey;
    }
    const uint32_t p2 = next_pow2_dev(kp);
    for (uint32_t i = kp + threadIdx.x; i < p2; i += SEL_THREADS) keys[i] = kSentinelKey;
    __syncthreads();
    block_bitonic_sort(keys, p2);

    if (s.boundary && s.k <= kp && keys[s.k - 1] != kSentinelKey) {
      // ||q||^2 for the band's width, summed by warp 0 (lane-strided, tree)
      float qn = 0.f;
      if (warp == 0) {
        for (uint32_t d = lane; d < s.dim; d += 32) qn = fmaf(qv[d], qv[d], qn);
        qn = warp_tree_sum(qn);
      }
      if (threadIdx.x == 0) {
        const float dk = key_dist(keys[s.k - 1]);
        // scale of the accumulated terms: |d_k| for L2; |q||x| bounds |dot|
        float scale = fabsf(dk) + (s.metric == METRIC_L2 ? 0.f : sqrtf(qn) * 2.0f);
        const float band = s.eps * scale;
        int lo = (int)s.k - 1, hi = (int)s.k;
        while (lo > 0 && key_dist(keys[lo - 1]) >= dk - band) --lo;
        while (hi < (int)kp && keys[hi] != kSentinelKey && key_dist(keys[hi]) <= dk + band) ++hi;
        if (hi - lo > BAND_MAX || hi - lo < 2) lo = hi = 0;
        band_lo = lo;
        band_hi = hi;
      }
      __syncthreads();
      const int lo = band_lo, hi = band_hi;
      for (int c = lo + warp; c < hi; c += SEL_THREADS / 32) {
        const double d = warp_distance_f64(qv, s.vectors + (size_t)key_slot(keys[c]) * s.dim, s.dim, lane, s.metric);
        if (lane == 0) band_d[c - lo] = d;
      }
      __syncthreads();
      if (threadIdx.x == 0 && hi > lo) {
        // insertion sort of the band by (fp64 distance, slot); distances
        // reported for the band are the fp64 values rounded to fp32
        for (int i = lo + 1; i < hi; ++i) {
          const double di = band_d[i - lo];
          const uint64_t ki = keys[i];
          int j = i - 1;
          while (j >= lo && (band_d[j - lo] > di || (band_d[j - lo] == di && key_slot(keys[j]) > key_slot(ki)))) {
            band_d[j + 1 - lo] = band_d[j - lo];
            keys[j + 1] = keys[j];
            --j;
          }
          band_d[j + 1 - lo] = di;
          keys[j + 1] = ki;
        }
        for (int i = lo; i < hi; ++i) keys[i] = make_key((float)band_d[i - lo], key_slot(keys[i]));
      }
      __syncthreads();
    }
  }
  for (uint32_t r = threadIdx.x; r < s.k; r += SEL_THREADS)
    s.out[(size_t)q * s.k + r] = key_to_result(r < kp ? keys[r] : kSentinelKey, nullptr);
}

// Pre-pass result: per query, the distance of the r-th best key among the
// sample's per-range heaps -- the query's admission bound for the full scan
// (1e30, i.e. no bound, when the sample holds fewer than r admissible rows).
__global__ void __launch_bounds__(128) tc_tau_kernel(const uint64_t* __restrict__ partial, uint32_t total,
                                                     uint32_t pow2, uint32_t r, float* __restrict__ tau) {
  extern __shared__ uint64_t keys[];
  __shared__ uint32_t n_live;
  const uint32_t q = blockIdx.x;
  const uint64_t* src = partial + (size_t)q * total;
  const uint32_t live = block_compact_keys(src, total, keys, &n_live);
  if (live < r) {
    // fewer than r sampled keys: no bound
    if (threadIdx.x == 0) tau[q] = kSentinelDist;
    return;
  }
  const uint32_t sp2 = next_pow2_dev(max(live, 2u));
  for (uint32_t i = live + threadIdx.x; i < sp2; i += blockDim.x) keys[i] = kSentinelKey;
  __syncthreads();
  block_bitonic_sort(keys, sp2);
  if (threadIdx.x == 0) tau[q] = key_dist(keys[r - 1]);
}

// cuTensorMapEncodeTiled resolved through the runtime, so the library does
// not link libcuda (it must load on hosts without a driver).
PFN_cuTensorMapEncodeTiled_v12000 tmap_encoder() {
  static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
  if (!fn) {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q{};
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
  }
  return fn;
}

bool encode_tmap(CUtensorMap* m, const void* ptr, bool fp8, uint64_t inner_elems, uint64_t rows, uint64_t row_bytes,
                 uint32_t box_rows) {
  PFN_cuTensorMapEncodeTiled_v12000 enc = tmap_encoder();
  if (!enc) return false;
  cuuint64_t dims[2] = {inner_elems, rows};
  cuuint64_t strides[1] = {row_bytes};
  cuuint32_t box[2] = {(cuuint32_t)(fp8 ? 128 : 64), box_rows};
  cuuint32_t estr[2] = {1, 1};
  CUresult r = enc(m, fp8 ? CU_TENSOR_MAP_DATA_TYPE_UINT8 : CU_TENSOR_MAP_DATA_TYPE_FLOAT16, 2,
                                      const_cast<void*>(ptr), dims, strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
                                      CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                                      CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  return r == CUDA_SUCCESS;
}

size_t align_up(size_t v, size_t a) { return (v + a - 1) / a * a; }

// ---------------------------------------------------------------------------
// Committed autotuner results (flashvector-gpu_gb300/tuning/gb300.json,
// compiled in by build.py as tuning_table.inc): per shape range, the CTA-pair
// choice, the pre-pass choice and stride, and the over-fetch that reached
// recall@10 >= 0.99 fastest on this GPU. Explicit knobs (fv_tune_set) and
// explicit scan options take precedence; "tc.table" = 0 ignores the table.
// ---------------------------------------------------------------------------
struct TuneEntry {
  int fp8, metric;
  uint32_t dim_lo, dim_hi;
  uint64_t n_lo, n_hi;
  uint32_t nq_lo, nq_hi, k_lo, k_hi;
  int pair, prepass, stride, overfetch;
};
const TuneEntry kTuneTable[] = {
#include "tuning_table.inc"
    {-1, -1, 0, 0, 0, 0, 0, 0, 0, 0, -1, -1, 0, 0}};

const TuneEntry* tune_lookup(bool fp8, int metric, uint32_t dim, uint64_t n, uint32_t nq, uint32_t k) {
  if (tune_value("tc.table", 1) == 0) return nullptr;
  for (const TuneEntry& e : kTuneTable) {
    if (e.fp8 < 0) break;
    if (e.fp8 == (fp8 ? 1 : 0) && e.metric == metric && dim >= e.dim_lo && dim <= e.dim_hi && n >= e.n_lo &&
        n <= e.n_hi && nq >= e.nq_lo && nq <= e.nq_hi && k >= e.k_lo && k <= e.k_hi)
      return &e;
  }
  return nullptr;
}

// Sampled rank for the pre-pass bound. A sample of every stride-th tile
// holds each of a query's top (shortlist - 1) rows with probability
// 1 / stride, so the number of them in the sample is about Poisson(lambda =
// shortlist / stride); the sample's r-th best distance is below the query's
// shortlist-th distance (and the query needs the re-scan) only when that
// count reaches r. Returns the smallest r whose Poisson tail P(X >= r) is
// below `tail`.
uint32_t poisson_rank(double lambda, double tail) {
  double term = std::exp(-lambda), cdf = 0.0;
  uint32_t r = 0;
  while (1.0 - cdf >= tail && r < 4096) {
    cdf += term;
    ++r;
    term *= lambda / r;
  }
  return r;
}

// One CTA per SM at a time: a grid of nqb * splits CTAs runs in
// ceil(nqb * splits / sms) waves, the last one possibly part-empty. Among
// split counts in [s_min, max(2 s_min, 32)] (within the tile count and the
// select kernel's 16,384-key sort), take the smallest whose waves are at
// least 1% fuller than those of every smaller candidate (a grid of 79 query
// blocks x 1 split fills 53% of 148 SMs; x 13 splits, 99%).
uint32_t fill_waves(uint32_t s_min, uint32_t nqb, uint32_t ntiles, uint32_t sms, uint32_t keys_per_split) {
  auto fullness = [&](uint32_t s) {
    const uint64_t ctas = (uint64_t)nqb * s, waves = (ctas + sms - 1) / sms;
    return (double)ctas / (double)(waves * sms);
  };
  uint32_t best = s_min;
  double best_f = fullness(s_min);
  for (uint32_t s = s_min + 1; s <= std::max(2 * s_min, 32u) && s <= ntiles; ++s) {
    if (next_pow2(s * keys_per_split) > 16384u) break;
    const double f = fullness(s);
    if (f > best_f + 0.01) {
      best = s;
      best_f = f;
    }
  }
  return best;
}

}  // namespace

// Every launch parameter of one tensor-core scan call and the scratch it
// takes, computed once: launch_tc_scan launches from it and the serving
// loop admits a batch by its scratch_bytes (tc_scan_scratch_bytes).
struct TcPlan {
  bool fp8 = false, pair = false, prepass = false;
  uint32_t elem = 0, kblocks = 0, shortlist = 0, kl = 0, kl_tmpl = 0;
  int groups = 1, pgroups = 1;  // epilogue groups of the main scan and of the pre-pass
  uint32_t nqb = 0, nqb_grid = 0, splits = 0, tps = 0;
  uint32_t pstride = 0, pr = 0, pkl_tmpl = 0, psplits = 0, ptps = 0;
  uint32_t nq_rows = 0, slot_stride = 0;
  size_t q_bytes = 0, qn_bytes = 0, part_bytes = 0, slot_bytes = 0, ppart_bytes = 0, tau_bytes = 0;
  size_t scratch_bytes = 0;
};

TcPlan plan_tc_scan(const TcTables& t, uint32_t nq, uint32_t k, MetricType metric, const FvScanOptions& opt) {
  TcPlan P{};
  const bool fp8 = t.fp8;
  const uint32_t elem = fp8 ? 1 : 2;
  const uint32_t kb_elems = fp8 ? 128 : 64;
  const uint32_t kblocks = (t.padded_dim + kb_elems - 1) / kb_elems;
  const TuneEntry* te = tune_lookup(fp8, (int)metric, t.dim, t.n, nq, k);
  const uint32_t overfetch = opt.overfetch ? opt.overfetch : (te && te->overfetch > 0 ? (uint32_t)te->overfetch : 4u);
  const uint32_t shortlist = t.vectors ? std::min<uint32_t>(std::max(k, overfetch * k), 4096u) : k;
  // short K (at most two 64-element fp16 / 128-element fp8 blocks per tile):
  // a tile costs the MMA little and the epilogue much, so two epilogue
  // groups drain the two accumulator buffers in parallel. Fused fp8 with one
  // K block and a shortlist above 48 keys (where two groups' heaps hold less
  // than the shortlist too) runs four ("tc.groups": -1 auto, 2 or 4).
  const bool fused_fp8 = fp8 && t.fp8_table_scale && metric != METRIC_COSINE && kblocks == 1;
  const int64_t groups_knob = tune_value("tc.groups", -1);
  const bool four = fused_fp8 && (groups_knob == 4 || (groups_knob < 0 && shortlist > 48u));
  const int groups = kblocks > 2 ? 1 : (four ? 4 : 2);
  const uint32_t kl_cap = groups == 4 ? 32u : (groups == 2 ? 48u : 64u);
  const uint32_t kl = std::min<uint32_t>(kl_cap, shortlist);         // heap entries per (query, range, group)
  const uint32_t kl_tmpl = std::min<uint32_t>(kl_cap, (kl + 15) / 16 * 16);  // heap capacity (template)
  const uint32_t nqb = (nq + TC_M - 1) / TC_M;
  const uint32_t ntiles = (t.n + TC_N - 1) / TC_N;
  const int sms = device_sm_count();
  // CTA pairs (cta_group::2) for long rows: two query blocks share each
  // base tile, each SM streaming half of it
  int64_t pair_knob = tune_value("tc.pair", -1);
  if (pair_knob < 0 && te && te->pair >= 0) pair_knob = te->pair;
  const bool pair = groups == 1 && pair_knob != 0;
  const uint32_t nqb_grid = pair ? 2 * ((nqb + 1) / 2) : nqb;  // CTAs per split
  uint32_t splits = opt.splits ? opt.splits : std::max<uint32_t>(1u, (uint32_t)sms / nqb_grid);
  if (!opt.splits && shortlist > kl) {
    // a (query, range, group) heap keeps kl keys: split the base so that each
    // heap holds, in expectation, a third of its share of the shortlist (a
    // heap that still overflows is reported through the status word)
    splits = std::max<uint32_t>(splits, (3 * shortlist + kl * groups - 1) / (kl * groups));
  }
  splits = std::max(1u, std::min(splits, ntiles));
  if (!opt.splits) splits = fill_waves(splits, nqb_grid, ntiles, (uint32_t)sms, groups * kl);
  // the select kernel sorts lists*kl keys in shared memory: <= 16384
  while (splits > 1 && next_pow2(splits * groups * kl) > 16384u) --splits;
  uint32_t tps = (ntiles + splits - 1) / splits;
  splits = (ntiles + tps - 1) / tps;

  // Sampled pre-pass: the CTAs of a query cannot share a bound when the
  // shortlist exceeds the per-range heap, so each range would insert
  // ~kl (1 + ln(rows / kl)) keys per query. A scan of every stride-th tile
  // gives each query its r-th best sampled distance (r from the Poisson tail
  // below, or ceil(margin * shortlist / stride) when the margin knob is
  // set), an upper bound on its shortlist-th distance unless the sample is
  // unlucky (probability < 1e-7 per query); the full scan then admits only
  // rows within it. Queries whose bounded scan comes up short are scanned
  // again without the bound (device-side, no host round trip).
  int64_t pp_knob = tune_value("tc.prepass", -1);
  if (pp_knob < 0 && te && te->prepass >= 0) pp_knob = te->prepass;
  int64_t stride_knob = tune_value("tc.prepass_stride", 0);
  if (stride_knob <= 0) stride_knob = (te && te->stride > 0) ? te->stride : 32;
  const uint32_t pstride = (uint32_t)std::max<int64_t>(2, stride_knob);
  const int64_t pmargin = tune_value("tc.prepass_margin", 0);
  const uint32_t pr = std::max<uint32_t>(
      1u, std::min<uint32_t>(kl_cap, pmargin > 0 ? (uint32_t)((pmargin * shortlist + pstride - 1) / pstride)
                                                 : poisson_rank((double)shortlist / pstride, 1e-7)));
  const uint32_t psampled = (ntiles + pstride - 1) / pstride;
  // automatic: bases of >= 64 sampled tiles (the main scan then uses the
  // pre-pass bound instead of the cross-CTA shared one); forced on (knob 1):
  // any base
  const bool prepass = psampled > 0 && (pp_knob == 1 || (pp_knob != 0 && psampled >= 64u));
  // the pre-pass keeps two groups where the main scan runs four: its tiles
  // are far apart, and two groups alternating them (each its own
  // accumulator buffer) beat four splitting every tile's columns
  const int pgroups = groups == 4 ? 2 : groups;
  const uint32_t pkl_tmpl = std::min<uint32_t>(pgroups == 2 ? 48u : 64u, (pr + 15) / 16 * 16);
  uint32_t psplits = std::max<uint32_t>(1u, std::min<uint32_t>((uint32_t)sms / nqb_grid, psampled));
  psplits = fill_waves(psplits, nqb_grid, psampled, (uint32_t)sms, pgroups * pr);
  while (psplits > 1 && next_pow2(psplits * pgroups * pr) > 16384u) --psplits;
  const uint32_t ptps = (psampled + psplits - 1) / psplits;
  psplits = (psampled + ptps - 1) / ptps;

  // scratch: prepared queries | ||q||^2 | q scales | partial heaps | slots
  //          [| pre-pass heaps | tau | redo flags]
  // prepared queries padded with zero rows to whole query blocks (of the
  // CTA pairs' grid when pairs run)
  const uint32_t nq_rows = nqb_grid * TC_M;
  const size_t q_bytes = align_up((size_t)nq_rows * t.padded_dim * elem, 1024);
  const size_t qn_bytes = align_up((size_t)nq * 4, 256);
  const size_t part_bytes = align_up((size_t)nq * splits * groups * kl * 8, 256);
  const uint32_t slot_stride = ((prepass ? std::max(kl, pr) : kl) + 3) / 4 * 4;
  const size_t slot_bytes = align_up((size_t)nq * slot_stride * 4, 256);
  const size_t ppart_bytes = prepass ? align_up((size_t)nq * psplits * pgroups * pr * 8, 256) : 0;
  const size_t tau_bytes = prepass ? 2 * qn_bytes : 0;
  P.fp8 = fp8;
  P.elem = elem;
  P.kblocks = kblocks;
  P.shortlist = shortlist;
  P.groups = groups;
  P.pgroups = pgroups;
  P.kl = kl;
  P.kl_tmpl = kl_tmpl;
  P.nqb = nqb;
  P.pair = pair;
  P.nqb_grid = nqb_grid;
  P.splits = splits;
  P.tps = tps;
  P.prepass = prepass;
  P.pstride = pstride;
  P.pr = pr;
  P.pkl_tmpl = pkl_tmpl;
  P.psplits = psplits;
  P.ptps = ptps;
  P.nq_rows = nq_rows;
  P.q_bytes = q_bytes;
  P.qn_bytes = qn_bytes;
  P.part_bytes = part_bytes;
  P.slot_stride = slot_stride;
  P.slot_bytes = slot_bytes;
  P.ppart_bytes = ppart_bytes;
  P.tau_bytes = tau_bytes;
  P.scratch_bytes = q_bytes + 2 * qn_bytes + part_bytes + slot_bytes + ppart_bytes + tau_bytes;
  return P;
}

size_t tc_scan_scratch_bytes(const TcTables& t, uint32_t nq, uint32_t k, MetricType metric,
                             const FvScanOptions& opt) {
  return plan_tc_scan(t, nq, k, metric, opt).scratch_bytes;
}

int launch_tc_scan(const TcTables& t, const float* queries, uint32_t nq, uint32_t k, MetricType metric,
                   const uint32_t* mask, GpuSearchResult* out, const FvScanOptions& opt, cudaStream_t stream,
                   const QueryFilter* filters) {
  return launch_tc_scan_ext(t, queries, nq, k, metric, mask, out, opt, stream, filters, nullptr, nullptr);
}

int launch_tc_scan_ext(const TcTables& t, const float* queries, uint32_t nq, uint32_t k, MetricType metric,
                       const uint32_t* mask, GpuSearchResult* out, const FvScanOptions& opt, cudaStream_t stream,
                       const QueryFilter* filters, void* ext_scratch, uint32_t* incomplete_q) {
  const TcPlan P = plan_tc_scan(t, nq, k, metric, opt);
  const bool fp8 = P.fp8;
  const uint32_t elem = P.elem, kblocks = P.kblocks, shortlist = P.shortlist, kl = P.kl, kl_tmpl = P.kl_tmpl;
  const int groups = P.groups, pgroups = P.pgroups;
  const uint32_t nqb = P.nqb, nqb_grid = P.nqb_grid, splits = P.splits, tps = P.tps;
  const bool pair = P.pair, prepass = P.prepass;
  const uint32_t pstride = P.pstride, pr = P.pr, pkl_tmpl = P.pkl_tmpl, psplits = P.psplits, ptps = P.ptps;
  const uint32_t nq_rows = P.nq_rows, slot_stride = P.slot_stride;
  const size_t q_bytes = P.q_bytes, qn_bytes = P.qn_bytes, part_bytes = P.part_bytes, slot_bytes = P.slot_bytes;
  const size_t ppart_bytes = P.ppart_bytes;
  uint8_t* scratch = static_cast<uint8_t*>(ext_scratch ? ext_scratch : scratch_get(stream, P.scratch_bytes));
  if (!scratch) return (int)cudaErrorMemoryAllocation;
  void* qprep = scratch;
  float* qnorm = reinterpret_cast<float*>(scratch + q_bytes);
  float* qscale = reinterpret_cast<float*>(scratch + q_bytes + qn_bytes);
  uint64_t* partial = reinterpret_cast<uint64_t*>(scratch + q_bytes + 2 * qn_bytes);
  uint32_t* tslot = reinterpret_cast<uint32_t*>(scratch + q_bytes + 2 * qn_bytes + part_bytes);
  uint8_t* extra = scratch + q_bytes + 2 * qn_bytes + part_bytes + slot_bytes;
  uint64_t* ppartial = prepass ? reinterpret_cast<uint64_t*>(extra) : nullptr;
  float* tau = prepass ? reinterpret_cast<float*>(extra + ppart_bytes) : nullptr;
  uint32_t* redo = prepass ? reinterpret_cast<uint32_t*>(extra + ppart_bytes + qn_bytes) : nullptr;

  {
    ProfScope ps(fp8 ? "tc_prep_queries_fp8" : "tc_prep_queries_fp16", stream);
    const uint32_t blocks = (nq_rows * 32 + 255) / 256;
    // the shared-bound slots serve the scan that shares a bound: the main
    // scan when its heap holds the whole shortlist, else the pre-pass
    const uint32_t slot_kl = prepass ? pr : kl;
    if (fp8)
      tc_prep_queries_kernel<true><<<blocks, 256, 0, stream>>>(queries, nq, t.dim, t.padded_dim, qprep, qnorm, qscale,
                                                               tslot, slot_kl, slot_stride, t.scales, (int)metric,
                                                               nq_rows, t.fp8_table_scale);
    else
      tc_prep_queries_kernel<false><<<blocks, 256, 0, stream>>>(queries, nq, t.dim, t.padded_dim, qprep, qnorm,
                                                                qscale, tslot, slot_kl, slot_stride, nullptr,
                                                                (int)metric, nq_rows, false);
    note_launch();
  }

  CUtensorMap ta, tb, tb_half;
  if (!encode_tmap(&ta, qprep, fp8, t.padded_dim, nq_rows, (uint64_t)t.padded_dim * elem, TC_M) ||
      !encode_tmap(&tb, t.base, fp8, t.padded_dim, t.n, (uint64_t)t.padded_dim * elem, TC_N) ||
      (pair && !encode_tmap(&tb_half, t.base, fp8, t.padded_dim, t.n, (uint64_t)t.padded_dim * elem, TC_N / 2)))
    return FV_ERR_ARG;

  TcScanArgs a{};
  a.n = t.n;
  a.nq = nq;
  a.kblocks = kblocks;
  a.nqb = nqb;
  a.xnorm = t.norms;
  a.xscale = t.scales;
  a.qnorm = qnorm;
  a.qscale = qscale;
  a.mask = mask;
  a.tslot = tslot;
  a.tslot_stride = slot_stride;
  a.status = status_word();
  a.filters = filters;
  a.tile_stride = 1;
  // "tc.wait_limit_ns" (0: 2 s) bounds the pipeline's waits; a wait that runs
  // out ends the scan early and is reported through the status word
  const int64_t wl = tune_value("tc.wait_limit_ns", 0);
  a.wait_ns = wl > 0 ? (uint64_t)wl : 2000000000ull;
  // use_pair: the CTA-pair variant (not for the re-scan of flagged queries,
  // whose blocks leave independently)
  auto scan = [&](const TcScanArgs& args, int kl_t, uint32_t splits_n, const char* name, bool use_pair,
                  int groups_n) -> cudaError_t {
    ProfScope ps(name, stream);
    const int g = use_pair ? -1 : groups_n;
    const uint32_t grid = (use_pair ? nqb_grid : nqb) * splits_n;
    const CUtensorMap& b = use_pair ? tb_half : tb;
    return fp8 ? dispatch_tc_scan_fp8(kl_t, g, (int)metric, t.fp8_table_scale, ta, b, args, grid, stream)
               : dispatch_tc_scan_fp16(kl_t, g, (int)metric, true, ta, b, args, grid, stream);
  };
  cudaError_t e;
  if (prepass) {
    TcScanArgs p = a;
    p.splits = psplits;
    p.tiles_per_split = ptps;
    p.partial = ppartial;
    p.kl = pr;
    p.share = 1;  // the pre-pass heap holds its whole "shortlist" (pr keys)
    p.tile_stride = pstride;
    e = scan(p, (int)pkl_tmpl, psplits, fp8 ? "tc_prepass_fp8" : "tc_prepass_fp16", pair, pgroups);
    if (e != cudaSuccess) return (int)e;
    const uint32_t total = psplits * pgroups * pr, pow2 = next_pow2(total);
    e = cudaFuncSetAttribute(tc_tau_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)(pow2 * 8));
    if (e != cudaSuccess) return (int)e;
    {
      ProfScope ps("tc_tau", stream);
      tc_tau_kernel<<<nq, 128, pow2 * 8, stream>>>(ppartial, total, pow2, pr, tau);
      note_launch();
    }
    e = cudaMemsetAsync(redo, 0, (size_t)nq * 4, stream);
    if (e != cudaSuccess) return (int)e;
  }
  a.splits = splits;
  a.tiles_per_split = tps;
  a.partial = partial;
  a.kl = kl;
  a.share = (kl == shortlist && !prepass) ? 1u : 0u;
  a.qbound = tau;
  e = scan(a, (int)kl_tmpl, splits, fp8 ? "tc_scan_fp8" : "tc_scan_fp16", pair, groups);
  if (e != cudaSuccess) return (int)e;

  SelectArgs s{partial, splits * groups, kl, next_pow2(splits * groups * kl), shortlist, k, queries, t.vectors, t.dim,
               (int)metric,
               opt.boundary_fp64 ? 1u : 0u, 0.f, out, status_word(), tau, redo, nullptr, incomplete_q};
  s.eps = opt.boundary_eps > 0.f ? opt.boundary_eps : (float)((t.dim + 31) / 32 + 5) * 2.0f * 5.960464477539063e-08f;
  const size_t sel_smem = (size_t)std::max(s.pow2, next_pow2(shortlist)) * 8;
  e = cudaFuncSetAttribute(tc_select_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sel_smem);
  if (e != cudaSuccess) return (int)e;
  {
    ProfScope ps("tc_select_rescore", stream);
    tc_select_kernel<<<nq, SEL_THREADS, sel_smem, stream>>>(s);
    note_launch();
  }
  if (prepass) {
    // queries whose bound was too tight: scanned again without it (blocks
    // holding none of them exit at once), then selected again
    TcScanArgs f = a;
    f.qbound = nullptr;
    f.active = redo;
    f.share = 0;
    e = scan(f, (int)kl_tmpl, splits, fp8 ? "tc_rescan_fp8" : "tc_rescan_fp16", false, groups);
    if (e != cudaSuccess) return (int)e;
    SelectArgs r = s;
    r.tau = nullptr;
    r.redo = nullptr;
    r.only = redo;
    ProfScope ps("tc_select_rescore", stream);
    tc_select_kernel<<<nq, SEL_THREADS, sel_smem, stream>>>(r);
    note_launch();
  }
  return (int)cudaGetLastError();
}

}  // namespace fv

extern "C" int fv_tune_lookup(int fp8, MetricType metric, uint32_t dim, uint64_t num_vectors, uint32_t num_queries,
                              uint32_t top_k, int32_t* out_knobs) {
  if (!out_knobs) return FV_ERR_NULL;
  const fv::TuneEntry* e = fv::tune_lookup(fp8 != 0, (int)metric, dim, num_vectors, num_queries, top_k);
  if (!e) return FV_ERR_ARG;
  out_knobs[0] = e->pair;
  out_knobs[1] = e->prepass;
  out_knobs[2] = e->stride;
  out_knobs[3] = e->overfetch;
  return 0;
}

