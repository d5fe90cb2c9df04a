// tc_scan.cu -- tensor-core flat scan (FP16 and FP8-E4M3) fused with top-k,
// followed by an exact fp32 rescore of an over-fetched shortlist and an
// fp64 re-rank of the candidates that straddle the k-th distance.
//
// Replaces the reference's fp16_tc_wmma_search_kernel / launch_fp16_tc_search
// (ivf_quant_lookup.cu:894-1058): same inputs (Fp16GpuTables) and result
// layout; the reference scores 16 queries x 64 rows per step with wmma and
// re-streams the whole fp16 base set once per 16 queries.
//
// Machine mapping (one CTA per SM, 192 threads):
//   warp 0    TMA producer: per K block, a 128-query tile (A) and a 256-row
//             base tile (B), 128-byte-swizzled, into a STAGES-deep ring;
//   warp 1    TMEM owner + single-thread tcgen05.mma issuer (M=128, N=256,
//             fp32 accumulators, two 256-column buffers so the epilogue of
//             tile i overlaps the MMAs of tile i+1);
//   warps 2-5 epilogue: thread r owns query r of the block (TMEM lane r),
//             turns dot products into distances, applies the slot mask and
//             keeps that query's best KL (distance, slot) keys in a shared-
//             memory max-heap. No distance matrix ever reaches HBM.
// A CTA scans a contiguous range of base tiles; the per-(query, range)
// heaps are merged by tc_select_kernel, which also rescoring in fp32.
#include <cuda_fp16.h>
#include <cuda_fp8.h>
#include <cudaTypedefs.h>

#include "../../include/fv_bridge.h"
#include "common.cuh"
#include "kernels.h"
#include "tc_ptx.cuh"
#include "topk.cuh"

namespace fv {

namespace {

constexpr int TC_M = 128;                  // queries per CTA (TMEM lanes)
constexpr int TC_N = 256;                  // base rows per tile (MMA N)
constexpr int KB_BYTES = 128;              // K bytes per stage row (one 128B swizzle atom)
constexpr int A_STAGE = TC_M * KB_BYTES;   // 16 KB
constexpr int B_STAGE = TC_N * KB_BYTES;   // 32 KB
constexpr int SCAN_THREADS = 192;

struct TcScanArgs {
  uint32_t n, nq, kblocks, nqb, splits, tiles_per_split;
  int metric;
  const float* xnorm;    // [n] ||x||^2 of the fp32 rows (L2, cosine)
  const float* xscale;   // [n] per-row fp8 scale (FP8 only)
  const float* qnorm;    // [nq] ||q||^2
  const float* qscale;   // [nq] per-query fp8 scale (FP8 only)
  const uint32_t* mask;
  uint64_t* partial;     // [nq][splits][KL]
  uint32_t* tau;         // [nq] shared bound on each query's kl-th distance (float_order)
  uint32_t kl;           // heap entries used (<= KL); == shortlist when shared bounds are on
  uint32_t share_tau;    // 1: CTAs of one query publish / read tau (kl == shortlist)
  uint32_t* status;
};

template <int KL, int STAGES>
struct ScanSmem {
  static constexpr size_t a_off = 0;
  static constexpr size_t b_off = a_off + (size_t)STAGES * A_STAGE;
  static constexpr size_t heap_off = b_off + (size_t)STAGES * B_STAGE;
  static constexpr size_t col_off = heap_off + (size_t)KL * TC_M * 8;   // [4 warps][2][TC_N] floats
  static constexpr size_t cmask_off = col_off + 4 * 2 * TC_N * 4;       // [4 warps][8] words
  static constexpr size_t bar_off = cmask_off + 4 * 8 * 4;              // barriers
  static constexpr size_t nbars = 2 * STAGES + 5;
  static constexpr size_t misc_off = bar_off + nbars * 8;
  static constexpr size_t bytes = misc_off + 16 + 1024;                 // + alignment slack
};

__device__ __noinline__ void heap_sift(uint64_t* h, int kl, uint64_t key) {
  // replace the root of a max-heap stored with stride TC_M
  int i = 0;
  while (true) {
    int l = 2 * i + 1;
    if (l >= kl) break;
    uint64_t cv = h[l * TC_M];
    int c = l;
    if (l + 1 < kl) {
      uint64_t rv = h[(l + 1) * TC_M];
      if (rv > cv) { cv = rv; c = l + 1; }
    }
    if (cv <= key) break;
    h[i * TC_M] = cv;
    i = c;
  }
  h[i * TC_M] = key;
}

// v[j] for a lane-varying j without local memory: a 6-level select tree.
__device__ __forceinline__ float select64(const float (&v)[64], int j) {
  float t[32];
#pragma unroll
  for (int i = 0; i < 32; ++i) t[i] = (j & 1) ? v[2 * i + 1] : v[2 * i];
#pragma unroll
  for (int i = 0; i < 16; ++i) t[i] = (j & 2) ? t[2 * i + 1] : t[2 * i];
#pragma unroll
  for (int i = 0; i < 8; ++i) t[i] = (j & 4) ? t[2 * i + 1] : t[2 * i];
#pragma unroll
  for (int i = 0; i < 4; ++i) t[i] = (j & 8) ? t[2 * i + 1] : t[2 * i];
#pragma unroll
  for (int i = 0; i < 2; ++i) t[i] = (j & 16) ? t[2 * i + 1] : t[2 * i];
  return (j & 32) ? t[1] : t[0];
}

template <bool FP8, int KL, int STAGES>
__global__ void __launch_bounds__(SCAN_THREADS, 1)
    tc_scan_kernel(const __grid_constant__ CUtensorMap tmA, const __grid_constant__ CUtensorMap tmB, TcScanArgs a) {
  using L = ScanSmem<KL, STAGES>;
  extern __shared__ uint8_t smem_raw[];
  uint8_t* sm = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~(uintptr_t)1023);
  uint8_t* sA = sm + L::a_off;
  uint8_t* sB = sm + L::b_off;
  uint64_t* heap = reinterpret_cast<uint64_t*>(sm + L::heap_off);
  float* colbuf = reinterpret_cast<float*>(sm + L::col_off);
  uint32_t* colmask = reinterpret_cast<uint32_t*>(sm + L::cmask_off);
  uint64_t* bars = reinterpret_cast<uint64_t*>(sm + L::bar_off);
  uint64_t* full = bars;
  uint64_t* empty = bars + STAGES;
  uint64_t* acc_full = bars + 2 * STAGES;
  uint64_t* acc_empty = acc_full + 2;
  uint64_t* mma_done = acc_empty + 2;
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(sm + L::misc_off);
  volatile uint32_t* abort_flag = tmem_slot + 1;

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const uint32_t qb = blockIdx.x % a.nqb, split = blockIdx.x / a.nqb;
  const uint32_t ntiles = (a.n + TC_N - 1) / TC_N;
  const uint32_t t_begin = split * a.tiles_per_split;
  const uint32_t t_end = min(t_begin + a.tiles_per_split, ntiles);
  const uint32_t my_tiles = t_end > t_begin ? t_end - t_begin : 0;

  if (threadIdx.x == 0) {
    for (int s = 0; s < STAGES; ++s) {
      tc::mbar_init(&full[s], 1);
      tc::mbar_init(&empty[s], 1);
    }
    for (int b = 0; b < 2; ++b) {
      tc::mbar_init(&acc_full[b], 1);
      tc::mbar_init(&acc_empty[b], 4);
    }
    tc::mbar_init(mma_done, 1);
    *abort_flag = 0;
    tc::fence_mbar_init();
  }
  if (warp == 1) {
    tc::tmem_alloc(tmem_slot, 512);
    tc::tc_fence_before();
  }
  __syncthreads();
  tc::tc_fence_after();
  const uint32_t tmem = *tmem_slot;

  if (warp == 0) {
    // ------------------------------------------------------ TMA producer
    if (lane == 0) {
      tc::prefetch_tmap(&tmA);
      tc::prefetch_tmap(&tmB);
      const uint64_t pol_a = tc::policy_evict_last();
      const uint64_t pol_b = tc::policy_evict_first();
      const int kb_elems = FP8 ? 128 : 64;
      uint32_t stage = 0, phase = 0;
      int32_t issued_parity[STAGES];
#pragma unroll
      for (int s = 0; s < STAGES; ++s) issued_parity[s] = -1;
      bool ok = true;
      for (uint32_t i = 0; ok && i < my_tiles; ++i) {
        const int32_t row_b = (int32_t)((t_begin + i) * TC_N);
        for (uint32_t kb = 0; kb < a.kblocks; ++kb) {
          if (!tc::mbar_wait(&empty[stage], phase ^ 1, abort_flag, a.status)) {
            ok = false;
            break;
          }
          tc::mbar_arrive_expect_tx(&full[stage], A_STAGE + B_STAGE);
          tc::tma_load_2d(sA + stage * A_STAGE, &tmA, &full[stage], (int32_t)(kb * kb_elems), (int32_t)(qb * TC_M),
                          pol_a);
          tc::tma_load_2d(sB + stage * B_STAGE, &tmB, &full[stage], (int32_t)(kb * kb_elems), row_b, pol_b);
          issued_parity[stage] = (int32_t)phase;
          if (++stage == STAGES) {
            stage = 0;
            phase ^= 1;
          }
        }
      }
      // drain: every copy issued must have landed before the CTA may exit
      // (normally they all have; after an abort this waits a bounded time)
      uint32_t no_abort = 0;
#pragma unroll
      for (int s = 0; s < STAGES; ++s)
        if (issued_parity[s] >= 0)
          tc::mbar_wait(&full[s], (uint32_t)issued_parity[s], &no_abort, a.status, 100000000ull);
    }
  } else if (warp == 1) {
    // ------------------------------------------------------- MMA issuer
    if (lane == 0) {
      constexpr uint32_t idesc = tc::idesc_f32acc(0, 0, TC_M, TC_N);
      uint32_t stage = 0, phase = 0;
      bool ok = true;
      for (uint32_t i = 0; ok && i < my_tiles; ++i) {
        const uint32_t buf = i & 1, use = i >> 1;
        if (!tc::mbar_wait(&acc_empty[buf], (use & 1) ^ 1, abort_flag, a.status)) break;
        tc::tc_fence_after();
        const uint32_t d_tmem = tmem + buf * TC_N;
        for (uint32_t kb = 0; kb < a.kblocks; ++kb) {
          if (!tc::mbar_wait(&full[stage], phase, abort_flag, a.status)) {
            ok = false;
            break;
          }
          tc::tc_fence_after();
          const uint32_t a_base = tc::smem_addr(sA + stage * A_STAGE);
          const uint32_t b_base = tc::smem_addr(sB + stage * B_STAGE);
#pragma unroll
          for (uint32_t kk = 0; kk < 4; ++kk) {
            tc::mma<FP8>(d_tmem, tc::sdesc_k_sw128(a_base + kk * 32), tc::sdesc_k_sw128(b_base + kk * 32), idesc,
                         (kb | kk) != 0);
          }
          tc::mma_commit(&empty[stage]);
          if (++stage == STAGES) {
            stage = 0;
            phase ^= 1;
          }
        }
        if (ok) tc::mma_commit(&acc_full[buf]);
      }
      tc::mma_commit(mma_done);
    }
  } else {
    // --------------------------------------------------------- epilogue
    const int quad = warp & 3;                    // TMEM lane quadrant of this warp
    const int row = quad * 32 + lane;             // query row in the block
    const uint32_t q = qb * TC_M + row;
    const bool qvalid = q < a.nq;
    uint64_t* h = heap + row;
    const int kl = (int)a.kl;
    for (int i = 0; i < kl; ++i) h[i * TC_M] = kSentinelKey;
    // Shared bound: every CTA scanning query q publishes the distance of its
    // kl-th best key once its heap is full; the minimum over CTAs bounds the
    // query's global kl-th best distance from above, so any row farther
    // than it cannot be in the shortlist and is skipped by every CTA.
    float tau_d = kSentinelDist;
    float published = kSentinelDist;
    uint32_t* tau_ptr = (a.share_tau && qvalid) ? a.tau + q : nullptr;
    const float qn = qvalid ? __ldg(a.qnorm + q) : 0.f;
    const float qs = (FP8 && qvalid) ? __ldg(a.qscale + q) : 1.f;
    float worst = kSentinelDist;
    const int metric = a.metric;

    // per-warp copy of the current tile's column data (norms, fp8 scales,
    // mask words): staged by the warp itself, so the epilogue warps never
    // wait on one another
    float* cb = colbuf + (warp - 2) * 2 * TC_N;
    uint32_t* cm = colmask + (warp - 2) * 8;
    for (uint32_t i = 0; i < my_tiles; ++i) {
      const uint32_t buf = i & 1, use = i >> 1;
      const uint32_t v0 = (t_begin + i) * TC_N;
      __syncwarp();
      for (int c = lane; c < TC_N; c += 32) {
        const uint32_t slot = v0 + c;
        const bool in = slot < a.n;
        cb[c] = (in && a.xnorm) ? __ldg(a.xnorm + slot) : 0.f;
        if (FP8) cb[TC_N + c] = in ? __ldg(a.xscale + slot) : 0.f;
      }
      if (lane < 8) {
        const uint32_t c0 = v0 + lane * 32;
        uint32_t w = 0;
        if (c0 < a.n) {
          const uint32_t cnt = min(32u, a.n - c0);
          w = cnt == 32 ? 0xFFFFFFFFu : ((1u << cnt) - 1u);
          if (a.mask) w &= __ldg(a.mask + (c0 >> 5));
        }
        cm[lane] = w;
      }
      __syncwarp();
      const uint32_t tau_raw = tau_ptr ? __ldcg(tau_ptr) : 0u;
      if (!tc::mbar_wait(&acc_full[buf], use & 1, abort_flag, a.status)) break;
      tc::tc_fence_after();
      if (tau_ptr) tau_d = fminf(tau_d, order_float(tau_raw));

      const uint32_t t_row = tmem + ((uint32_t)(quad * 32) << 16) + buf * TC_N;
#pragma unroll 1
      for (int c0 = 0; c0 < TC_N; c0 += 64) {
        uint32_t ra[32], rb[32];
        tc::tmem_ld32_async(t_row + c0, ra);
        tc::tmem_ld32_async(t_row + c0 + 32, rb);
        tc::tmem_wait_ld(ra);
        tc::reg_fence(rb);
        const uint64_t mw = qvalid ? ((uint64_t)cm[(c0 >> 5) + 1] << 32 | cm[c0 >> 5]) : 0ull;
        if (mw == 0ull) continue;
        // exact per-column distances (the same expressions the insertion
        // test uses), reduced to their minimum: a 64-column batch whose
        // minimum cannot beat the worst kept distance is skipped whole
        float v[64];
#pragma unroll
        for (int j = 0; j < 64; ++j) {
          float dot = __uint_as_float(j < 32 ? ra[j] : rb[j - 32]);
          if (FP8) dot = dot * (qs * cb[TC_N + c0 + j]);
          float dist;
          if (metric == METRIC_INNER_PRODUCT) {
            dist = -dot;
          } else if (metric == METRIC_COSINE) {
            dist = 1.0f - dot / (sqrtf(qn * cb[c0 + j]) + 1e-8f);
          } else {
            dist = fmaxf(0.f, fmaf(-2.0f, dot, qn + cb[c0 + j]));
          }
          v[j] = dist;
        }
        float m[32];
#pragma unroll
        for (int j = 0; j < 32; ++j) m[j] = fminf(v[j], v[j + 32]);
#pragma unroll
        for (int w = 16; w > 0; w >>= 1)
#pragma unroll
          for (int j = 0; j < w; ++j) m[j] = fminf(m[j], m[j + w]);
        if (!(m[0] < worst && m[0] <= tau_d)) continue;
        // columns that may enter: the warp walks them lane-parallel, one
        // per lane per round, fetching v[j] with a depth-6 select tree
        uint64_t pass = 0;
#pragma unroll
        for (int j = 0; j < 64; ++j) pass |= (uint64_t)(v[j] < worst && v[j] <= tau_d) << j;
        pass &= mw;
        while (pass) {
          const int j = __ffsll((long long)pass) - 1;
          pass &= pass - 1;
          const float dist = select64(v, j);
          if (dist < worst && dist <= tau_d) {
            heap_sift(h, kl, make_key(dist, v0 + c0 + j));
            const uint64_t root = h[0];
            worst = root == kSentinelKey ? kSentinelDist : key_dist(root);
          }
        }
      }
      if (tau_ptr && worst < published) {
        // heap full (worst < 1e30 only then): publish its kl-th distance
        atomicMin(tau_ptr, float_order(worst));
        published = worst;
      }
      tc::tc_fence_before();
      __syncwarp();
      if (lane == 0) tc::mbar_arrive(&acc_empty[buf]);
    }
    if (qvalid) {
      uint64_t* dst = a.partial + ((size_t)q * a.splits + split) * kl;
      for (int i = 0; i < kl; ++i) dst[i] = h[i * TC_M];
    }
  }

  __syncthreads();
  if (warp == 1) {
    // all MMAs must have retired before the accumulators are released; this
    // wait ignores the abort flag (bounded by time only)
    uint32_t no_abort = 0;
    tc::mbar_wait(mma_done, 0, &no_abort, a.status, 100000000ull);
    __syncwarp();
    tc::tc_fence_after();
    tc::tmem_dealloc(tmem, 512);
  }
}

// ---------------------------------------------------------------------------
// Query preparation: fp32 -> fp16 (round to nearest even, as the reference
// converts queries: ivf_quant_lookup.cu:953) or fp32 -> e4m3 with a per-query
// scale amax/448; ||q||^2 with fmaf in dimension order (:922-928).
// One warp per query.
// ---------------------------------------------------------------------------
template <bool FP8>
__global__ void __launch_bounds__(256) tc_prep_queries_kernel(const float* __restrict__ q, uint32_t nq, uint32_t dim,
                                                              uint32_t pd, void* __restrict__ out,
                                                              float* __restrict__ qnorm, float* __restrict__ qscale,
                                                              uint32_t* __restrict__ tau) {
  const uint32_t qi = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (qi >= nq) return;
  const float* src = q + (size_t)qi * dim;
  if (lane == 0) {
    tau[qi] = float_order(kSentinelDist);
    float s = 0.f;
    for (uint32_t d = 0; d < dim; ++d) s = fmaf(src[d], src[d], s);
    qnorm[qi] = s;
  }
  if (FP8) {
    float amax = 0.f;
    for (uint32_t d = lane; d < dim; d += 32) amax = fmaxf(amax, fabsf(src[d]));
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) amax = fmaxf(amax, __shfl_xor_sync(0xffffffffu, amax, o));
    const float scale = amax > 0.f ? amax / 448.0f : 1.0f;
    if (lane == 0) qscale[qi] = scale;
    uint8_t* o8 = static_cast<uint8_t*>(out) + (size_t)qi * pd;
    for (uint32_t d = lane; d < pd; d += 32)
      o8[d] = d < dim ? (uint8_t)__nv_cvt_float_to_fp8(src[d] / scale, __NV_SATFINITE, __NV_E4M3) : (uint8_t)0;
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
  for (uint32_t d = lane; d < dim; d += 32) {
    const double u = q[d], w = __ldg(x + d);
    if (metric == METRIC_L2) {
      const double t = u - w;
      a += t * t;
    } else {
      a += u * w;
      b += u * u;
      c += w * w;
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
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const uint32_t total = s.lists * s.kl;
  const uint64_t* src = s.partial + (size_t)q * total;
  if (threadIdx.x == 0) incomplete = 0;
  for (uint32_t i = threadIdx.x; i < s.pow2; i += SEL_THREADS) keys[i] = i < total ? src[i] : kSentinelKey;
  __syncthreads();
  block_bitonic_sort(keys, s.pow2);
  const uint32_t kp = min(s.shortlist, total);
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
  if (incomplete && threadIdx.x == 0) set_status(s.status, kStatusOverflow);

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
      if (threadIdx.x == 0) {
        const float dk = key_dist(keys[s.k - 1]);
        float qn = 0.f;
        for (uint32_t d = 0; d < s.dim; ++d) qn = fmaf(qv[d], qv[d], qn);
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

template <bool FP8, int KL, int STAGES>
cudaError_t launch_scan_kernel(const CUtensorMap& ta, const CUtensorMap& tb, const TcScanArgs& a, uint32_t grid,
                               cudaStream_t stream) {
  using L = ScanSmem<KL, STAGES>;
  auto kern = tc_scan_kernel<FP8, KL, STAGES>;
  cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)L::bytes);
  if (e != cudaSuccess) return e;
  kern<<<grid, SCAN_THREADS, L::bytes, stream>>>(ta, tb, a);
  note_launch();
  return cudaGetLastError();
}

template <bool FP8>
cudaError_t dispatch_scan(int kl, const CUtensorMap& ta, const CUtensorMap& tb, const TcScanArgs& a, uint32_t grid,
                          cudaStream_t stream) {
  switch (kl) {
    case 16: return launch_scan_kernel<FP8, 16, 4>(ta, tb, a, grid, stream);
    case 32: return launch_scan_kernel<FP8, 32, 3>(ta, tb, a, grid, stream);
    case 48: return launch_scan_kernel<FP8, 48, 3>(ta, tb, a, grid, stream);
    default: return launch_scan_kernel<FP8, 64, 3>(ta, tb, a, grid, stream);
  }
}

size_t align_up(size_t v, size_t a) { return (v + a - 1) / a * a; }

}  // namespace

int launch_tc_scan(const TcTables& t, const float* queries, uint32_t nq, uint32_t k, MetricType metric,
                   const uint32_t* mask, GpuSearchResult* out, const FvScanOptions& opt, cudaStream_t stream) {
  const bool fp8 = t.fp8;
  const uint32_t elem = fp8 ? 1 : 2;
  const uint32_t kb_elems = fp8 ? 128 : 64;
  const uint32_t kblocks = (t.padded_dim + kb_elems - 1) / kb_elems;
  const uint32_t overfetch = opt.overfetch ? opt.overfetch : 4;
  const uint32_t shortlist = t.vectors ? std::min<uint32_t>(std::max(k, overfetch * k), 4096u) : k;
  const uint32_t kl = std::min<uint32_t>(64u, shortlist);            // heap entries per (query, range)
  const uint32_t kl_tmpl = std::min<uint32_t>(64u, (kl + 15) / 16 * 16);  // heap capacity (template)
  const uint32_t nqb = (nq + TC_M - 1) / TC_M;
  const uint32_t ntiles = (t.n + TC_N - 1) / TC_N;
  const int sms = device_sm_count();
  uint32_t splits = opt.splits ? opt.splits : std::max<uint32_t>(1u, (uint32_t)sms / nqb);
  splits = std::max(1u, std::min(splits, ntiles));
  // the select kernel sorts lists*kl keys in shared memory: <= 16384
  while (splits > 1 && next_pow2(splits * kl) > 16384u) --splits;
  uint32_t tps = (ntiles + splits - 1) / splits;
  splits = (ntiles + tps - 1) / tps;

  // scratch: prepared queries | ||q||^2 | q scales | partial heaps
  const size_t q_bytes = align_up((size_t)nq * t.padded_dim * elem, 1024);
  const size_t qn_bytes = align_up((size_t)nq * 4, 256);
  const size_t part_bytes = align_up((size_t)nq * splits * kl * 8, 256);
  uint8_t* scratch = static_cast<uint8_t*>(scratch_get(stream, q_bytes + 3 * qn_bytes + part_bytes));
  if (!scratch) return (int)cudaErrorMemoryAllocation;
  void* qprep = scratch;
  float* qnorm = reinterpret_cast<float*>(scratch + q_bytes);
  float* qscale = reinterpret_cast<float*>(scratch + q_bytes + qn_bytes);
  uint64_t* partial = reinterpret_cast<uint64_t*>(scratch + q_bytes + 2 * qn_bytes);
  uint32_t* tau = reinterpret_cast<uint32_t*>(scratch + q_bytes + 2 * qn_bytes + part_bytes);

  {
    ProfScope ps(fp8 ? "tc_prep_queries_fp8" : "tc_prep_queries_fp16", stream);
    const uint32_t blocks = (nq * 32 + 255) / 256;
    if (fp8)
      tc_prep_queries_kernel<true><<<blocks, 256, 0, stream>>>(queries, nq, t.dim, t.padded_dim, qprep, qnorm, qscale,
                                                               tau);
    else
      tc_prep_queries_kernel<false><<<blocks, 256, 0, stream>>>(queries, nq, t.dim, t.padded_dim, qprep, qnorm,
                                                                qscale, tau);
    note_launch();
  }

  CUtensorMap ta, tb;
  if (!encode_tmap(&ta, qprep, fp8, t.padded_dim, nq, (uint64_t)t.padded_dim * elem, TC_M) ||
      !encode_tmap(&tb, t.base, fp8, t.padded_dim, t.n, (uint64_t)t.padded_dim * elem, TC_N))
    return FV_ERR_ARG;

  TcScanArgs a{t.n,   nq,      kblocks, nqb, splits, tps, (int)metric, t.norms, t.scales, qnorm, qscale, mask, partial,
               tau, kl,     kl == shortlist ? 1u : 0u, status_word()};
  cudaError_t e;
  {
    ProfScope ps(fp8 ? "tc_scan_fp8" : "tc_scan_fp16", stream);
    e = fp8 ? dispatch_scan<true>((int)kl_tmpl, ta, tb, a, nqb * splits, stream)
            : dispatch_scan<false>((int)kl_tmpl, ta, tb, a, nqb * splits, stream);
  }
  if (e != cudaSuccess) return (int)e;

  SelectArgs s{partial, splits, kl, next_pow2(splits * kl), shortlist, k, queries, t.vectors, t.dim, (int)metric,
               opt.boundary_fp64 ? 1u : 0u, 0.f, out, status_word()};
  s.eps = opt.boundary_eps > 0.f ? opt.boundary_eps : (float)((t.dim + 31) / 32 + 5) * 2.0f * 5.960464477539063e-08f;
  const size_t sel_smem = (size_t)std::max(s.pow2, next_pow2(shortlist)) * 8;
  e = cudaFuncSetAttribute(tc_select_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sel_smem);
  if (e != cudaSuccess) return (int)e;
  {
    ProfScope ps("tc_select_rescore", stream);
    tc_select_kernel<<<nq, SEL_THREADS, sel_smem, stream>>>(s);
    note_launch();
  }
  return (int)cudaGetLastError();
}

}  // namespace fv
