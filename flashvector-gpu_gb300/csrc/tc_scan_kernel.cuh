// tc_scan_kernel.cuh -- the tcgen05 scan kernel template shared by the fp16
// and fp8 translation units (tc_scan_fp16.cu, tc_scan_fp8.cu), which each
// instantiate one precision so the two compile in parallel.
//
// Warp roles (64 + 128 G threads, one CTA per SM; G = 1, 2 or 4 epilogue
// groups, see below):
//   warp 0    TMA producer: per K block, a 128-query tile (A) and a 256-row
//             base tile (B), 128-byte-swizzled, into a STAGES-deep ring;
//   warp 1    TMEM owner + single-thread tcgen05.mma issuer (M=128, N=256,
//             fp32 accumulators, two 256-column buffers so the epilogue of
//             tile i overlaps the MMAs of tile i+1);
//   warps 2.. epilogue, 4 warps per group: thread r of a group owns query r
//             of the block (TMEM lane r),
//             turns dot products into distances, applies the slot mask and
//             keeps that query's best kl (distance, slot) keys in a shared-
//             memory max-heap. No distance matrix ever reaches HBM.
//
// Shared bound. Every query owns kl global "slots"; a CTA that keeps a key
// also lowers slot hash(row) of its query to the key's distance (red.min).
// Each slot then holds a distance of a distinct real row, so the maximum
// over the kl slots is >= the query's global kl-th best distance: a row
// farther than it cannot be in the shortlist, and every CTA scanning the
// query drops it. The maximum sits near rank kl * H(kl) of all rows scanned
// so far, so after the first tiles almost no row reaches the heap.
#pragma once

#include <cuda_fp16.h>
#include <cuda_fp8.h>

#include <type_traits>

#include "common.cuh"
#include "kernels.h"
#include "tc_ptx.cuh"
#include "topk.cuh"

namespace fv {

constexpr int TC_M = 128;                  // queries per CTA (TMEM lanes)
constexpr int TC_N = 256;                  // base rows per tile (MMA N)
constexpr int KB_BYTES = 128;              // K bytes per stage row (one 128B swizzle atom)
constexpr int A_STAGE = TC_M * KB_BYTES;   // 16 KB
constexpr int B_STAGE = TC_N * KB_BYTES;   // 32 KB

// threads of a scan CTA with G epilogue groups: warp 0 TMA, warp 1 MMA,
// 4 epilogue warps per group
__host__ __device__ constexpr int scan_threads(int G) { return 64 + 128 * G; }

struct TcScanArgs {
  uint32_t n, nq, kblocks, nqb, splits, tiles_per_split;
  const float* xnorm;    // [n] ||x||^2 of the fp32 rows (L2, cosine)
  const float* xscale;   // [n] per-row fp8 scale (FP8 only)
  const float* qnorm;    // [nq] ||q||^2
  const float* qscale;   // [nq] per-query fp8 scale (FP8 only)
  const uint32_t* mask;
  uint64_t* partial;     // [nq][splits][kl]
  uint32_t* tslot;       // [nq][tslot_stride] shared-bound slots (float_order distances)
  uint32_t tslot_stride; // kl rounded up to a multiple of 4 (padding slots hold 0)
  uint32_t kl;           // heap entries used (<= KL); == shortlist when the bound is shared
  uint32_t share;        // 1: the CTAs of a query share the slot bound (kl == shortlist)
  uint32_t* status;
  const QueryFilter* filters;  // per-query filters over slots (== logical ids), or null
  const float* qbound;         // per-query admission bound (distance), or null
  const uint32_t* active;      // per-query flags: only flagged queries are scanned (null: all)
  uint32_t tile_stride;        // scan every tile_stride-th 256-row tile (a sample when > 1)
  uint64_t wait_ns;            // limit of the pipeline's waits (the drains keep their own)
};

// PAIR: a CTA of a cta_group::2 pair holds half of each 256-row base tile.
// COLS: the epilogue stages per-column norms / scales (not the fused fp8
// forms, whose accumulator is the ranking value). A_STAGES: query-tile
// buffers (1 where the query tile is always resident).
template <int KL, int STAGES, int G, bool PAIR = false, bool COLS = true, int A_STAGES = STAGES>
struct ScanSmem {
  static constexpr size_t b_stage = PAIR ? B_STAGE / 2 : B_STAGE;
  static constexpr size_t a_off = 0;
  static constexpr size_t b_off = a_off + (size_t)A_STAGES * A_STAGE;
  static constexpr size_t heap_off = b_off + (size_t)STAGES * b_stage;
  static constexpr size_t col_off = heap_off + (size_t)G * KL * TC_M * 8;  // [4G warps][2][TC_N] floats
  static constexpr size_t cmask_off = col_off + (COLS ? 4 * G * 2 * TC_N * 4 : 0);  // [4G warps][8] words
  static constexpr size_t bar_off = cmask_off + 4 * G * 8 * 4;          // barriers
  static constexpr size_t nbars = 2 * STAGES + 5;
  static constexpr size_t misc_off = bar_off + nbars * 8;
  static constexpr size_t bytes = misc_off + 16 + 1024;                 // + alignment slack
};

// The fused fp8 forms (table scale, L2 / inner product): the accumulator is
// the ranking value, so no column data is staged.
template <bool FP8, int METRIC, bool TS>
constexpr bool kFusedScan = FP8 && TS && METRIC != METRIC_COSINE;

// G = 4 runs only the fused fp8 forms with one K block per tile, whose query
// tile is resident: one query-tile buffer.
template <bool FP8, int KL, int STAGES, int METRIC, int G, bool PAIR, bool TS>
using ScanLayout = ScanSmem<KL, STAGES, G, PAIR, !kFusedScan<FP8, METRIC, TS>, G == 4 ? 1 : STAGES>;

// Sift `key` down from position i of a max-heap of kl keys stored with
// stride TC_M (one heap per query row of the block).
static __device__ __forceinline__ void heap_down(uint64_t* h, int kl, int i, uint64_t key) {
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

// Turns kl unordered keys into a max-heap (bottom-up).
static __device__ __forceinline__ void heap_build(uint64_t* h, int kl) {
  for (int i = kl / 2 - 1; i >= 0; --i) heap_down(h, kl, i, h[i * TC_M]);
}

static __device__ __forceinline__ void heap_sift(uint64_t* h, int kl, uint64_t key) {
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

// v[j] for a lane-varying j without local memory: a 5-level select tree.
static __device__ __forceinline__ float select32(const float* v, int j) {
  float t[16];
#pragma unroll
  for (int i = 0; i < 16; ++i) t[i] = (j & 1) ? v[2 * i + 1] : v[2 * i];
#pragma unroll
  for (int i = 0; i < 8; ++i) t[i] = (j & 2) ? t[2 * i + 1] : t[2 * i];
#pragma unroll
  for (int i = 0; i < 4; ++i) t[i] = (j & 4) ? t[2 * i + 1] : t[2 * i];
#pragma unroll
  for (int i = 0; i < 2; ++i) t[i] = (j & 8) ? t[2 * i + 1] : t[2 * i];
  return (j & 16) ? t[1] : t[0];
}

// G epilogue groups, each with its own heaps, dumped as separate lists
// (partial row split * G + g). With G = 2 a full scan splits columns: both
// groups drain every tile, group g the columns [128 g, 128 g + 128) of it,
// so the MMA of tile i + 1 (the other accumulator buffer) runs while tile i
// is drained. A sampled scan (tile stride > 1, whose tile loads are further
// apart) alternates tiles instead: group g drains tiles g, g + 2, .. (each
// group owns one buffer), so each group's wait for its next tile overlaps
// the other group's work.
//
// G = 4 (fused fp8 with one K block per tile, shortlists above 48 keys; the
// host runs that call's sampled pre-pass with G = 2): 16 epilogue warps,
// group g draining the 32-column chunks g and g + 4 of every tile, in any
// scan (alternating tiles would put two groups on one accumulator buffer,
// and a parity wait cannot tell its phase from the phase two uses later).
// Heaps of at most 32 keys fit four groups' heaps in shared memory;
// interleaved chunks spread runs of consecutive slots over the groups.
//
// PAIR: the CTA is one of a cluster of two (a cta_group::2 pair) sharing the
// same base range: CTA r holds query block 2p + r and rows [128 r, 128 r +
// 128) of every 256-row tile; the even CTA issues M=256 MMAs whose 128
// accumulator lanes land in each CTA's TMEM, so each SM streams 16 KB of
// base per K block instead of 32 KB and the ring gets deeper. Both CTAs'
// TMA loads count on the even CTA's full barriers; the even CTA's commits
// are multicast to both CTAs' barriers; the odd CTA's epilogue arrives on
// the even CTA's accumulator barriers.
template <bool FP8, int KL, int STAGES, int METRIC, int G, bool PAIR, bool TS>
__global__ void __launch_bounds__(scan_threads(G), 1)
    tc_scan_kernel(const __grid_constant__ CUtensorMap tmA, const __grid_constant__ CUtensorMap tmB, TcScanArgs a) {
  using L = ScanLayout<FP8, KL, STAGES, METRIC, G, PAIR, TS>;
  constexpr uint32_t b_stage = (uint32_t)L::b_stage;
  constexpr int SCAN_THREADS = scan_threads(G);
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
  uint32_t qb, split, rank = 0;
  if constexpr (PAIR) {
    rank = tc::cluster_ctarank();
    const uint32_t c = blockIdx.x >> 1, npairs = (a.nqb + 1) / 2;
    qb = 2 * (c % npairs) + rank;
    split = c / npairs;
  } else {
    qb = blockIdx.x % a.nqb;
    split = blockIdx.x / a.nqb;
  }
  if (!PAIR && a.active) {
    // a re-scan of flagged queries: a block holding none of them leaves at once
    int any = 0;
    for (int r = threadIdx.x; r < TC_M; r += SCAN_THREADS) {
      const uint32_t q = qb * TC_M + r;
      any |= (q < a.nq && a.active[q]) ? 1 : 0;
    }
    if (!__syncthreads_or(any)) return;
  }
  const uint32_t tstride = a.tile_stride ? a.tile_stride : 1u;
  const bool col_split = G == 4 || (G == 2 && tstride == 1);
  const uint32_t ntiles = ((a.n + TC_N - 1) / TC_N + tstride - 1) / tstride;
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
      // the epilogue warps (of both CTAs) that drain buffer b
      tc::mbar_init(&acc_empty[b], PAIR ? 8 : (col_split ? 4 * G : 4));
    }
    tc::mbar_init(mma_done, 1);
    *abort_flag = 0;
    tc::fence_mbar_init();
  }
  if (warp == 1) {
    if constexpr (PAIR)
      tc::tmem_alloc_pair(tmem_slot, 512);
    else
      tc::tmem_alloc(tmem_slot, 512);
    tc::tc_fence_before();
  }
  __syncthreads();
  if constexpr (PAIR) tc::cluster_sync();  // both CTAs' barriers exist before either signals the other's
  tc::tc_fence_after();
  const uint32_t tmem = *tmem_slot;
  // one K block per tile: the query tile is loaded once (with the first base
  // tile, into stage 0) and stays resident; only base tiles stream after it
  const bool a_resident = !PAIR && a.kblocks == 1;

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
        const int32_t row_b = (int32_t)((t_begin + i) * tstride * TC_N);
        for (uint32_t kb = 0; kb < a.kblocks; ++kb) {
          if (!tc::mbar_wait(&empty[stage], phase ^ 1, abort_flag, a.status, a.wait_ns)) {
            ok = false;
            break;
          }
          if constexpr (PAIR) {
            const uint32_t fb = tc::mapa(tc::smem_addr(&full[stage]), 0);  // the even CTA's full barrier
            if (rank == 0) tc::mbar_arrive_expect_tx(&full[stage], 2 * (A_STAGE + b_stage));
            tc::tma_load_2d_pair(sA + stage * A_STAGE, &tmA, fb, (int32_t)(kb * kb_elems), (int32_t)(qb * TC_M),
                                 pol_a);
            tc::tma_load_2d_pair(sB + stage * b_stage, &tmB, fb, (int32_t)(kb * kb_elems),
                                 row_b + (int32_t)(rank * (TC_N / 2)), pol_b);
          } else {
            const bool load_a = !a_resident || i == 0;
            tc::mbar_arrive_expect_tx(&full[stage], (load_a ? A_STAGE : 0) + B_STAGE);
            if (load_a)
              tc::tma_load_2d(sA + stage * A_STAGE, &tmA, &full[stage], (int32_t)(kb * kb_elems),
                              (int32_t)(qb * TC_M), pol_a);
            tc::tma_load_2d(sB + stage * B_STAGE, &tmB, &full[stage], (int32_t)(kb * kb_elems), row_b, pol_b);
          }
          issued_parity[stage] = (int32_t)phase;
          if (++stage == STAGES) {
            stage = 0;
            phase ^= 1;
          }
        }
      }
      // drain: every copy issued must have landed before the CTA may exit
      // (normally they all have; after an abort this waits a bounded time).
      // A pair's copies all count on the even CTA's barriers, which it drains.
      uint32_t no_abort = 0;
      if (!PAIR || rank == 0) {
#pragma unroll
        for (int s = 0; s < STAGES; ++s)
          if (issued_parity[s] >= 0)
            tc::mbar_wait(&full[s], (uint32_t)issued_parity[s], &no_abort, a.status, 100000000ull);
      }
    }
  } else if (warp == 1) {
    // ------------------------------------------------------- MMA issuer
    if (lane == 0 && (!PAIR || rank == 0)) {
      constexpr uint32_t idesc = tc::idesc_f32acc(0, 0, PAIR ? 2 * TC_M : TC_M, TC_N);
      uint32_t stage = 0, phase = 0;
      bool ok = true;
      for (uint32_t i = 0; ok && i < my_tiles; ++i) {
        const uint32_t buf = i & 1, use = i >> 1;
        if (!tc::mbar_wait(&acc_empty[buf], (use & 1) ^ 1, abort_flag, a.status, a.wait_ns)) break;
        tc::tc_fence_after();
        const uint32_t d_tmem = tmem + buf * TC_N;
        for (uint32_t kb = 0; kb < a.kblocks; ++kb) {
          if (!tc::mbar_wait(&full[stage], phase, abort_flag, a.status, a.wait_ns)) {
            ok = false;
            break;
          }
          tc::tc_fence_after();
          const uint32_t a_base = tc::smem_addr(sA + (a_resident ? 0u : stage * A_STAGE));
          const uint32_t b_base = tc::smem_addr(sB + stage * b_stage);
#pragma unroll
          for (uint32_t kk = 0; kk < 4; ++kk) {
            if constexpr (PAIR)
              tc::mma_pair<FP8>(d_tmem, tc::sdesc_k_sw128(a_base + kk * 32), tc::sdesc_k_sw128(b_base + kk * 32),
                                idesc, (kb | kk) != 0);
            else
              tc::mma<FP8>(d_tmem, tc::sdesc_k_sw128(a_base + kk * 32), tc::sdesc_k_sw128(b_base + kk * 32), idesc,
                           (kb | kk) != 0);
          }
          if constexpr (PAIR)
            tc::mma_commit_pair(&empty[stage], 3);
          else
            tc::mma_commit(&empty[stage]);
          if (++stage == STAGES) {
            stage = 0;
            phase ^= 1;
          }
        }
        if (ok) {
          if constexpr (PAIR)
            tc::mma_commit_pair(&acc_full[buf], 3);
          else
            tc::mma_commit(&acc_full[buf]);
        }
      }
      if constexpr (PAIR)
        tc::mma_commit_pair(mma_done, 3);
      else
        tc::mma_commit(mma_done);
    }
  } else {
    // --------------------------------------------------------- epilogue
    const int quad = warp & 3;                    // TMEM lane quadrant of this warp
    const int grp = (warp - 2) >> 2;              // epilogue group
    const int row = quad * 32 + lane;             // query row in the block
    const uint32_t q = qb * TC_M + row;
    const bool qvalid = q < a.nq && (a.active == nullptr || a.active[q] != 0u);
    uint64_t* h = heap + (size_t)grp * KL * TC_M + row;
    const int kl = (int)a.kl;
    for (int i = 0; i < kl; ++i) h[i * TC_M] = kSentinelKey;
    const float qn = qvalid ? __ldg(a.qnorm + q) : 0.f;
    const QueryFilter qf = (a.filters && qvalid) ? load_filter(a.filters, q) : QueryFilter{nullptr, 0u, 0u};
    const float qs = (FP8 && qvalid) ? __ldg(a.qscale + q) : 1.f;
    // fp8 L2 and inner product over a table-scale table: the accumulator is
    // the ranking value in the table's units (L2: the norm digits fold
    // -||x||^2 / (2 s s_q) into the dot product), v = sc * acc with
    // sc = -2 s s_q (L2) or -s s_q (IP), a power of two, so the scaling is
    // exact and no per-row data is read. A per-row-scale table reads each
    // row's scale (and norm) per value instead.
    constexpr bool fused = FP8 && METRIC != METRIC_COSINE && TS;
    const float sc = fused ? (METRIC == METRIC_L2 ? -2.0f : -1.0f) * qs * __ldg(a.xscale) : 1.f;
    const float inv_sc = fused ? __fdiv_rn(1.0f, sc) : 1.f;
    float worst = kSentinelDist;  // this CTA's kl-th best distance (1e30 until the heap is full)
    // admission bound: the query's pre-pass bound, lowered by the shared slots
    float bound = (a.qbound && qvalid) ? __ldg(a.qbound + q) : kSentinelDist;
    uint32_t* slots = (a.share && qvalid) ? a.tslot + (size_t)q * a.tslot_stride : nullptr;

    // Until kl keys are held the heap is an unordered list (appends cost
    // one store); on the kl-th key it is heapified once and from then on a
    // key replaces the root. The kept set is the same either way.
    int fill = 0;
    auto keep = [&](float dist, uint32_t slot) {
      const uint64_t key = make_key(dist, slot);
      if (fill < kl) {
        h[fill * TC_M] = key;
        if (++fill == kl) {
          heap_build(h, kl);
          worst = key_dist(h[0]);
        }
      } else {
        heap_sift(h, kl, key);
        worst = key_dist(h[0]);
      }
      if (slots) atomicMin(slots + __umulhi(slot * 2654435761u, (uint32_t)kl), float_order(dist));
    };
    // admission threshold in the v domain, refreshed when worst or bound
    // moves: every v whose distance could enter (D(v) < worst and D(v) <=
    // bound) has v <= thr (for L2 the subtraction of the query norm is padded
    // by a relative slack, so thr errs on the admitting side; exact tests
    // follow). Fused fp8 tests the accumulator instead: v <= thr <=> acc >=
    // thr / sc (sc < 0, a power of two), padded the same way against underflow.
    float thr = 0.f;
    auto refresh = [&]() {
      const float w = fminf(worst, bound);
      thr = METRIC == METRIC_L2 ? (w - qn) + 1e-6f * (fabsf(w) + fabsf(qn)) + 1e-30f : w;
      if (fused) {
        thr *= inv_sc;
        thr -= 1e-6f * fabsf(thr) + 1e-37f;
      }
    };

    // per-warp copy of the current tile's column data (norms, fp8 factors,
    // mask words): staged by the warp itself, so the epilogue warps never
    // wait on one another. The global loads for tile i + G are issued into
    // registers while tile i is processed (lane l holds columns l + 32 r).
    float* cb = colbuf + (warp - 2) * 2 * TC_N;
    uint32_t* cm = colmask + (warp - 2) * 8;
    // this group's tiles (first, step) and columns [c_lo, c_hi) of each;
    // only its own columns' data is staged
    const uint32_t t_first = col_split ? 0u : (uint32_t)grp, t_step = col_split ? 1u : (uint32_t)G;
    const int c_lo = col_split ? grp * (TC_N / G) : 0, c_hi = col_split ? c_lo + TC_N / G : TC_N;
    float pre_n[TC_N / 32], pre_s[TC_N / 32];
    uint32_t pre_m = 0;
    auto prefetch = [&](uint32_t tile) {
      const uint32_t v0n = (t_begin + tile) * tstride * TC_N;
#pragma unroll
      for (int r = 0; r < TC_N / 32; ++r) {
        const uint32_t slot = v0n + lane + 32 * r;
        const bool in = slot < a.n && 32 * r >= c_lo && 32 * r < c_hi;
        pre_n[r] = (METRIC != METRIC_INNER_PRODUCT && !fused && in) ? __ldg(a.xnorm + slot) : 0.f;
        // per-column factor of the scaled dot: -2 xs (L2), -xs (IP), xs
        // (cosine) for per-row scales; a table-scale table needs none
        const float xs = (FP8 && !fused && in) ? __ldg(a.xscale + slot) : 0.f;
        pre_s[r] = METRIC == METRIC_L2 ? -2.0f * xs : (METRIC == METRIC_INNER_PRODUCT ? -xs : xs);
      }
      pre_m = 0;
      if (lane < 8) {
        const uint32_t c0 = v0n + lane * 32;
        if (c0 < a.n) {
          const uint32_t cnt = min(32u, a.n - c0);
          pre_m = cnt == 32 ? 0xFFFFFFFFu : ((1u << cnt) - 1u);
          if (a.mask) pre_m &= __ldg(a.mask + (c0 >> 5));
        }
      }
    };
    if (t_first < my_tiles) prefetch(t_first);
    for (uint32_t i = t_first; i < my_tiles; i += t_step) {
      const uint32_t buf = i & 1, use = i >> 1;
      const uint32_t v0 = (t_begin + i) * tstride * TC_N;
      __syncwarp();
#pragma unroll
      for (int r = 0; r < TC_N / 32; ++r) {
        if (32 * r < c_lo || 32 * r >= c_hi) continue;
        if (METRIC != METRIC_INNER_PRODUCT && !fused) cb[lane + 32 * r] = pre_n[r];
        if (FP8 && !fused) cb[TC_N + lane + 32 * r] = pre_s[r];
      }
      if (lane < 8) cm[lane] = pre_m;
      __syncwarp();
      if (i + t_step < my_tiles) prefetch(i + t_step);
      // the shared bound, loaded before the accumulator wait hides its latency
      uint32_t smax = 0;
      if (slots)
        for (uint32_t s4 = 0; s4 < a.tslot_stride; s4 += 4) {
          const uint4 w = __ldcg(reinterpret_cast<const uint4*>(slots + s4));
          smax = max(smax, max(max(w.x, w.y), max(w.z, w.w)));
        }
      if (!tc::mbar_wait(&acc_full[buf], use & 1, abort_flag, a.status, a.wait_ns)) break;
      tc::tc_fence_after();
      if (slots && smax != 0xFFFFFFFFu) bound = fminf(bound, order_float(smax));
      refresh();

      const uint32_t t_row = tmem + ((uint32_t)(quad * 32) << 16) + buf * TC_N;
      if constexpr (G == 4) {
        // fused fp8, the group's 32-column chunks at 32 g and 128 + 32 g: the
        // accumulator is the ranking value (v = sc * acc, sc < 0), so a
        // larger accumulator is better; a chunk whose largest value cannot
        // enter is skipped whole
        auto chunk32 = [&](const uint32_t (&rr)[32], uint32_t col, uint32_t m32) {
          if (m32 == 0u) return;
          auto max3 = [](float x, float y, float z) {
            float d;
            asm("max.f32 %0, %1, %2, %3;" : "=f"(d) : "f"(x), "f"(y), "f"(z));
            return d;
          };
          float v[32];
#pragma unroll
          for (int j = 0; j < 32; ++j) v[j] = __uint_as_float(rr[j]);
          float t1[11];
#pragma unroll
          for (int j = 0; j < 10; ++j) t1[j] = max3(v[3 * j], v[3 * j + 1], v[3 * j + 2]);
          t1[10] = fmaxf(v[30], v[31]);
          const float top = fmaxf(max3(max3(t1[0], t1[1], t1[2]), max3(t1[3], t1[4], t1[5]), max3(t1[6], t1[7], t1[8])),
                                  fmaxf(t1[9], t1[10]));
          if (!(top >= thr)) return;
          uint32_t pass = 0;
#pragma unroll
          for (int j = 0; j < 32; ++j) pass |= (uint32_t)(v[j] >= thr) << j;
          pass &= m32;
          while (pass) {
            const int j = __ffs(pass) - 1;
            pass &= pass - 1;
            const float x = select32(v, j) * sc;
            const float d = METRIC == METRIC_L2 ? fmaxf(0.f, qn + x) : x;
            if (d < worst && d <= bound) {
              keep(d, v0 + col + (uint32_t)j);
              refresh();
            }
          }
        };
#pragma unroll 1
        for (int h = 0; h < 2; ++h) {
          const uint32_t col = 128u * (uint32_t)h + 32u * (uint32_t)grp;
          uint32_t ra[32];
          __syncwarp();  // tcgen05.ld is warp-collective: reconverge after the divergent insertions
          tc::tmem_ld32_async(t_row + col, ra);
          uint32_t m32 = qvalid ? cm[col >> 5] : 0u;
          if (qf.words) m32 &= filter_word(qf, (v0 + col) >> 5);
          tc::tmem_wait_ld(ra);
          chunk32(ra, col, m32);
        }
      } else {
#pragma unroll 1
        for (int c0 = c_lo; c0 < c_hi; c0 += 64) {
          uint32_t ra[32], rb[32];
          __syncwarp();  // tcgen05.ld is warp-collective: reconverge after the divergent insertions
          tc::tmem_ld32_async(t_row + c0, ra);
          tc::tmem_ld32_async(t_row + c0 + 32, rb);
          uint64_t mw = qvalid ? ((uint64_t)cm[(c0 >> 5) + 1] << 32 | cm[c0 >> 5]) : 0ull;
          if (qf.words) {
            const uint32_t w0 = (v0 + (uint32_t)c0) >> 5;
            mw &= ((uint64_t)filter_word(qf, w0 + 1) << 32) | filter_word(qf, w0);
          }
          tc::tmem_wait_ld(ra);
          tc::reg_fence(rb);
          if (mw == 0ull) continue;
          // the chunk's admission test and insertions; FU: the accumulator is
          // the ranking value (fp8 table-scale tables)
          auto chunk = [&](auto fu_tag) {
            constexpr bool FU = decltype(fu_tag)::value;
            // per-column values v, v[0..32) columns c0.., v[32..64) columns
            // c0+32..; the distance is D(v): L2  D(v) = max(0, ||q||^2 + v) with
            // v = ||x||^2 - 2 <q, x> (the query's norm is added after the
            // minimum, D being monotone), IP  D(v) = v = -<q, x>, cosine the
            // full expression. FP8 cosine dots carry the query and table scales.
            float v[64];
            if constexpr (FU) {
#pragma unroll
              for (int j = 0; j < 64; ++j) v[j] = __uint_as_float(j < 32 ? ra[j] : rb[j - 32]);
            } else if (METRIC == METRIC_COSINE) {
#pragma unroll
              for (int j = 0; j < 64; ++j) {
                float dot = __uint_as_float(j < 32 ? ra[j] : rb[j - 32]);
                if (FP8) dot = dot * (qs * cb[TC_N + c0 + j]);
                v[j] = 1.0f - dot / (sqrtf(qn * cb[c0 + j]) + 1e-8f);
              }
            } else {
              const float4* nb = reinterpret_cast<const float4*>(cb + c0);
              const float4* sb = reinterpret_cast<const float4*>(cb + TC_N + c0);
#pragma unroll
              for (int j4 = 0; j4 < 16; ++j4) {
                const float4 n4 = METRIC == METRIC_L2 ? nb[j4] : make_float4(0.f, 0.f, 0.f, 0.f);
                const float4 s4 = FP8 ? sb[j4] : make_float4(0.f, 0.f, 0.f, 0.f);
                const float nv[4] = {n4.x, n4.y, n4.z, n4.w};
                const float sv[4] = {s4.x, s4.y, s4.z, s4.w};
#pragma unroll
                for (int e = 0; e < 4; ++e) {
                  const int j = 4 * j4 + e;
                  const float dot = __uint_as_float(j < 32 ? ra[j] : rb[j - 32]);
                  if (FP8)  // per-row scales: -2 xs (L2) or -xs (IP) in sv
                    v[j] = METRIC == METRIC_L2 ? fmaf(dot * qs, sv[e], nv[e]) : (dot * qs) * sv[e];
                  else
                    v[j] = METRIC == METRIC_L2 ? fmaf(-2.0f, dot, nv[e]) : -dot;
                }
              }
            }
            // D: distance from v (fused fp8: from the accumulator, v = sc * acc)
            auto D = [&](float x) {
              if (FU) x *= sc;
              return METRIC == METRIC_L2 ? fmaxf(0.f, qn + x) : x;
            };
            // better(x, y): the smaller v, i.e. the larger accumulator when fused
            auto better = [](float x, float y) { return FU ? fmaxf(x, y) : fminf(x, y); };
            auto may = [&](float x) { return FU ? x >= thr : x <= thr; };
            // a tree of three-input bests: a 64-column batch whose best cannot
            // enter is skipped whole (the common case once warm); the pairwise
            // bests (j, j + 32) are formed only for a batch that passes
            // best of three in one instruction (three-input min / max)
            auto best3 = [](float x, float y, float z) {
              float d;
              if (FU)
                asm("max.f32 %0, %1, %2, %3;" : "=f"(d) : "f"(x), "f"(y), "f"(z));
              else
                asm("min.f32 %0, %1, %2, %3;" : "=f"(d) : "f"(x), "f"(y), "f"(z));
              return d;
            };
            float r[22], s8[8];
#pragma unroll
            for (int i = 0; i < 21; ++i) r[i] = best3(v[3 * i], v[3 * i + 1], v[3 * i + 2]);
            r[21] = v[63];
#pragma unroll
            for (int i = 0; i < 7; ++i) s8[i] = best3(r[3 * i], r[3 * i + 1], r[3 * i + 2]);
            s8[7] = r[21];
            const float top = best3(best3(s8[0], s8[1], s8[2]), best3(s8[3], s8[4], s8[5]), better(s8[6], s8[7]));
            if (!(mw != 0ull && may(top))) return;
            float m1[32];
#pragma unroll
            for (int j = 0; j < 32; ++j) m1[j] = better(v[j], v[j + 32]);
            // pairs (j, j+32) that may hold a candidate, walked lane-parallel
            uint32_t pass = 0;
#pragma unroll
            for (int j = 0; j < 32; ++j) pass |= (uint32_t)may(m1[j]) << j;
            pass &= (uint32_t)mw | (uint32_t)(mw >> 32);
            while (pass) {
              const int j = __ffs(pass) - 1;
              pass &= pass - 1;
              const float dlo = D(select32(v, j));
              const float dhi = D(select32(v + 32, j));
              if (((mw >> j) & 1ull) && dlo < worst && dlo <= bound) {
                keep(dlo, v0 + c0 + j);
                refresh();
              }
              if (((mw >> (j + 32)) & 1ull) && dhi < worst && dhi <= bound) {
                keep(dhi, v0 + c0 + j + 32);
                refresh();
              }
            }
          };
          chunk(std::integral_constant<bool, fused>{});
        }
      }
      tc::tc_fence_before();
      __syncwarp();
      if (lane == 0) {
        // relaxed: the buffer's TMEM values are in registers (wait::ld); the
        // arrival must not wait for this lane's shared-bound red.min updates
        if (PAIR && rank != 0)
          tc::mbar_arrive_cluster_relaxed(tc::mapa(tc::smem_addr(&acc_empty[buf]), 0));
        else
          tc::mbar_arrive_relaxed(&acc_empty[buf]);
      }
    }
    if (qvalid) {
      // entry 0 of a dumped list is its largest key (the select kernel tests
      // it for overflow): a full heap has it there already; a list that never
      // filled gets one of its sentinels moved there
      if (fill > 0 && fill < kl) {
        h[fill * TC_M] = h[0];
        h[0] = kSentinelKey;
      }
      uint64_t* dst = a.partial + (((size_t)q * a.splits + split) * G + grp) * kl;
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
    if constexpr (PAIR)
      tc::tmem_dealloc_pair(tmem, 512);
    else
      tc::tmem_dealloc(tmem, 512);
  }
  // a pair's CTAs read each other's shared memory (MMA operands, barriers):
  // neither leaves before the other is done
  if constexpr (PAIR) tc::cluster_sync();
}


template <bool FP8, int KL, int STAGES, int METRIC, int G, bool PAIR = false, bool TS = true>
cudaError_t launch_scan_kernel(const CUtensorMap& ta, const CUtensorMap& tb, const TcScanArgs& a, uint32_t grid,
                               cudaStream_t stream) {
  using L = ScanLayout<FP8, KL, STAGES, METRIC, G, PAIR, TS>;
  static_assert(L::bytes <= 227 * 1024, "scan shared memory above the 227 KB per-CTA limit");
  auto kern = tc_scan_kernel<FP8, KL, STAGES, METRIC, G, PAIR, TS>;
  cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)L::bytes);
  if (e != cudaSuccess) return e;
  if constexpr (PAIR) {
    // grid = 2 CTAs per (query-block pair, split), clusters of two
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(grid, 1, 1);
    cfg.blockDim = dim3(scan_threads(G), 1, 1);
    cfg.dynamicSmemBytes = L::bytes;
    cfg.stream = stream;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = 2;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    e = cudaLaunchKernelEx(&cfg, kern, ta, tb, a);
    note_launch();
    return e;
  }
  kern<<<grid, scan_threads(G), L::bytes, stream>>>(ta, tb, a);
  note_launch();
  return cudaGetLastError();
}

// groups == 2 (short K: one or two K blocks per tile, where the epilogue
// rather than the MMA bounds a tile) halves the stage ring and caps the heap
// at 48 entries so that two groups' heaps fit next to it; groups == 4 (fused
// fp8, one K block) caps it at 32. groups == -1 selects the CTA-pair
// variant (grid = 2 CTAs per cluster).
template <bool FP8, int METRIC, bool TS>
cudaError_t dispatch_scan_kl(int kl, int groups, const CUtensorMap& ta, const CUtensorMap& tb, const TcScanArgs& a,
                             uint32_t grid, cudaStream_t stream) {
  if (groups == -1) {
    // cta_group::2 pairs (one epilogue group): 16 KB of base per stage frees
    // room for 4-6 stages
    switch (kl) {
      case 16: return launch_scan_kernel<FP8, 16, 6, METRIC, 1, true, TS>(ta, tb, a, grid, stream);
      case 32: return launch_scan_kernel<FP8, 32, 5, METRIC, 1, true, TS>(ta, tb, a, grid, stream);
      case 48: return launch_scan_kernel<FP8, 48, 5, METRIC, 1, true, TS>(ta, tb, a, grid, stream);
      default: return launch_scan_kernel<FP8, 64, 4, METRIC, 1, true, TS>(ta, tb, a, grid, stream);
    }
  }
  if (groups == 4) {
    // fused fp8 with one K block per tile only (the layout keeps one
    // query-tile buffer); heaps of 16 or 32 keys
    if constexpr (kFusedScan<FP8, METRIC, TS>) {
      if (a.kblocks != 1) return cudaErrorInvalidValue;
      if (kl <= 16) return launch_scan_kernel<FP8, 16, 4, METRIC, 4, false, TS>(ta, tb, a, grid, stream);
      return launch_scan_kernel<FP8, 32, 2, METRIC, 4, false, TS>(ta, tb, a, grid, stream);
    }
    return cudaErrorInvalidValue;
  }
  if (groups == 2) {
    switch (kl) {
      case 16: return launch_scan_kernel<FP8, 16, 3, METRIC, 2, false, TS>(ta, tb, a, grid, stream);
      case 32: return launch_scan_kernel<FP8, 32, 2, METRIC, 2, false, TS>(ta, tb, a, grid, stream);
      default: return launch_scan_kernel<FP8, 48, 2, METRIC, 2, false, TS>(ta, tb, a, grid, stream);
    }
  }
  switch (kl) {
    case 16: return launch_scan_kernel<FP8, 16, 4, METRIC, 1, false, TS>(ta, tb, a, grid, stream);
    case 32: return launch_scan_kernel<FP8, 32, 3, METRIC, 1, false, TS>(ta, tb, a, grid, stream);
    case 48: return launch_scan_kernel<FP8, 48, 3, METRIC, 1, false, TS>(ta, tb, a, grid, stream);
    default: return launch_scan_kernel<FP8, 64, 3, METRIC, 1, false, TS>(ta, tb, a, grid, stream);
  }
}

template <bool FP8>
cudaError_t dispatch_scan(int kl, int groups, int metric, bool table_scale, const CUtensorMap& ta,
                          const CUtensorMap& tb, const TcScanArgs& a, uint32_t grid, cudaStream_t stream) {
  // TS (fp8 only): false for a per-row-scale table, whose L2 / IP epilogue
  // reads each row's scale and norm; cosine reads them either way
  if constexpr (FP8) {
    if (!table_scale && metric == METRIC_INNER_PRODUCT)
      return dispatch_scan_kl<FP8, METRIC_INNER_PRODUCT, false>(kl, groups, ta, tb, a, grid, stream);
    if (!table_scale && metric == METRIC_L2)
      return dispatch_scan_kl<FP8, METRIC_L2, false>(kl, groups, ta, tb, a, grid, stream);
  }
  switch (metric) {
    case METRIC_INNER_PRODUCT:
      return dispatch_scan_kl<FP8, METRIC_INNER_PRODUCT, true>(kl, groups, ta, tb, a, grid, stream);
    case METRIC_COSINE: return dispatch_scan_kl<FP8, METRIC_COSINE, true>(kl, groups, ta, tb, a, grid, stream);
    default: return dispatch_scan_kl<FP8, METRIC_L2, true>(kl, groups, ta, tb, a, grid, stream);
  }
}

}  // namespace fv
