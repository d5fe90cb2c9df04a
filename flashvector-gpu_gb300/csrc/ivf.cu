// ivf.cu -- IVF-PQ, IVF-SQ8 and IVF-RaBitQ inverted-list scans.
//
// Replaces launch_ivf_pq_search / launch_ivf_sq_search /
// launch_ivf_rabitq_search and their kernels (ivf_pq_lookup.cu:14-444,
// ivf_quant_lookup.cu:18-870, ivf_rerank.cuh:49-160) with the same inputs,
// clamps and result semantics:
//   * top_k <= 256; nprobe clamped to [1, nlist];
//     shortlist = rerank_k ? rerank_k : top_k, >= top_k, <= 10240;
//     exact rerank when rerank_k != 1 and fp32 rows are present;
//   * coarse probe: the nprobe nearest centroids by squared L2 accumulated
//     with fmaf in dimension order (ivf_rerank.cuh:78-84) -- exact here, by
//     (distance, list id);
//   * PQ: residual LUT[m][c] = sum_sd fmaf(((q - centroid) - codeword)^2)
//     per (query, list) in shared memory (ivf_pq_lookup.cu:150-162), ADC =
//     the LUT entries of a row's codes added in sub-space order (:176-178);
//     SQ8: sum_d fmaf over (q - centroid) - fmaf(code, scale, min)
//     (ivf_quant_lookup.cu:83-87), L2 whatever the metric;
//     RaBitQ: the query rotated once per query (three rounds of sign flip,
//     Walsh-Hadamard butterflies, 1/sqrt(P) scale: ivf_quant_lookup.cu:
//     337-376), per (query, list) its rotated residual quantised to 4 bits
//     over [min, max] as four bit-planes (:381-460), per posting the
//     popcount estimate (:462-489) with its roundings fixed
//     (rabitq_estimate below);
//   * shortlist = the best `shortlist` (approx distance, id) keys; rerank
//     with the reference's warp-order fp32 distance; the first top_k by
//     (distance, id) are returned.
// Because every distance is evaluated in the reference's operation order,
// the results are bit-identical to the oracle's restatement.
//
// Machine mapping. The coarse probe is the exact flat scan kernel in its
// fused-FMA mode (a Q x nlist tiled scan with a fused top-nprobe). The list
// scan is one persistent launch: CTAs pull queries from a device work
// counter and drain that query's (query, list) pairs: per pair the LUT (or
// the query residual) is built in shared memory, the posting list is
// streamed with 16-byte code loads (contiguous rows when the codes are laid
// out list-major, gathered by id in the reference's layout), and a running
// shortlist is kept in shared memory: rows whose key cannot beat the
// current shortlist's worst key are dropped, the rest are appended to a
// buffer that is bitonic-merged into the shortlist when it fills.
#include <cuda_fp16.h>

#include "../../include/fv_bridge.h"
#include "common.cuh"
#include "kernels.h"
#include "topk.cuh"

namespace fv {

namespace {

constexpr int IVF_THREADS = 256;
constexpr uint32_t IVF_BUF = 1536;         // candidate buffer entries (>= 1.5 rounds of 1,024 postings)
constexpr uint32_t MAX_SHORTLIST = 10240;  // reference clamp (ivf_rerank.cuh:12)

enum IvfMode { IVF_PQ = IVF_MODE_PQ, IVF_SQ8 = IVF_MODE_SQ8, IVF_RABITQ = IVF_MODE_RABITQ };

struct IvfArgs {
  const float* centroids;   // [nlist][dim]
  const float* codebooks;   // PQ: [m][256][sub]
  const float* sq_mins;     // SQ8: [dim]
  const float* sq_scales;   // SQ8: [dim]
  const uint8_t* codes;     // [N][code_bytes] by id, or by list position when list_major
                            // (RaBitQ: the sign bits, code_bytes = 4 W)
  const uint32_t* offsets;  // [nlist + 1]
  const uint32_t* vec_ids;  // [N] ids in list order
  const float* vectors;     // fp32 rows (rerank) or null
  uint32_t num_vectors, dim, nlist, m_pq, sub_dim, code_bytes;
  const float* queries;
  uint32_t nq, top_k, nprobe, rerank_k, list_major;
  int metric;
  const uint32_t* mask;
  // the mask in list order: bit i of this array = mask bit of vec_ids[i], for
  // list positions i < list_n (null when there is no mask; positions past the
  // lists hold 0); one shared word per 32 postings replaces a dependent id +
  // mask-word load per posting
  const uint32_t* list_allow;
  uint32_t list_n;
  // the admitted list positions in list order (compacted from list_allow),
  // and per bit word the count of admitted positions before it: a list
  // whose mask admits under half of its postings is scanned over these
  // positions only (null when there is no mask)
  const uint32_t* adm_pos;
  const uint32_t* adm_prefix;  // [ceil(list_n / 32) + 1]
  const uint32_t* q_topk;         // per-query top_k / nprobe / rerank_k, or null (uniform)
  const uint32_t* q_nprobe;
  const uint32_t* q_rerank;
  const QueryFilter* filters;     // per-query filters over ids, or null
  const GpuSearchResult* probes;  // [nq][nprobe] coarse result (id = list)
  uint32_t* work;                 // work counter (zeroed before the launch)
  GpuSearchResult* out;
  uint32_t* status;
  uint32_t keys_pow2;             // pow2(largest shortlist + IVF_BUF)
  uint32_t items_per_q;           // G: a query's probed postings are cut into G ranges
  uint64_t* partial;              // G > 1: [nq * G][part_stride] sorted shortlists of the ranges
  uint32_t part_stride;           // >= every query's shortlist
  // RaBitQ
  const float* rot_centroids;     // [nlist][P]
  const float* rq_meta;           // [N][4] by id, or by list position when list_major
  const float* rot_signs;         // [3][P]
  uint32_t P, W;                  // rotated dimension (power of two), words of bits per row
  float inv_sqrt_p;               // 1.0f / sqrtf(P), correctly rounded
};

// Index of list position p in the compacted admitted positions (the count of
// admitted positions before p). p <= list_n.
__device__ __forceinline__ uint32_t adm_index(const IvfArgs& a, uint32_t p) {
  const uint32_t w = p >> 5, b = p & 31u;
  return __ldg(a.adm_prefix + w) + (b ? __popc(__ldg(a.list_allow + w) & ((1u << b) - 1u)) : 0u);
}

// The postings of list l as the scan walks them: [beg, end) list positions
// (compact = false), or [beg, end) indices into adm_pos (compact = true)
// when the list-order mask admits under half of the list.
struct ListSpan {
  uint32_t beg, end;
  bool compact;
};
__device__ __forceinline__ ListSpan list_span(const IvfArgs& a, uint32_t l) {
  const uint32_t lbeg = __ldg(a.offsets + l), lend = __ldg(a.offsets + l + 1);
  if (a.adm_pos != nullptr && lend > lbeg) {
    const uint32_t a0 = adm_index(a, lbeg), a1 = adm_index(a, lend);
    if (2 * (a1 - a0) < lend - lbeg) return ListSpan{a0, a1, true};
  }
  return ListSpan{lbeg, lend, false};
}

// Rerank of a query's shortlist keys[0, S) (sorted, sentinels last) with the
// reference's warp-order fp32 distance, sort, and the query's top k into
// out[q][0, top_k) (sentinels past k). Block-collective.
__device__ void ivf_finish_query(const IvfArgs& a, uint64_t* keys, uint32_t q, uint32_t S, uint32_t kq,
                                 bool do_rerank, const float* qv) {
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  if (do_rerank) {
    // Two candidates per warp pass (c and c + NW, both owned by warp c % NW
    // as with one at a time), so two rows' gathers are in flight per warp.
    constexpr uint32_t NW = IVF_THREADS / 32;
    for (uint32_t c0 = warp; c0 < S; c0 += 2 * NW) {
      const uint32_t c1 = c0 + NW;
      const uint64_t k0 = keys[c0], k1 = c1 < S ? keys[c1] : kSentinelKey;
      const bool v0 = k0 != kSentinelKey && key_slot(k0) < a.num_vectors;
      const bool v1 = k1 != kSentinelKey && key_slot(k1) < a.num_vectors;
      if (!v0 && !v1) continue;
      // an unused slot re-reads the other (valid) row and its result is dropped
      const uint32_t s0 = key_slot(v0 ? k0 : k1), s1 = key_slot(v1 ? k1 : k0);
      const float* const rows[2] = {a.vectors + (size_t)s0 * a.dim, a.vectors + (size_t)s1 * a.dim};
      float d[2];
      warp_metric_distances<2, 4>(qv, rows, a.dim, lane, (MetricType)a.metric, d);
      if (lane == 0) {
        if (v0) keys[c0] = make_key(d[0], s0);
        if (v1) keys[c1] = make_key(d[1], s1);
      }
    }
    const uint32_t p2 = next_pow2_dev(S);
    for (uint32_t i = S + tid; i < p2; i += IVF_THREADS) keys[i] = kSentinelKey;
    __syncthreads();
    block_bitonic_sort(keys, p2);
  }
  for (uint32_t r = tid; r < a.top_k; r += IVF_THREADS)
    a.out[(size_t)q * a.top_k + r] = key_to_result(r < S && r < kq ? keys[r] : kSentinelKey, nullptr);
}

// The reference's clamps (ivf_pq_lookup.cu:351-362) for one query: returns
// the shortlist length; top_k and nprobe are clamped in place.
__host__ __device__ __forceinline__ uint32_t ivf_clamps(uint32_t& top_k, uint32_t& nprobe, uint32_t rerank_k,
                                                        uint32_t nlist) {
  top_k = top_k < (uint32_t)kMaxTopK ? top_k : (uint32_t)kMaxTopK;
  nprobe = nprobe == 0 ? 1u : nprobe;
  nprobe = nprobe < nlist ? nprobe : nlist;
  uint32_t s = rerank_k == 0 ? top_k : rerank_k;
  s = s > top_k ? s : top_k;
  return s < MAX_SHORTLIST ? s : MAX_SHORTLIST;
}

struct IvfSmem {
  // [keys_pow2] u64 keys | table | query (dim f32) | PQ: query residual to the probed centroid (dim f32)
  // table: PQ LUT (m*256 f32); SQ8 residual+mins+scales (3*dim f32);
  //        RaBitQ rotated query (P f32) + rotated residual (P f32) + bit-planes (4*W u32)
  __host__ __device__ static size_t table_floats(int mode, uint32_t dim, uint32_t m_pq, uint32_t P) {
    return mode == IVF_PQ ? (size_t)m_pq * 256 : mode == IVF_SQ8 ? (size_t)3 * dim : (size_t)2 * P + P / 8;
  }
  static size_t bytes(int mode, uint32_t keys_pow2, uint32_t dim, uint32_t m_pq, uint32_t P) {
    size_t b = (size_t)keys_pow2 * 8;
    b += table_floats(mode, dim, m_pq, P) * 4;
    b += (size_t)dim * 4;
    if (mode == IVF_PQ) b += (size_t)dim * 4;
    return b + 64;
  }
};

// RaBitQ: the query rotated into rq[0, P) (block-collective). The rounds of
// the reference's rotation (sign flip; butterflies x + y, x - y at half
// length 1, 2, ..., P/2; scale by 1/sqrt(P)) with each round's scale and
// the next round's sign flip applied in one pass -- the same two roundings.
__device__ void rabitq_rotate_query(float* rq, const float* qs, const IvfArgs& a) {
  const int tid = threadIdx.x;
  const uint32_t P = a.P;
  for (uint32_t d = tid; d < P; d += IVF_THREADS) rq[d] = __fmul_rn(d < a.dim ? qs[d] : 0.f, __ldg(a.rot_signs + d));
  __syncthreads();
  for (int st = 0; st < 3; ++st) {
    for (uint32_t h = 1; h < P; h <<= 1) {
      for (uint32_t i = tid; i < P / 2; i += IVF_THREADS) {
        const uint32_t x0 = ((i & ~(h - 1)) << 1) | (i & (h - 1));  // (i / h) * 2h + i % h
        const float x = rq[x0], y = rq[x0 + h];
        rq[x0] = __fadd_rn(x, y);
        rq[x0 + h] = __fsub_rn(x, y);
      }
      __syncthreads();
    }
    const float* next = st < 2 ? a.rot_signs + (size_t)(st + 1) * P : nullptr;
    for (uint32_t d = tid; d < P; d += IVF_THREADS) {
      const float v = __fmul_rn(rq[d], a.inv_sqrt_p);
      rq[d] = next ? __fmul_rn(v, __ldg(next + d)) : v;
    }
    __syncthreads();
  }
}

// RaBitQ: the 4-bit code of the rotated query residual to list l
// (ivf_quant_lookup.cu:381-460): diff = rq - rot_centroid over all P
// coordinates, u = clamp(rint((diff - min) * (15 / range)), 0, 15) (all 0
// when range <= 1e-12), bit-plane j word w bit l = bit j of u[32 w + l].
// Writes planes[4][W]; returns (min, delta = range / 15, sum u) in s_par.
// Block-collective.
__device__ void rabitq_query_code(const float* rq, float* rdiff, uint32_t* planes, const IvfArgs& a, uint32_t l,
                                  float* s_par) {
  __shared__ float s_lo[IVF_THREADS / 32], s_hi[IVF_THREADS / 32];
  __shared__ uint32_t s_sum;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const float* rc = a.rot_centroids + (size_t)l * a.P;
  float lo = 1e30f, hi = -1e30f;
  for (uint32_t d = tid; d < a.P; d += IVF_THREADS) {
    const float v = __fsub_rn(rq[d], __ldg(rc + d));
    rdiff[d] = v;
    lo = fminf(lo, v);
    hi = fmaxf(hi, v);
  }
#pragma unroll
  for (int o = 16; o; o >>= 1) {
    lo = fminf(lo, __shfl_xor_sync(0xffffffffu, lo, o));
    hi = fmaxf(hi, __shfl_xor_sync(0xffffffffu, hi, o));
  }
  if (lane == 0) {
    s_lo[warp] = lo;
    s_hi[warp] = hi;
  }
  __syncthreads();
  if (tid == 0) {
    for (int w = 1; w < IVF_THREADS / 32; ++w) {
      lo = fminf(lo, s_lo[w]);
      hi = fmaxf(hi, s_hi[w]);
    }
    const float range = __fsub_rn(hi, lo);
    const bool live = range > 1e-12f;
    s_par[0] = lo;
    s_par[1] = live ? __fdiv_rn(range, 15.0f) : 0.f;
    s_par[2] = live ? __fdiv_rn(15.0f, range) : 0.f;
    s_sum = 0;
  }
  __syncthreads();
  const float qmin = s_par[0], delta = s_par[1], inv = s_par[2];
  uint32_t su = 0;
  for (uint32_t w = warp; w < a.W; w += IVF_THREADS / 32) {
    uint32_t u = 0;
    if (delta > 0.f) {
      const int qi = __float2int_rn(__fmul_rn(__fsub_rn(rdiff[w * 32 + lane], qmin), inv));
      u = (uint32_t)min(max(qi, 0), 15);
    }
    su += u;
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const uint32_t pj = __ballot_sync(0xffffffffu, (u >> j) & 1u);
      if (lane == 0) planes[j * a.W + w] = pj;
    }
  }
  su = __reduce_add_sync(0xffffffffu, su);
  if (lane == 0 && su) atomicAdd(&s_sum, su);
  __syncthreads();
  if (tid == 0) s_par[3] = (float)s_sum;  // exact: sum u <= 15 * 4096
  __syncthreads();
}

// RaBitQ estimate of one posting from s_bu = sum_j 2^j popc(bits & plane_j)
// and its meta m = {|r|^2, rescale, popcount, |x|^2}
// (ivf_quant_lookup.cu:462-489). The reference leaves the roundings to the
// compiler; here they are fixed:
//   t = fmaf(delta, 2 s_bu - sum_u, q_min * (2 popcount - P))
//   est_l2 = (q_c + |r|^2) - 2 (rescale * t)
//   IP: -0.5 ((|q|^2 + |x|^2) - est_l2); cosine: 0.5 est_l2.
__device__ __forceinline__ float rabitq_estimate(uint32_t s_bu, float4 m, float P, float qmin, float delta,
                                                 float sum_u, float qc, float qn, int metric) {
  const float A = __fsub_rn(__fmul_rn(2.f, m.z), P);
  const float B = __fsub_rn(__fmul_rn(2.f, (float)s_bu), sum_u);
  const float t = __fmaf_rn(delta, B, __fmul_rn(qmin, A));
  const float est = __fsub_rn(__fadd_rn(qc, m.x), __fmul_rn(2.f, __fmul_rn(m.y, t)));
  if (metric == METRIC_INNER_PRODUCT) return __fmul_rn(-0.5f, __fsub_rn(__fadd_rn(qn, m.w), est));
  if (metric == METRIC_COSINE) return __fmul_rn(0.5f, est);
  return est;
}

// s_bu of a row of MW 16-byte words of bits held in registers
template <int MW>
__device__ __forceinline__ uint32_t rabitq_sbu(const uint32_t* planes, const uint4 (&b)[MW]) {
  uint32_t acc = 0;
#pragma unroll
  for (int j = 0; j < 4; ++j) {
    uint32_t c = 0;
#pragma unroll
    for (int w = 0; w < MW; ++w) {
      const uint4 p = *reinterpret_cast<const uint4*>(planes + j * 4 * MW + 4 * w);
      c += __popc(b[w].x & p.x) + __popc(b[w].y & p.y) + __popc(b[w].z & p.z) + __popc(b[w].w & p.w);
    }
    acc += c << j;
  }
  return acc;
}

// s_bu of a row read word by word (any W, any alignment)
__device__ __forceinline__ uint32_t rabitq_sbu_any(const uint32_t* planes, const uint32_t* __restrict__ row,
                                                   uint32_t W) {
  uint32_t c[4] = {0, 0, 0, 0};
  for (uint32_t w = 0; w < W; ++w) {
    const uint32_t b = __ldg(row + w);
#pragma unroll
    for (int j = 0; j < 4; ++j) c[j] += __popc(b & planes[j * W + w]);
  }
  return c[0] + (c[1] << 1) + (c[2] << 2) + (c[3] << 3);
}

// PQ: ADC of one row from its code bytes; LUT rows of 256 floats.
__device__ __forceinline__ float adc_row(const float* __restrict__ lut, const uint8_t* __restrict__ row, uint32_t m_pq,
                                         bool vec16) {
  float s = 0.f;
  if (vec16) {
    for (uint32_t m0 = 0; m0 < m_pq; m0 += 16) {
      const uint4 w = __ldg(reinterpret_cast<const uint4*>(row + m0));
      const uint32_t ws[4] = {w.x, w.y, w.z, w.w};
#pragma unroll
      for (int b = 0; b < 16; ++b) {
        const uint32_t c = (ws[b >> 2] >> ((b & 3) * 8)) & 0xFFu;
        s = __fadd_rn(s, lut[(m0 + b) * 256 + c]);
      }
    }
  } else {
    for (uint32_t m = 0; m < m_pq; ++m) s = __fadd_rn(s, lut[m * 256 + __ldg(row + m)]);
  }
  return s;
}

// PQ: ADC of a code row already in registers (MW 16-byte words, m_pq = 16 MW),
// sub-spaces added in order as adc_row does.
template <int MW>
__device__ __forceinline__ float adc_words(const float* __restrict__ lut, const uint4 (&w)[MW]) {
  float s = 0.f;
#pragma unroll
  for (int j = 0; j < MW; ++j) {
    const uint32_t ws[4] = {w[j].x, w[j].y, w[j].z, w[j].w};
#pragma unroll
    for (int b = 0; b < 16; ++b) {
      const uint32_t c = (ws[b >> 2] >> ((b & 3) * 8)) & 0xFFu;
      s = __fadd_rn(s, lut[(j * 16 + b) * 256 + c]);
    }
  }
  return s;
}

// SQ8: squared L2 between the query residual and the decoded row.
__device__ __forceinline__ float sq8_row(const float* __restrict__ qres, const float* __restrict__ mins,
                                         const float* __restrict__ scales, const uint8_t* __restrict__ row,
                                         uint32_t dim, bool vec16) {
  float s = 0.f;
  uint32_t d = 0;
  if (vec16) {
    for (; d + 16 <= dim; d += 16) {
      const uint4 w = __ldg(reinterpret_cast<const uint4*>(row + d));
      const uint32_t ws[4] = {w.x, w.y, w.z, w.w};
#pragma unroll
      for (int b = 0; b < 16; ++b) {
        const float c = (float)((ws[b >> 2] >> ((b & 3) * 8)) & 0xFFu);
        const float rec = fmaf(c, scales[d + b], mins[d + b]);
        const float t = qres[d + b] - rec;
        s = fmaf(t, t, s);
      }
    }
  }
  for (; d < dim; ++d) {
    const float rec = fmaf((float)__ldg(row + d), scales[d], mins[d]);
    const float t = qres[d] - rec;
    s = fmaf(t, t, s);
  }
  return s;
}

// MODE: PQ, SQ8 or RaBitQ. MW > 0: code rows of 16 * MW bytes at 16-byte-
// aligned rows (PQ m_pq = 16, 32, 64; RaBitQ P = 128 MW with 16-byte-aligned
// meta rows), scanned by the register-prefetching loop with R postings per
// thread per round, software-pipelined across rounds (PIPE).
// Resident CTAs per SM each variant is compiled for (its register budget:
// 4 -> 64, 3 -> 85, 2 -> 128 registers per thread): the list scans are
// load-latency bound, so occupancy is worth more than registers.
template <int MODE, int MW, bool PIPE>
constexpr int ivf_min_blocks() {
  return (MODE == IVF_PQ && (MW == 4 || (PIPE && MW == 2))) ? 2 : (PIPE || (MODE == IVF_RABITQ && MW >= 4)) ? 3 : 4;
}

template <int MODE, int MW, int R = 4, bool PIPE = false>
__global__ void __launch_bounds__(IVF_THREADS, ivf_min_blocks<MODE, MW, PIPE>()) ivf_scan_kernel(IvfArgs a) {
  // a round offers at most IVF_THREADS * R candidates, appended after the
  // shortlist; the buffer is flushed between rounds, so one round must fit
  static_assert((uint32_t)IVF_THREADS * R <= IVF_BUF, "a round of postings must fit the candidate buffer");
  extern __shared__ __align__(16) uint8_t smem[];
  uint64_t* keys = reinterpret_cast<uint64_t*>(smem);
  float* tab = reinterpret_cast<float*>(smem + (size_t)a.keys_pow2 * 8);
  float* qs = tab + IvfSmem::table_floats(MODE, a.dim, a.m_pq, a.P);
  __shared__ uint32_t s_q, s_cnt;
  __shared__ uint64_t s_tau;

  const int tid = threadIdx.x;
  const bool vec16 = (a.code_bytes % 16u) == 0 && ((uintptr_t)a.codes % 16u) == 0;
  float* mins = tab + a.dim;      // SQ8 only
  float* scales = tab + 2 * a.dim;
  float* qres = qs + a.dim;       // PQ only: q - centroid of the probed list
  float* rq = tab;                // RaBitQ only: rotated query, rotated residual, bit-planes
  float* rdiff = tab + a.P;
  uint32_t* planes = reinterpret_cast<uint32_t*>(tab + 2 * a.P);
  __shared__ float s_par[4];      // RaBitQ: min, delta, 15 / range, sum u of the list's query code
  __shared__ float s_red[IVF_THREADS];
  const bool cb4 = a.sub_dim == 4 && ((uintptr_t)a.codebooks % 16u) == 0;

  if (MODE == IVF_SQ8) {
    for (uint32_t d = tid; d < a.dim; d += IVF_THREADS) {
      mins[d] = __ldg(a.sq_mins + d);
      scales[d] = __ldg(a.sq_scales + d);
    }
  }

  __shared__ unsigned long long s_total;
  const uint32_t G = a.items_per_q;
  while (true) {
    __syncthreads();
    if (tid == 0) s_q = atomicAdd(a.work, 1u);
    __syncthreads();
    const uint32_t item = s_q;
    if (item >= a.nq * G) break;
    const uint32_t q = item / G, g = item % G;
    uint32_t kq = a.q_topk ? __ldg(a.q_topk + q) : a.top_k;
    uint32_t npq = a.q_nprobe ? __ldg(a.q_nprobe + q) : a.nprobe;
    const uint32_t rrq = a.q_rerank ? __ldg(a.q_rerank + q) : a.rerank_k;
    const uint32_t S = ivf_clamps(kq, npq, rrq, a.nlist);
    npq = min(npq, a.nprobe);
    kq = min(kq, a.top_k);
    const bool do_rerank = rrq != 1u && a.vectors != nullptr;
    const QueryFilter qf = load_filter(a.filters, q);

    const float* qv = a.queries + (size_t)q * a.dim;
    for (uint32_t d = tid; d < a.dim; d += IVF_THREADS) qs[d] = __ldg(qv + d);
    for (uint32_t i = tid; i < S; i += IVF_THREADS) keys[i] = kSentinelKey;
    if (tid == 0) {
      s_cnt = 0;
      s_tau = kSentinelKey;
      unsigned long long total = 0;
      if (G > 1)
        for (uint32_t p = 0; p < npq; ++p) {
          const uint32_t l = a.probes[(size_t)q * a.nprobe + p].id;
          if (l < a.nlist) {
            const ListSpan sp = list_span(a, l);
            total += sp.end - sp.beg;
          }
        }
      s_total = total;
    }
    __syncthreads();
    float qn = 0.f;  // RaBitQ, inner product: ||q||^2
    if (MODE == IVF_RABITQ) {
      if (a.metric == METRIC_INNER_PRODUCT) {
        // in the order of the reference's 256-thread block
        // (ivf_quant_lookup.cu:686-697): strided fmaf partials, pairwise fold
        float part = 0.f;
        for (uint32_t d = tid; d < a.dim; d += IVF_THREADS) part = __fmaf_rn(qs[d], qs[d], part);
        s_red[tid] = part;
        __syncthreads();
        for (int st = IVF_THREADS / 2; st > 0; st >>= 1) {
          if (tid < st) s_red[tid] = __fadd_rn(s_red[tid], s_red[tid + st]);
          __syncthreads();
        }
        qn = s_red[0];
      }
      rabitq_rotate_query(rq, qs, a);
    }
    // this item's range of the query's probed postings (lists in probe order)
    const uint64_t lo = G > 1 ? s_total * g / G : 0ull;
    const uint64_t hi = G > 1 ? s_total * (g + 1) / G : ~0ull;
    uint64_t cum = 0;

    auto flush = [&]() {
      // keys[0, S) sorted shortlist, keys[S, S + cnt) new candidates
      const uint32_t cnt = s_cnt;  // block-uniform (read after a barrier)
      if (cnt == 0) return;
      const uint32_t p2 = next_pow2_dev(S + cnt);  // sort only the occupied prefix
      for (uint32_t i = S + cnt + tid; i < p2; i += IVF_THREADS) keys[i] = kSentinelKey;
      __syncthreads();
      block_bitonic_sort(keys, p2);
      if (tid == 0) {
        s_cnt = 0;
        s_tau = keys[S - 1];
      }
      __syncthreads();
    };

    for (uint32_t p = 0; p < npq; ++p) {
      const uint32_t l = a.probes[(size_t)q * a.nprobe + p].id;
      if (l >= a.nlist) continue;  // uniform over the block
      const ListSpan sp = list_span(a, l);
      const uint32_t lbeg = sp.beg, llen = sp.end - sp.beg;
      const bool compact = sp.compact;  // uniform over the block
      const uint64_t s0 = max(lo, cum), s1 = min(hi, cum + llen);
      const uint64_t at = cum;
      cum += llen;
      if (s0 >= s1) continue;  // uniform: the list lies outside this item's range
      const float* cent = a.centroids + (size_t)l * a.dim;
      if (MODE == IVF_PQ) {
        // LUT[m][c] = sum_sd ((q - centroid) - codeword)^2 with fmaf in
        // sub-dimension order; q - centroid is rounded once per dimension, as
        // the reference's expression rounds it (ivf_pq_lookup.cu:150-162)
        for (uint32_t d = tid; d < a.dim; d += IVF_THREADS) qres[d] = qs[d] - __ldg(cent + d);
        __syncthreads();
        const uint32_t entries = a.m_pq * 256;
        if (cb4) {
          const float4* cbv = reinterpret_cast<const float4*>(a.codebooks);
          auto entry = [&](uint32_t e, float4 w) {  // codeword (m, c) = row e of 4 floats
            const float* r = qres + (e >> 8) * 4;
            const float t0 = r[0] - w.x, t1 = r[1] - w.y, t2 = r[2] - w.z, t3 = r[3] - w.w;
            tab[e] = fmaf(t3, t3, fmaf(t2, t2, fmaf(t1, t1, fmaf(t0, t0, 0.f))));
          };
          // B codeword loads in flight per thread before any is used (the
          // codebooks, 16 KB per sub-space, stream from L2 for every list)
          constexpr uint32_t B = MW >= 2 ? 8 : 4;  // fewer where the register budget is small
          uint32_t e0 = tid;
          for (; e0 + (B - 1) * IVF_THREADS < entries; e0 += B * IVF_THREADS) {
            float4 w[B];
#pragma unroll
            for (uint32_t b = 0; b < B; ++b) w[b] = __ldg(cbv + e0 + b * IVF_THREADS);
#pragma unroll
            for (uint32_t b = 0; b < B; ++b) entry(e0 + b * IVF_THREADS, w[b]);
          }
          for (uint32_t e = e0; e < entries; e += IVF_THREADS) entry(e, __ldg(cbv + e));
        } else {
          for (uint32_t e = tid; e < entries; e += IVF_THREADS) {
            const uint32_t m = e >> 8, c = e & 255u;
            const float* cb = a.codebooks + ((size_t)m * 256 + c) * a.sub_dim;
            float s = 0.f;
            for (uint32_t sd = 0; sd < a.sub_dim; ++sd) {
              const float t = qres[m * a.sub_dim + sd] - __ldg(cb + sd);
              s = fmaf(t, t, s);
            }
            tab[e] = s;
          }
        }
      } else if (MODE == IVF_SQ8) {
        for (uint32_t d = tid; d < a.dim; d += IVF_THREADS) tab[d] = qs[d] - __ldg(cent + d);
      } else {
        rabitq_query_code(rq, rdiff, planes, a, l, s_par);
      }
      __syncthreads();
      // RaBitQ: the list's query code and the query-to-centroid distance
      const float qc = MODE == IVF_RABITQ ? a.probes[(size_t)q * a.nprobe + p].distance : 0.f;
      const float qmin = s_par[0], qdelta = s_par[1], sum_u = s_par[3], Pf = (float)a.P;

      const uint32_t beg = lbeg + (uint32_t)(s0 - at), end = lbeg + (uint32_t)(s1 - at);
      auto offer = [&](float d, uint32_t vid) {
        if (d < kSentinelDist) {
          const uint64_t key = make_key(d, vid);
          if (key < s_tau) {
            const uint32_t pos = atomicAdd(&s_cnt, 1u);
            keys[S + pos] = key;
          }
        }
      };
      if (MODE != IVF_SQ8 && MW > 0) {
        // R postings per thread per round: the ids of all of them, then their
        // mask / filter words, then the code rows of the admitted ones only
        // (a 10% mask leaves 9 of 10 rows unread), all before any is scored.
        // PIPE: the next round's loads are issued before this round is
        // scored, so global-load latency overlaps the LUT arithmetic.
        constexpr int MWW = MW > 0 ? MW : 1;
        constexpr uint32_t step = IVF_THREADS * R;
        auto issue = [&](uint32_t b0, uint32_t (&v)[R], uint4 (&c)[R][MWW], float4 (&mt)[R], bool (&o)[R]) {
          // in: the posting exists and, where the list-order bits cover it,
          // the mask admits it -- known from the bit word alone, so the code
          // rows (list-major: addressed by position) load alongside the ids
          bool bits[R], in[R];
          uint32_t pos[R];
#pragma unroll
          for (int r = 0; r < R; ++r) {
            const uint32_t i = b0 + r * IVF_THREADS + tid;
            if (compact) {  // i indexes the admitted positions: all pass the mask
              bits[r] = true;
              in[r] = i < end;
              pos[r] = in[r] ? __ldg(a.adm_pos + i) : 0u;
            } else {
              bits[r] = a.list_allow != nullptr && i < a.list_n;
              in[r] = i < end && (!bits[r] || ((__ldg(a.list_allow + (i >> 5)) >> (i & 31u)) & 1u));
              pos[r] = i;
            }
            v[r] = in[r] ? __ldg(a.vec_ids + pos[r]) : 0xFFFFFFFFu;
          }
#pragma unroll
          for (int r = 0; r < R; ++r) {
            const size_t row_i = a.list_major ? pos[r] : v[r];
            const uint4* row = reinterpret_cast<const uint4*>(a.codes + row_i * (16u * MW));
#pragma unroll
            for (int j = 0; j < MWW; ++j) c[r][j] = in[r] ? __ldg(row + j) : make_uint4(0u, 0u, 0u, 0u);
            if (MODE == IVF_RABITQ)
              mt[r] = in[r] ? __ldg(reinterpret_cast<const float4*>(a.rq_meta) + row_i) : make_float4(0.f, 0.f, 0.f, 0.f);
          }
          // scored: also the id-based mask (positions the bits do not cover)
          // and the query's filter
#pragma unroll
          for (int r = 0; r < R; ++r)
            o[r] = in[r] && (bits[r] || mask_allows(a.mask, v[r])) && filter_allows(qf, v[r]);
        };
        auto score = [&](const uint4 (&c)[MWW], const float4& mt) -> float {
          if (MODE == IVF_RABITQ)
            return rabitq_estimate(rabitq_sbu<MWW>(planes, c), mt, Pf, qmin, qdelta, sum_u, qc, qn, a.metric);
          return adc_words<MWW>(tab, c);
        };
        uint32_t vid[R];
        uint4 w[R][MWW];
        float4 mt[R];
        bool ok[R];
        if (PIPE && beg < end) issue(beg, vid, w, mt, ok);
        for (uint32_t base = beg; base < end; base += step) {
          if (PIPE) {
            uint32_t vn[R];
            uint4 wn[R][MWW];
            float4 mn[R];
            bool okn[R];
            const bool more = base + step < end;  // uniform over the block
            if (more) issue(base + step, vn, wn, mn, okn);
#pragma unroll
            for (int r = 0; r < R; ++r)
              if (ok[r]) offer(score(w[r], mt[r]), vid[r]);
            if (more) {
#pragma unroll
              for (int r = 0; r < R; ++r) {
                vid[r] = vn[r];
                ok[r] = okn[r];
                mt[r] = mn[r];
#pragma unroll
                for (int j = 0; j < MWW; ++j) w[r][j] = wn[r][j];
              }
            }
          } else {
            issue(base, vid, w, mt, ok);
#pragma unroll
            for (int r = 0; r < R; ++r)
              if (ok[r]) offer(score(w[r], mt[r]), vid[r]);
          }
          __syncthreads();
          if (s_cnt > IVF_BUF - step) flush();
        }
      } else {
        for (uint32_t base = beg; base < end; base += IVF_THREADS) {
          const uint32_t j = base + tid;
          const bool bits = compact || (a.list_allow != nullptr && j < a.list_n);
          const uint32_t i = compact ? (j < end ? __ldg(a.adm_pos + j) : 0u) : j;
          if (j < end && (compact || !bits || ((__ldg(a.list_allow + (i >> 5)) >> (i & 31u)) & 1u))) {
            const uint32_t vid = __ldg(a.vec_ids + i);
            if ((bits || mask_allows(a.mask, vid)) && filter_allows(qf, vid)) {
              const size_t row_i = a.list_major ? i : vid;
              const uint8_t* row = a.codes + row_i * a.code_bytes;
              if (MODE == IVF_RABITQ) {
                const float* mp = a.rq_meta + row_i * 4;
                const float4 mt = make_float4(__ldg(mp), __ldg(mp + 1), __ldg(mp + 2), __ldg(mp + 3));
                const uint32_t sbu = rabitq_sbu_any(planes, reinterpret_cast<const uint32_t*>(row), a.W);
                offer(rabitq_estimate(sbu, mt, Pf, qmin, qdelta, sum_u, qc, qn, a.metric), vid);
              } else {
                offer(MODE == IVF_PQ ? adc_row(tab, row, a.m_pq, vec16)
                                     : sq8_row(tab, mins, scales, row, a.dim, vec16),
                      vid);
              }
            }
          }
          __syncthreads();
          if (s_cnt > IVF_BUF - IVF_THREADS) flush();
        }
      }
      __syncthreads();  // the table is rebuilt for the next list
    }
    flush();
    if (G > 1) {
      // a range's shortlist goes to the merge kernel
      uint64_t* dst = a.partial + (size_t)item * a.part_stride;
      for (uint32_t i = tid; i < S; i += IVF_THREADS) dst[i] = keys[i];
      continue;
    }
    ivf_finish_query(a, keys, q, S, kq, do_rerank, qv);
  }
}

// G > 1: one CTA per query merges the G range shortlists (top S of their
// union, by key), reranks and writes the top k -- the same answer as one
// range holding every posting.
__global__ void __launch_bounds__(IVF_THREADS) ivf_merge_kernel(IvfArgs a) {
  extern __shared__ __align__(16) uint8_t smem[];
  uint64_t* keys = reinterpret_cast<uint64_t*>(smem);
  const uint32_t q = blockIdx.x, G = a.items_per_q;
  uint32_t kq = a.q_topk ? __ldg(a.q_topk + q) : a.top_k;
  uint32_t npq = a.q_nprobe ? __ldg(a.q_nprobe + q) : a.nprobe;
  const uint32_t rrq = a.q_rerank ? __ldg(a.q_rerank + q) : a.rerank_k;
  const uint32_t S = ivf_clamps(kq, npq, rrq, a.nlist);
  kq = min(kq, a.top_k);
  const bool do_rerank = rrq != 1u && a.vectors != nullptr;
  const uint32_t total = G * S, p2 = next_pow2_dev(total);
  for (uint32_t i = threadIdx.x; i < p2; i += IVF_THREADS) {
    uint64_t v = kSentinelKey;
    if (i < total) v = a.partial[((size_t)q * G + i / S) * a.part_stride + i % S];
    keys[i] = v;
  }
  __syncthreads();
  block_bitonic_sort(keys, p2);
  ivf_finish_query(a, keys, q, S, kq, do_rerank, a.queries + (size_t)q * a.dim);
}

// The mask in list order (one word per 32 list positions), for one call.
// Only positions inside the lists (< offsets[nlist]) read an id: vec_ids may
// be shorter than the id space n (an engine whose slots carry remapped ids).
__global__ void __launch_bounds__(256) ivf_list_mask_kernel(const uint32_t* __restrict__ vec_ids,
                                                            const uint32_t* __restrict__ offsets, uint32_t nlist,
                                                            uint32_t n, const uint32_t* __restrict__ mask,
                                                            uint32_t* __restrict__ out) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  const uint32_t postings = min(n, __ldg(offsets + nlist));
  const bool b = i < postings && mask_allows(mask, __ldg(vec_ids + i));
  const uint32_t w = __ballot_sync(0xffffffffu, b);
  if ((threadIdx.x & 31u) == 0 && i < n) out[i >> 5] = w;
}

// Compaction of the list-order mask (three launches): per 1,024-word block
// the count of admitted positions; an exclusive scan of those counts; per
// word the exclusive prefix count and the admitted positions themselves,
// in list order.
constexpr uint32_t ADM_BLOCK = 1024;

__device__ __forceinline__ uint32_t warp_incl_scan(uint32_t x, int lane) {
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  return x;
}

// exclusive prefix of v over the block (ADM_BLOCK threads), plus the block total
__device__ __forceinline__ uint32_t block_excl_scan(uint32_t v, uint32_t* total) {
  __shared__ uint32_t s_warp[ADM_BLOCK / 32];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const uint32_t x = warp_incl_scan(v, lane);
  if (lane == 31) s_warp[warp] = x;
  __syncthreads();
  if (warp == 0) s_warp[lane] = warp_incl_scan(s_warp[lane], lane);
  __syncthreads();
  const uint32_t excl = (warp ? s_warp[warp - 1] : 0u) + x - v;
  *total = s_warp[ADM_BLOCK / 32 - 1];
  __syncthreads();
  return excl;
}

__global__ void __launch_bounds__(ADM_BLOCK) adm_count_kernel(const uint32_t* __restrict__ words, uint32_t nwords,
                                                              uint32_t* __restrict__ block_sums) {
  const uint32_t w = blockIdx.x * ADM_BLOCK + threadIdx.x;
  uint32_t total;
  block_excl_scan(w < nwords ? __popc(__ldg(words + w)) : 0u, &total);
  if (threadIdx.x == 0) block_sums[blockIdx.x] = total;
}

// in place, one block, ADM_BLOCK entries at a time with a running carry
__global__ void __launch_bounds__(ADM_BLOCK) adm_scan_kernel(uint32_t* __restrict__ sums, uint32_t n) {
  uint32_t carry = 0;
  for (uint32_t base = 0; base < n; base += ADM_BLOCK) {
    const uint32_t i = base + threadIdx.x;
    uint32_t total;
    const uint32_t excl = block_excl_scan(i < n ? sums[i] : 0u, &total);
    if (i < n) sums[i] = carry + excl;
    carry += total;
  }
}

__global__ void __launch_bounds__(ADM_BLOCK) adm_compact_kernel(const uint32_t* __restrict__ words, uint32_t nwords,
                                                                const uint32_t* __restrict__ block_off,
                                                                uint32_t* __restrict__ prefix,
                                                                uint32_t* __restrict__ pos) {
  const uint32_t w = blockIdx.x * ADM_BLOCK + threadIdx.x;
  uint32_t bits = w < nwords ? __ldg(words + w) : 0u, total;
  const uint32_t o = __ldg(block_off + blockIdx.x) + block_excl_scan(__popc(bits), &total);
  if (w < nwords) {
    prefix[w] = o;
    if (w == nwords - 1) prefix[nwords] = o + __popc(bits);
    for (uint32_t k = o; bits; ++k) {
      const uint32_t b = __ffs(bits) - 1;
      bits &= bits - 1;
      pos[k] = w * 32 + b;
    }
  }
}

// ---------------------------------------------------------------------------
// Tensor-core coarse probe (large nlist). The exact coarse probe is a Q x
// nlist fp32 scan; here an fp16 tensor-core scan of the centred queries
// (q - mu) against the centred centroids (c - mu; L2 distances do not move
// under the shift, the fp16 rounding error shrinks with the magnitudes)
// returns each query's K best lists by that approximate distance, their
// exact distances are recomputed with the exact probe's arithmetic (fmaf of
// q - c in dimension order), and the first nprobe by (distance, list) are
// kept. That is the exact probe list whenever no list outside the K can
// reach the nprobe-th place: every list outside has approximate distance
// >= t16 (the K-th approximate distance), an approximate distance is within
// `err` of the exact one (a bound from the fp16 unit roundoff, the fp32
// accumulation and the norms), so d_nprobe < (t16 - err) (1 - dim 2^-22)
// proves it. A query that fails the test, or whose candidate heaps may have
// dropped a key, is recomputed by the exact scan (coarse_exact_kernel).
constexpr int CO_THREADS = 256;
constexpr uint32_t CO_CHUNK = 2048;  // centroids per step of the exact fallback

// mu: the mean of up to 1,024 evenly spaced centroids (any shift is exact
// for L2; the mean keeps the fp16 values small)
__global__ void __launch_bounds__(CO_THREADS) coarse_mu_kernel(const float* __restrict__ cent, uint32_t nlist,
                                                               uint32_t dim, float* __restrict__ mu) {
  const uint32_t d = blockIdx.x * CO_THREADS + threadIdx.x;
  if (d >= dim) return;
  const uint32_t s = min(nlist, 1024u);
  float acc = 0.f;
  for (uint32_t i = 0; i < s; ++i) acc += __ldg(cent + (size_t)((uint64_t)i * nlist / s) * dim + d);
  mu[d] = acc / (float)s;
}

// One block per row: rows [0, nlist) are centroids -> fp16 (c - mu) padded to
// pd, ||c - mu||^2, and the largest ||c - mu|| (float bits, atomicMax);
// rows [nlist, nlist + nq) are queries -> q - mu in fp32.
__global__ void __launch_bounds__(128) coarse_prep_kernel(const float* __restrict__ cent, uint32_t nlist,
                                                          const float* __restrict__ queries, uint32_t nq,
                                                          uint32_t dim, uint32_t pd, const float* __restrict__ mu,
                                                          __half* __restrict__ c16, float* __restrict__ cnorm,
                                                          uint32_t* __restrict__ cmax, float* __restrict__ qc) {
  const uint32_t r = blockIdx.x;
  if (r >= nlist) {
    const uint32_t q = r - nlist;
    for (uint32_t d = threadIdx.x; d < dim; d += 128)
      qc[(size_t)q * dim + d] = __fsub_rn(__ldg(queries + (size_t)q * dim + d), mu[d]);
    return;
  }
  __shared__ float s_red[4];
  float part = 0.f;
  for (uint32_t d = threadIdx.x; d < pd; d += 128) {
    const float v = d < dim ? __fsub_rn(__ldg(cent + (size_t)r * dim + d), mu[d]) : 0.f;
    c16[(size_t)r * pd + d] = __float2half_rn(v);
    part = fmaf(v, v, part);
  }
#pragma unroll
  for (int o = 16; o; o >>= 1) part += __shfl_xor_sync(0xffffffffu, part, o);
  if ((threadIdx.x & 31) == 0) s_red[threadIdx.x >> 5] = part;
  __syncthreads();
  if (threadIdx.x == 0) {
    const float n2 = (s_red[0] + s_red[1]) + (s_red[2] + s_red[3]);
    cnorm[r] = n2;
    atomicMax(cmax, __float_as_uint(sqrtf(n2)));
  }
}

// exact coarse distance of query row qv (shared) to centroid c: the exact
// probe's arithmetic (flat_f32_scan_kernel, FUSED)
__device__ __forceinline__ float coarse_exact(const float* qv, const float* __restrict__ c, uint32_t dim) {
  float acc = 0.f;
  for (uint32_t d = 0; d < dim; ++d) {
    const float diff = __fsub_rn(qv[d], __ldg(c + d));
    acc = fmaf(diff, diff, acc);
  }
  return acc;
}

// Per query: exact distances of the K candidates, the first nprobe, and the
// exactness test. flags[q] = 1 sends the query to the exact fallback.
__global__ void __launch_bounds__(CO_THREADS) coarse_finish_kernel(const float* __restrict__ queries,
                                                                   const float* __restrict__ cent, uint32_t nlist,
                                                                   uint32_t dim, const GpuSearchResult* __restrict__ cand,
                                                                   uint32_t K, uint32_t nprobe,
                                                                   const float* __restrict__ qc,
                                                                   const uint32_t* __restrict__ cmax,
                                                                   uint32_t force_exact, uint32_t* __restrict__ flags,
                                                                   GpuSearchResult* __restrict__ probes) {
  extern __shared__ __align__(16) uint8_t co_smem[];
  uint64_t* keys = reinterpret_cast<uint64_t*>(co_smem);          // [256]
  float* qv = reinterpret_cast<float*>(co_smem + 256 * 8);        // [dim]
  __shared__ float s_red[CO_THREADS / 32];
  const uint32_t q = blockIdx.x;
  const int tid = threadIdx.x;
  float part = 0.f;
  for (uint32_t d = tid; d < dim; d += CO_THREADS) {
    qv[d] = __ldg(queries + (size_t)q * dim + d);
    const float c = __ldg(qc + (size_t)q * dim + d);
    part = fmaf(c, c, part);
  }
#pragma unroll
  for (int o = 16; o; o >>= 1) part += __shfl_xor_sync(0xffffffffu, part, o);
  if ((tid & 31) == 0) s_red[tid >> 5] = part;
  __syncthreads();
  const GpuSearchResult* cq = cand + (size_t)q * K;
  if (tid < (int)K) {
    const uint32_t id = cq[tid].id;
    keys[tid] = id < nlist ? make_key(coarse_exact(qv, cent + (size_t)id * dim, dim), id) : kSentinelKey;
  } else if (tid < 256) {
    keys[tid] = kSentinelKey;
  }
  __syncthreads();
  block_bitonic_sort(keys, 256);
  for (uint32_t j = tid; j < nprobe; j += CO_THREADS) probes[(size_t)q * nprobe + j] = key_to_result(keys[j], nullptr);
  if (tid == 0 && K < nlist) {
    float qn2 = 0.f;
    for (int w = 0; w < CO_THREADS / 32; ++w) qn2 += s_red[w];
    const float qn = sqrtf(qn2), cm = __uint_as_float(*cmax);
    const GpuSearchResult last = cq[K - 1];
    const float dnp = key_dist(keys[nprobe - 1]);
    bool ok = last.id < nlist && keys[nprobe - 1] != kSentinelKey && qn < 3.0e4f && cm < 3.0e4f;
    if (ok) {
      const float t16 = last.distance;
      const float fd = (float)dim;
      // |q.c - fp16(q).fp16(c)| <= (2.01 u16 + dim 2^-23) |q| |c| + dim 2^-25 (|q| + |c|)
      const float e_dot = (2.01f * 4.8828125e-4f + fd * 1.1920929e-7f) * qn * cm + fd * 2.9802322e-8f * (qn + cm);
      const float e_norm = fd * 1.1920929e-7f * (qn2 + cm * cm);
      const float e_add = 4.7683716e-7f * (qn2 + cm * cm + 2.f * qn * cm);
      const float err = 2.f * e_dot + e_norm + e_add;
      ok = dnp < (t16 - err) * (1.f - fd * 2.3841858e-7f);
    }
    if (!ok || force_exact) flags[q] = 1u;
  }
}

// The exact probe of a flagged query (the others return at once): every
// centroid's exact distance, the running best nprobe kept by sorting it
// with each chunk of CO_CHUNK new keys.
__global__ void __launch_bounds__(CO_THREADS) coarse_exact_kernel(const float* __restrict__ queries,
                                                                  const float* __restrict__ cent, uint32_t nlist,
                                                                  uint32_t dim, uint32_t nprobe,
                                                                  const uint32_t* __restrict__ flags,
                                                                  GpuSearchResult* __restrict__ probes) {
  const uint32_t q = blockIdx.x;
  if (flags[q] == 0u) return;
  extern __shared__ __align__(16) uint8_t co_smem[];
  constexpr uint32_t NK = 4096;                                    // pow2 >= 256 + CO_CHUNK
  uint64_t* keys = reinterpret_cast<uint64_t*>(co_smem);          // [NK]
  float* qv = reinterpret_cast<float*>(co_smem + NK * 8);         // [dim]
  const int tid = threadIdx.x;
  for (uint32_t d = tid; d < dim; d += CO_THREADS) qv[d] = __ldg(queries + (size_t)q * dim + d);
  for (uint32_t i = tid; i < 256; i += CO_THREADS) keys[i] = kSentinelKey;
  __syncthreads();
  for (uint32_t c0 = 0; c0 < nlist; c0 += CO_CHUNK) {
    for (uint32_t i = tid; i < NK - 256; i += CO_THREADS) {
      const uint32_t c = c0 + i;
      keys[256 + i] = (i < CO_CHUNK && c < nlist) ? make_key(coarse_exact(qv, cent + (size_t)c * dim, dim), c)
                                                  : kSentinelKey;
    }
    __syncthreads();
    block_bitonic_sort(keys, NK);
  }
  for (uint32_t j = tid; j < nprobe; j += CO_THREADS) probes[(size_t)q * nprobe + j] = key_to_result(keys[j], nullptr);
}

__global__ void relayout_codes_kernel(const uint8_t* __restrict__ by_id, const uint32_t* __restrict__ vec_ids,
                                      uint32_t n, uint32_t row_bytes, uint8_t* __restrict__ by_list) {
  const uint64_t total = (uint64_t)n * row_bytes;
  for (uint64_t e = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; e < total; e += (uint64_t)gridDim.x * blockDim.x) {
    const uint64_t pos = e / row_bytes, b = e % row_bytes;
    by_list[e] = by_id[(uint64_t)__ldg(vec_ids + pos) * row_bytes + b];
  }
}

size_t align256(size_t v) { return (v + 255) & ~(size_t)255; }

// Committed autotuner results for the IVF scans (tuning/gb300.json
// "ivf_entries", compiled in by build.py as tuning_ivf.inc): per shape range
// the list-scan pipelining, the posting-range split and the coarse probe
// that searched fastest (every choice gives the same answer). Knobs set
// with fv_tune_set take precedence; "tc.table" = 0 ignores the table.
struct IvfTuneEntry {
  int mode;
  uint32_t dim_lo, dim_hi;
  uint64_t n_lo, n_hi;
  uint32_t nlist_lo, nlist_hi, nq_lo, nq_hi, np_lo, np_hi;
  int pipeline, split, tc_coarse;
};
const IvfTuneEntry kIvfTuneTable[] = {
#include "tuning_ivf.inc"
    {-1, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, -1, -1, -1}};

const IvfTuneEntry* ivf_tune_lookup(int mode, uint32_t dim, uint64_t n, uint32_t nlist, uint32_t nq,
                                    uint32_t nprobe) {
  if (tune_value("tc.table", 1) == 0) return nullptr;
  for (const IvfTuneEntry& e : kIvfTuneTable) {
    if (e.mode < 0) break;
    if (e.mode == mode && dim >= e.dim_lo && dim <= e.dim_hi && n >= e.n_lo && n <= e.n_hi && nlist >= e.nlist_lo &&
        nlist <= e.nlist_hi && nq >= e.nq_lo && nq <= e.nq_hi && nprobe >= e.np_lo && nprobe <= e.np_hi)
      return &e;
  }
  return nullptr;
}

// A knob's value: the explicit setting, else the table entry's, else `dflt`
// (-1 in both means automatic).
int64_t ivf_knob(const char* key, int table_value, int64_t dflt) {
  const int64_t v = tune_value(key, -1);
  if (v >= 0) return v;
  if (table_value >= 0) return table_value;
  return dflt;
}

// Every size of one IVF search call, computed once: launch_ivf_search
// launches from it and the serving loop admits a batch by scratch_bytes.
// rc: 0 to launch, 1 when the call has nothing to do, else an error code.
struct IvfPlan {
  int rc = 0;
  uint32_t P = 0, top_k = 0, nprobe = 0, shortlist = 0, G = 1, sms = 0, list_n = 0, nwords = 0, adm_blocks = 0;
  // tensor-core coarse probe: candidates per query and the byte offsets of
  // its buffers in the coarse part of the scratch
  bool tcc = false, force_exact = false, pipeline = false;
  uint32_t K = 0;
  size_t co_mu = 0, co_c16 = 0, co_cnorm = 0, co_qc = 0, co_cand = 0, co_flags = 0, co_cmax = 0, co_tc = 0;
  FlatPlan cp;
  size_t coarse_bytes = 0, probe_bytes = 0, part_bytes = 0, allow_bytes = 0, scratch_bytes = 0;
};

IvfPlan plan_ivf_search(int mode, const IvfLaunch& L) {
  IvfPlan Q{};
  auto refuse = [&](int rc) {
    Q.rc = rc;
    return Q;
  };
  if (L.nq == 0 || L.top_k == 0 || L.nlist == 0 || L.dim == 0 || (mode == IVF_PQ && L.m_pq == 0)) return refuse(1);
  const uint32_t P = mode == IVF_RABITQ ? L.padded_dim : 0;
  if (mode == IVF_RABITQ && (P < 32 || P > 4096 || (P & (P - 1)) || P < L.dim)) return refuse(FV_ERR_ARG);
  // uniform batch: the clamps of the call; heterogeneous batch: top_k,
  // nprobe and rerank_k are the batch maxima and bound every query's values
  uint32_t top_k = L.top_k, nprobe = L.nprobe;
  uint32_t shortlist = ivf_clamps(top_k, nprobe, L.rerank_k, L.nlist);
  if (L.q_rerank) shortlist = std::min(std::max(std::max(L.rerank_k, top_k), shortlist), MAX_SHORTLIST);
  if (nprobe > (uint32_t)kMaxTopK) return refuse(FV_ERR_ARG);  // coarse selection keeps <= 256 lists
  if (mode == IVF_PQ && (L.sub_dim == 0 || L.m_pq * L.sub_dim > L.dim)) return refuse(FV_ERR_ARG);

  // Work items: with fewer queries than ~4 CTAs per SM, each query's probed
  // postings are cut into G equal ranges (a Zipf-giant list spreads over G
  // CTAs); each range keeps its own shortlist and ivf_merge_kernel joins
  // them. "ivf.split": -1 automatic, 0 / 1 never, G > 1 force G.
  const uint32_t sms = (uint32_t)device_sm_count();
  const IvfTuneEntry* te = ivf_tune_lookup(mode, L.dim, L.num_vectors, L.nlist, L.nq, nprobe);
  Q.pipeline = ivf_knob("ivf.pipeline", te ? te->pipeline : -1, 0) == 1;
  const int64_t split_knob = ivf_knob("ivf.split", te ? te->split : -1, -1);
  uint32_t G = 1;
  if (split_knob > 1)
    G = (uint32_t)split_knob;
  else if (split_knob < 0 && L.nq < 4 * sms)
    G = (4 * sms + L.nq - 1) / L.nq;
  G = std::max(1u, std::min<uint32_t>(std::min(G, 64u), 16384u / next_pow2(shortlist)));

  // coarse probe: exact fp32 scan, or the tensor-core candidates + exact
  // rescore ("ivf.tc_coarse": -1 automatic, 0 off, 1 on, 2 on with every
  // query sent to the exact fallback -- a check of the fallback)
  const int64_t tcc_knob = ivf_knob("ivf.tc_coarse", te ? te->tc_coarse : -1, -1);
  const uint32_t K = std::min<uint32_t>(std::min(256u, nprobe + 16), L.nlist);
  // (tables of at least one 256-row tile and one 64-element K block, so no
  // TMA box is larger than the tensor it reads)
  const bool tcc_fits = L.nlist >= 256 && L.dim >= 64;
  const bool tcc = tcc_fits && (tcc_knob > 0 || (tcc_knob < 0 && L.nlist >= 2048 && L.nq >= 256 &&
                                                  K == nprobe + 16 && K < L.nlist));
  const uint32_t pd16 = (L.dim + 15) / 16 * 16;
  TcTables ct{false, nullptr, nullptr, nullptr, nullptr, L.nlist, L.dim, pd16};
  const FvScanOptions copt{0, 0, 0.f, 0};
  size_t tc_bytes = 0;
  if (tcc) {
    Q.co_mu = 0;
    Q.co_c16 = align256(Q.co_mu + (size_t)L.dim * 4);
    Q.co_cnorm = (Q.co_c16 + (size_t)L.nlist * pd16 * 2 + 1023) / 1024 * 1024;
    Q.co_qc = align256(Q.co_cnorm + (size_t)L.nlist * 4);
    Q.co_cand = align256(Q.co_qc + (size_t)L.nq * L.dim * 4);
    Q.co_flags = align256(Q.co_cand + (size_t)L.nq * K * 8);
    Q.co_cmax = align256(Q.co_flags + (size_t)L.nq * 4);
    Q.co_tc = (Q.co_cmax + 256 + 1023) / 1024 * 1024;
    tc_bytes = Q.co_tc + tc_scan_scratch_bytes(ct, L.nq, K, METRIC_L2, copt);
  }
  Q.tcc = tcc;
  Q.K = K;
  Q.force_exact = tcc_knob == 2;

  // scratch: coarse heaps | probes | range shortlists | work counter
  const FlatPlan cp = plan_flat_f32(L.nlist, L.nq, nprobe, 0);
  const size_t coarse_bytes = tcc ? (tc_bytes + 1023) / 1024 * 1024 : align256(cp.scratch_bytes);
  const size_t probe_bytes = align256((size_t)L.nq * nprobe * sizeof(GpuSearchResult));
  const size_t part_bytes = G > 1 ? align256((size_t)L.nq * G * shortlist * 8) : 0;
  const uint32_t list_n = L.mask ? L.num_vectors : 0u;
  const size_t nwords = ((size_t)list_n + 31) / 32;
  const size_t allow_bytes = align256(nwords * 4);
  // compaction of the admitted positions ("ivf.compact" 0 turns it off)
  const bool compact = list_n > 0 && tune_value("ivf.compact", 1) != 0;
  const uint32_t adm_blocks = compact ? (uint32_t)((nwords + ADM_BLOCK - 1) / ADM_BLOCK) : 0u;
  const size_t adm_bytes = compact ? align256((size_t)adm_blocks * 4) + align256((nwords + 1) * 4) +
                                         align256((size_t)list_n * 4)
                                   : 0;
  Q.P = P;
  Q.top_k = top_k;
  Q.nprobe = nprobe;
  Q.shortlist = shortlist;
  Q.G = G;
  Q.sms = sms;
  Q.list_n = list_n;
  Q.cp = cp;
  Q.coarse_bytes = coarse_bytes;
  Q.probe_bytes = probe_bytes;
  Q.part_bytes = part_bytes;
  Q.allow_bytes = allow_bytes;
  Q.adm_blocks = adm_blocks;
  Q.nwords = (uint32_t)nwords;
  Q.scratch_bytes = coarse_bytes + probe_bytes + part_bytes + 256 + allow_bytes + adm_bytes;
  return Q;
}

}  // namespace

// The tensor-core coarse probe of one call into probes[nq][nprobe] (exact:
// see coarse_finish_kernel); its buffers are the coarse part of `scratch`.
static int launch_coarse_tc(const IvfPlan& Q, const IvfLaunch& L, uint8_t* scratch, GpuSearchResult* probes,
                     cudaStream_t stream) {
  ProfScope ps("coarse_tc", stream);
  float* mu = reinterpret_cast<float*>(scratch + Q.co_mu);
  __half* c16 = reinterpret_cast<__half*>(scratch + Q.co_c16);
  float* cnorm = reinterpret_cast<float*>(scratch + Q.co_cnorm);
  float* qc = reinterpret_cast<float*>(scratch + Q.co_qc);
  GpuSearchResult* cand = reinterpret_cast<GpuSearchResult*>(scratch + Q.co_cand);
  uint32_t* flags = reinterpret_cast<uint32_t*>(scratch + Q.co_flags);
  uint32_t* cmax = reinterpret_cast<uint32_t*>(scratch + Q.co_cmax);
  const uint32_t pd16 = (L.dim + 15) / 16 * 16;
  cudaError_t e = cudaMemsetAsync(flags, 0, (size_t)L.nq * 4, stream);
  if (e == cudaSuccess) e = cudaMemsetAsync(cmax, 0, 4, stream);
  if (e != cudaSuccess) return (int)e;
  coarse_mu_kernel<<<(L.dim + CO_THREADS - 1) / CO_THREADS, CO_THREADS, 0, stream>>>(L.centroids, L.nlist, L.dim, mu);
  coarse_prep_kernel<<<L.nlist + L.nq, 128, 0, stream>>>(L.centroids, L.nlist, L.queries, L.nq, L.dim, pd16, mu, c16,
                                                         cnorm, cmax, qc);
  note_launch(2);
  const TcTables ct{false, c16, cnorm, nullptr, nullptr, L.nlist, L.dim, pd16};
  const FvScanOptions copt{0, 0, 0.f, 0};
  int rc = launch_tc_scan_ext(ct, qc, L.nq, Q.K, METRIC_L2, nullptr, cand, copt, stream, nullptr, scratch + Q.co_tc,
                              flags);
  if (rc != 0) return rc;
  const size_t fsmem = 256 * 8 + (size_t)L.dim * 4;
  const size_t xsmem = 4096 * 8 + (size_t)L.dim * 4;
  e = cudaFuncSetAttribute(coarse_finish_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)fsmem);
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute(coarse_exact_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)xsmem);
  if (e != cudaSuccess) return (int)e;
  coarse_finish_kernel<<<L.nq, CO_THREADS, fsmem, stream>>>(L.queries, L.centroids, L.nlist, L.dim, cand, Q.K, Q.nprobe,
                                                           qc, cmax, Q.force_exact ? 1u : 0u, flags, probes);
  coarse_exact_kernel<<<L.nq, CO_THREADS, xsmem, stream>>>(L.queries, L.centroids, L.nlist, L.dim, Q.nprobe, flags,
                                                          probes);
  note_launch(2);
  return (int)cudaGetLastError();
}

int ivf_tune_query(int mode, uint32_t dim, uint64_t n, uint32_t nlist, uint32_t nq, uint32_t nprobe,
                   int32_t* out3) {
  const IvfTuneEntry* e = ivf_tune_lookup(mode, dim, n, nlist, nq, nprobe);
  if (!e) return FV_ERR_ARG;
  out3[0] = e->pipeline;
  out3[1] = e->split;
  out3[2] = e->tc_coarse;
  return 0;
}

size_t ivf_search_scratch_bytes(int mode, const IvfLaunch& L) {
  const IvfPlan Q = plan_ivf_search(mode, L);
  return Q.rc == 0 ? Q.scratch_bytes : 0;
}

int launch_ivf_search(int mode, const IvfLaunch& L, cudaStream_t stream) {
  const IvfPlan Q = plan_ivf_search(mode, L);
  if (Q.rc) return Q.rc == 1 ? 0 : Q.rc;
  const uint32_t P = Q.P, top_k = Q.top_k, nprobe = Q.nprobe, shortlist = Q.shortlist, G = Q.G, sms = Q.sms;
  const uint32_t list_n = Q.list_n;
  const FlatPlan& cp = Q.cp;
  const size_t coarse_bytes = Q.coarse_bytes, probe_bytes = Q.probe_bytes, part_bytes = Q.part_bytes;
  uint8_t* scratch = static_cast<uint8_t*>(scratch_get(stream, Q.scratch_bytes));
  if (!scratch) return (int)cudaErrorMemoryAllocation;
  uint32_t* list_allow =
      list_n ? reinterpret_cast<uint32_t*>(scratch + coarse_bytes + probe_bytes + part_bytes + 256) : nullptr;
  GpuSearchResult* probes = reinterpret_cast<GpuSearchResult*>(scratch + coarse_bytes);
  uint64_t* partial = G > 1 ? reinterpret_cast<uint64_t*>(scratch + coarse_bytes + probe_bytes) : nullptr;
  uint32_t* work = reinterpret_cast<uint32_t*>(scratch + coarse_bytes + probe_bytes + part_bytes);

  int rc = 0;
  if (Q.tcc) {
    rc = launch_coarse_tc(Q, L, scratch, probes, stream);
  } else {
    rc = launch_flat_f32_planned(cp, L.centroids, nullptr, L.nlist, L.dim, L.queries, L.nq, nprobe, METRIC_L2,
                                 nullptr, probes, true, cp.scratch_bytes ? scratch : nullptr, stream);
  }
  if (rc != 0) return rc;
  cudaError_t e = cudaMemsetAsync(work, 0, sizeof(uint32_t), stream);
  if (e != cudaSuccess) return (int)e;
  if (list_n) {
    ProfScope ps("ivf_list_mask", stream);
    ivf_list_mask_kernel<<<(list_n + 255) / 256, 256, 0, stream>>>(L.vec_ids, L.offsets, L.nlist, list_n, L.mask,
                                                                     list_allow);
    note_launch();
  }
  uint32_t *adm_prefix = nullptr, *adm_pos = nullptr;
  if (Q.adm_blocks) {
    uint32_t* adm_sums = list_allow + Q.allow_bytes / 4;
    adm_prefix = adm_sums + align256((size_t)Q.adm_blocks * 4) / 4;
    adm_pos = adm_prefix + align256(((size_t)Q.nwords + 1) * 4) / 4;
    ProfScope ps("ivf_mask_compact", stream);
    adm_count_kernel<<<Q.adm_blocks, ADM_BLOCK, 0, stream>>>(list_allow, Q.nwords, adm_sums);
    adm_scan_kernel<<<1, ADM_BLOCK, 0, stream>>>(adm_sums, Q.adm_blocks);
    adm_compact_kernel<<<Q.adm_blocks, ADM_BLOCK, 0, stream>>>(list_allow, Q.nwords, adm_sums, adm_prefix, adm_pos);
    note_launch(3);
  }

  IvfArgs a{};
  a.centroids = L.centroids;
  a.codebooks = L.codebooks;
  a.sq_mins = L.sq_mins;
  a.sq_scales = L.sq_scales;
  a.codes = L.codes;
  a.offsets = L.offsets;
  a.vec_ids = L.vec_ids;
  a.vectors = L.vectors;
  a.num_vectors = L.num_vectors;
  a.dim = L.dim;
  a.nlist = L.nlist;
  a.m_pq = L.m_pq;
  a.sub_dim = L.sub_dim;
  a.code_bytes = mode == IVF_PQ ? L.m_pq : mode == IVF_SQ8 ? L.dim : P / 8;
  if (mode == IVF_RABITQ) {
    a.codes = reinterpret_cast<const uint8_t*>(L.rq_bits);
    a.rot_centroids = L.rot_centroids;
    a.rq_meta = L.rq_meta;
    a.rot_signs = L.rot_signs;
    a.P = P;
    a.W = P / 32;
    a.inv_sqrt_p = rabitq_inv_sqrt(P);
  }
  a.queries = L.queries;
  a.nq = L.nq;
  a.top_k = top_k;
  a.nprobe = nprobe;
  a.rerank_k = L.rerank_k;
  a.list_major = L.list_major ? 1u : 0u;
  a.metric = (int)L.metric;
  a.mask = L.mask;
  a.list_allow = list_allow;
  a.list_n = list_n;
  a.adm_pos = adm_pos;
  a.adm_prefix = adm_prefix;
  a.q_topk = L.q_topk;
  a.q_nprobe = L.q_nprobe;
  a.q_rerank = L.q_rerank;
  a.filters = L.filters;
  a.probes = probes;
  a.work = work;
  a.out = L.out;
  a.status = status_word();
  a.keys_pow2 = next_pow2(shortlist + IVF_BUF);
  a.items_per_q = G;
  a.partial = partial;
  a.part_stride = shortlist;

  const size_t smem = IvfSmem::bytes(mode, a.keys_pow2, L.dim, L.m_pq, P);
  if (smem > 227 * 1024) return FV_ERR_ARG;
  const bool rows16 = mode == IVF_PQ && ((uintptr_t)L.codes % 16u) == 0;
  // "ivf.pipeline": 1 software-pipelines the PQ list scan (2 postings per
  // thread per round, next round's loads in flight while scoring). Off by
  // default: its 78 registers allow 3 CTAs per SM where the plain loop
  // (60 registers, 4 postings per round) runs 4, which measured 7% faster.
  const bool pipe = Q.pipeline;
  auto kern = ivf_scan_kernel<IVF_SQ8, 0>;
  if (mode == IVF_RABITQ) {
    // bits rows of P/8 bytes as 16-byte words when they and the meta rows
    // are 16-byte aligned; R postings per thread per round as registers allow
    const bool al = ((uintptr_t)L.rq_bits % 16u) == 0 && ((uintptr_t)L.rq_meta % 16u) == 0;
    kern = ivf_scan_kernel<IVF_RABITQ, 0>;
    if (al && P == 128) kern = ivf_scan_kernel<IVF_RABITQ, 1, 4>;
    if (al && P == 256) kern = ivf_scan_kernel<IVF_RABITQ, 2, 2>;
    if (al && P == 512) kern = ivf_scan_kernel<IVF_RABITQ, 4, 2>;
    if (al && P == 1024) kern = ivf_scan_kernel<IVF_RABITQ, 8, 1>;
  }
  if (mode == IVF_PQ) {
    kern = ivf_scan_kernel<IVF_PQ, 0>;
    if (rows16 && L.m_pq == 16) kern = pipe ? ivf_scan_kernel<IVF_PQ, 1, 2, true> : ivf_scan_kernel<IVF_PQ, 1>;
    if (rows16 && L.m_pq == 32) kern = pipe ? ivf_scan_kernel<IVF_PQ, 2, 2, true> : ivf_scan_kernel<IVF_PQ, 2>;
    if (rows16 && L.m_pq == 64) kern = pipe ? ivf_scan_kernel<IVF_PQ, 4, 2, true> : ivf_scan_kernel<IVF_PQ, 4>;
  }
  e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return (int)e;
  int per_sm = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, IVF_THREADS, smem);
  const uint32_t grid = std::max(1u, std::min<uint32_t>(L.nq * G, (uint32_t)(std::max(1, per_sm) * sms)));
  {
    ProfScope ps(mode == IVF_PQ ? "ivf_pq_scan" : mode == IVF_SQ8 ? "ivf_sq8_scan" : "ivf_rabitq_scan", stream);
    kern<<<grid, IVF_THREADS, smem, stream>>>(a);
    note_launch();
  }
  if (G > 1) {
    const size_t msmem = (size_t)next_pow2(G * shortlist) * 8;
    e = cudaFuncSetAttribute(ivf_merge_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)msmem);
    if (e != cudaSuccess) return (int)e;
    ProfScope ps("ivf_merge", stream);
    ivf_merge_kernel<<<L.nq, IVF_THREADS, msmem, stream>>>(a);
    note_launch();
  }
  return (int)cudaGetLastError();
}

int launch_relayout_codes(const uint8_t* by_id, const uint32_t* vec_ids, uint32_t n, uint32_t row_bytes,
                          uint8_t* by_list, cudaStream_t stream) {
  if (n == 0 || row_bytes == 0) return 0;
  const uint64_t total = (uint64_t)n * row_bytes;
  const uint32_t blocks = (uint32_t)std::min<uint64_t>((total + 255) / 256, 65535ull * 16);
  relayout_codes_kernel<<<blocks, 256, 0, stream>>>(by_id, vec_ids, n, row_bytes, by_list);
  note_launch();
  return (int)cudaGetLastError();
}

}  // namespace fv

extern "C" int fv_tune_lookup_ivf(int mode, uint32_t dim, uint64_t num_vectors, uint32_t nlist, uint32_t num_queries,
                                  uint32_t nprobe, int32_t* out_knobs) {
  if (!out_knobs) return FV_ERR_NULL;
  return fv::ivf_tune_query(mode, dim, num_vectors, nlist, num_queries, nprobe, out_knobs);
}
