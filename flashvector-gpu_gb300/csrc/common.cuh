// common.cuh -- device helpers shared by every kernel of libfvgb300.
//
// Ordering convention used by all top-k code here: a candidate is the
// 64-bit key (order(dist) << 32) | slot, where order() maps an IEEE float
// to an unsigned integer with the same ordering. Comparing keys therefore
// compares (distance, slot) lexicographically, which is the reference's
// tie rule for the exact scans (strict `<` while scanning slots in
// ascending order keeps the lower slot: sparse_hybrid.cu:42-72,
// ivf_quant_lookup.cu:1010-1019).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/fv_types.h"
#include "kernels.h"

namespace fv {

constexpr uint32_t kInvalidId = 0xFFFFFFFFu;
constexpr float kSentinelDist = 1e30f;  // unfilled result slot distance
constexpr int kMaxTopK = 256;           // reference clamp (streams.rs:14)

// Device status word: bounded waits and bounds checks set bits here
// instead of trapping, so the context stays usable and the host can read
// the cause with fv_read_device_status().
enum : uint32_t {
  kStatusMbarTimeout = 1u << 0,
  kStatusBounds = 1u << 1,
  kStatusOverflow = 1u << 2,
};
// The word lives in device memory owned by the bridge (status_word());
// kernels receive its address as an argument.
__device__ __forceinline__ void set_status(uint32_t* status, uint32_t bits) {
  if (status) atomicOr(status, bits);
}

// Order-preserving float -> uint32 map. -0.0 is folded onto +0.0 first so
// that the two zeros compare equal, as they do under float `<`.
__host__ __device__ __forceinline__ uint32_t float_order(float f) {
  f = f + 0.0f;
#ifdef __CUDA_ARCH__
  uint32_t u = __float_as_uint(f);
#else
  uint32_t u;
  __builtin_memcpy(&u, &f, 4);
#endif
  return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}

__host__ __device__ __forceinline__ float order_float(uint32_t o) {
  uint32_t u = (o & 0x80000000u) ? (o & 0x7FFFFFFFu) : ~o;
#ifdef __CUDA_ARCH__
  return __uint_as_float(u);
#else
  float f;
  __builtin_memcpy(&f, &u, 4);
  return f;
#endif
}

__host__ __device__ __forceinline__ uint64_t make_key(float dist, uint32_t slot) {
  return ((uint64_t)float_order(dist) << 32) | slot;
}
__host__ __device__ __forceinline__ float key_dist(uint64_t k) { return order_float((uint32_t)(k >> 32)); }
__host__ __device__ __forceinline__ uint32_t key_slot(uint64_t k) { return (uint32_t)k; }

// Key of an empty slot: larger than the key of every admissible candidate
// (admissible = distance < 1e30, which also rejects NaN).
constexpr uint64_t kSentinelKey = 0xFFFFFFFFFFFFFFFFull;

__host__ __device__ __forceinline__ uint32_t next_pow2_dev(uint32_t v) {
  if (v <= 1) return 1;
  --v;
  v |= v >> 1;
  v |= v >> 2;
  v |= v >> 4;
  v |= v >> 8;
  v |= v >> 16;
  return v + 1;
}

// Packed LSB-first validity bit of slot `i` (nullptr = everything valid).
// Same bit convention as the reference (distance_metrics.cuh:17-20,
// filter.rs:364-371).
__device__ __forceinline__ bool mask_allows(const uint32_t* __restrict__ mask, uint32_t i) {
  return mask == nullptr || ((__ldg(mask + (i >> 5)) >> (i & 31u)) & 1u);
}

// Query q's filter row (an empty filter when there are no per-query filters).
__device__ __forceinline__ QueryFilter load_filter(const QueryFilter* __restrict__ f, uint32_t q) {
  if (f == nullptr) return QueryFilter{nullptr, 0u, 0u};
  const uint4 v = __ldg(reinterpret_cast<const uint4*>(f + q));
  QueryFilter r;
  r.words = reinterpret_cast<const uint32_t*>(((uint64_t)v.y << 32) | v.x);
  r.nwords = v.z;
  r.reserved = 0;
  return r;
}

// Logical id `id` passes the query's filter.
__device__ __forceinline__ bool filter_allows(const QueryFilter& f, uint32_t id) {
  if (f.words == nullptr) return true;
  return (id >> 5) < f.nwords && ((__ldg(f.words + (id >> 5)) >> (id & 31u)) & 1u);
}

// The filter word covering ids [32 w, 32 w + 32) (all ones without a filter).
__device__ __forceinline__ uint32_t filter_word(const QueryFilter& f, uint32_t w) {
  if (f.words == nullptr) return 0xFFFFFFFFu;
  return w < f.nwords ? __ldg(f.words + w) : 0u;
}

__device__ __forceinline__ GpuSearchResult key_to_result(uint64_t key, const uint32_t* __restrict__ vec_ids) {
  GpuSearchResult r;
  if (key == kSentinelKey) {
    r.id = kInvalidId;
    r.distance = kSentinelDist;
  } else {
    uint32_t slot = key_slot(key);
    r.id = vec_ids ? __ldg(vec_ids + slot) : slot;
    r.distance = key_dist(key);
  }
  return r;
}

// ---------------------------------------------------------------------------
// The reference's warp-cooperative fp32 distance, restated: lane l sums the
// dimensions l, l+32, ... with fmaf; the 32 partials are reduced with the
// shuffle-down tree 16, 8, 4, 2, 1 and lane 0's value is returned to every
// lane (distance_metrics.cuh:53-138). Using the same order makes the rerank
// distances of the IVF paths bit-identical to the reference's.
// ---------------------------------------------------------------------------
__device__ __forceinline__ float warp_tree_sum(float v) {
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) v += __shfl_down_sync(0xffffffffu, v, off);
  return __shfl_sync(0xffffffffu, v, 0);
}

// R rows against one query at once: every row keeps its own per-lane fmaf
// chain in dimension order and its own shuffle tree, so each result is the
// one-row result bit for bit, while the R rows' loads are in flight together.
// The lane-strided elements of a row are loaded B steps ahead of the
// accumulation for the same reason.
template <int R, int B>
__device__ __forceinline__ void warp_metric_distances(const float* __restrict__ q, const float* const (&x)[R],
                                                      uint32_t dim, int lane, MetricType metric, float (&out)[R]) {
  float acc[R], nx[R], nq = 0.f;
#pragma unroll
  for (int r = 0; r < R; ++r) acc[r] = nx[r] = 0.f;
  for (uint32_t d0 = lane; d0 < dim; d0 += 32 * B) {
    float qa[B], xa[R][B];
#pragma unroll
    for (int b = 0; b < B; ++b) {
      const uint32_t d = d0 + 32 * b;
      qa[b] = d < dim ? q[d] : 0.f;
#pragma unroll
      for (int r = 0; r < R; ++r) xa[r][b] = d < dim ? __ldg(x[r] + d) : 0.f;
    }
#pragma unroll
    for (int b = 0; b < B; ++b) {
      if (d0 + 32 * b >= dim) continue;
      if (metric == METRIC_COSINE) nq = fmaf(qa[b], qa[b], nq);
#pragma unroll
      for (int r = 0; r < R; ++r) {
        if (metric == METRIC_INNER_PRODUCT) {
          acc[r] = fmaf(qa[b], xa[r][b], acc[r]);
        } else if (metric == METRIC_COSINE) {
          acc[r] = fmaf(qa[b], xa[r][b], acc[r]);
          nx[r] = fmaf(xa[r][b], xa[r][b], nx[r]);
        } else {
          const float diff = qa[b] - xa[r][b];
          acc[r] = fmaf(diff, diff, acc[r]);
        }
      }
    }
  }
  if (metric == METRIC_COSINE) nq = warp_tree_sum(nq);
#pragma unroll
  for (int r = 0; r < R; ++r) {
    const float a = warp_tree_sum(acc[r]);
    if (metric == METRIC_INNER_PRODUCT) {
      out[r] = -a;
    } else if (metric == METRIC_COSINE) {
      const float denom = __fadd_rn(__fmul_rn(sqrtf(nq), sqrtf(warp_tree_sum(nx[r]))), 1e-8f);
      out[r] = __fsub_rn(1.0f, __fdiv_rn(a, denom));
    } else {
      out[r] = a;
    }
  }
}

__device__ __forceinline__ float warp_metric_distance(const float* __restrict__ q, const float* __restrict__ x,
                                                      uint32_t dim, int lane, MetricType metric) {
  const float* const rows[1] = {x};
  float d[1];
  warp_metric_distances<1, 8>(q, rows, dim, lane, metric, d);
  return d[0];
}

}  // namespace fv
