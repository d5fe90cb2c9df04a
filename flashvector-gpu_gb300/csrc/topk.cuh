// topk.cuh -- selection / sorting building blocks on 64-bit (distance,
// slot) keys (see common.cuh for the key encoding).
#pragma once

#include "common.cuh"

namespace fv {

// Ascending bitonic sort of n (power of two) keys in shared memory by all
// threads of the block; returns after a block barrier. Each step walks the
// n / 2 compare-exchange pairs (i, i + stride), i with bit `stride` clear,
// so every thread does useful work in every step.
__device__ __forceinline__ void block_bitonic_sort(uint64_t* keys, uint32_t n) {
  for (uint32_t size = 2; size <= n; size <<= 1) {
    for (uint32_t stride = size >> 1; stride > 0; stride >>= 1) {
      for (uint32_t p = threadIdx.x; p < n / 2; p += blockDim.x) {
        const uint32_t i = 2 * p - (p & (stride - 1));  // (p / stride) * 2 stride + p % stride
        const uint32_t j = i + stride;
        const uint64_t a = keys[i], b = keys[j];
        if ((a > b) == ((i & size) == 0)) {
          keys[i] = b;
          keys[j] = a;
        }
      }
      __syncthreads();
    }
  }
  __syncthreads();
}

// Gathers the keys src[0, total) that are not the sentinel into keys[0, m)
// (in no particular order) and returns m; block-collective (warp ballots and
// one shared counter). `counter` is a shared word the caller owns.
__device__ __forceinline__ uint32_t block_compact_keys(const uint64_t* __restrict__ src, uint32_t total,
                                                       uint64_t* keys, uint32_t* counter) {
  const int lane = threadIdx.x & 31;
  if (threadIdx.x == 0) *counter = 0;
  __syncthreads();
  // eight loads in flight per thread before any of them is compacted
  constexpr int B = 8;
  for (uint32_t i0 = 0; i0 < total; i0 += blockDim.x * B) {
    uint64_t kb[B];
#pragma unroll
    for (int b = 0; b < B; ++b) {
      const uint32_t i = i0 + (uint32_t)b * blockDim.x + threadIdx.x;
      kb[b] = i < total ? src[i] : kSentinelKey;
    }
#pragma unroll
    for (int b = 0; b < B; ++b) {
      const bool keep = kb[b] != kSentinelKey;
      const uint32_t m = __ballot_sync(0xffffffffu, keep);
      uint32_t base = 0;
      if (lane == 0 && m) base = atomicAdd(counter, (uint32_t)__popc(m));
      base = __shfl_sync(0xffffffffu, base, 0);
      if (keep) keys[base + __popc(m & ((1u << lane) - 1u))] = kb[b];
    }
  }
  __syncthreads();
  return *counter;
}

// Ascending bitonic sort of 32 keys held one per lane.
__device__ __forceinline__ uint64_t warp_bitonic_sort32(uint64_t key) {
  const int lane = threadIdx.x & 31;
#pragma unroll
  for (int size = 2; size <= 32; size <<= 1) {
#pragma unroll
    for (int stride = size >> 1; stride > 0; stride >>= 1) {
      uint64_t other = __shfl_xor_sync(0xffffffffu, key, stride);
      bool up = (lane & size) == 0;
      bool lower = (lane & stride) == 0;
      // the lower lane of a pair keeps min when sorting up, max otherwise
      bool keep_min = (lower == up);
      key = keep_min ? (key < other ? key : other) : (key < other ? other : key);
    }
  }
  return key;
}

}  // namespace fv
