// topk.cuh -- selection / sorting building blocks on 64-bit (distance,
// slot) keys (see common.cuh for the key encoding).
#pragma once

#include "common.cuh"

namespace fv {

// Ascending bitonic sort of n (power of two) keys in shared memory by all
// threads of the block; returns after a block barrier.
__device__ __forceinline__ void block_bitonic_sort(uint64_t* keys, uint32_t n) {
  for (uint32_t size = 2; size <= n; size <<= 1) {
    for (uint32_t stride = size >> 1; stride > 0; stride >>= 1) {
      for (uint32_t i = threadIdx.x; i < n; i += blockDim.x) {
        uint32_t j = i ^ stride;
        if (j > i) {
          uint64_t a = keys[i], b = keys[j];
          bool up = (i & size) == 0;
          if ((a > b) == up) {
            keys[i] = b;
            keys[j] = a;
          }
        }
      }
      __syncthreads();
    }
  }
  __syncthreads();
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
