// fixtures.cu -- the reference's two verification kernels, rebuilt.
//
//  * distance matrix (compute_distances_warp_kernel, hnsw_traverse.cu:387-415):
//    one warp per (query, row) pair using the reference's warp-order fp32
//    distance, so the values are bit-identical to the reference kernel's;
//  * key/value sort (bitonic_sort_test_kernel, hnsw_traverse.cu:418-437):
//    ascending by key; the reference handles n <= 32 in one warp, this one
//    sorts up to 4096 pairs in one CTA (ties ordered by value).
#include "common.cuh"
#include "kernels.h"
#include "topk.cuh"

namespace fv {

namespace {

__global__ void __launch_bounds__(256) distance_matrix_kernel(const float* __restrict__ queries,
                                                              const float* __restrict__ base, uint32_t nq, uint32_t n,
                                                              uint32_t dim, MetricType metric, float* __restrict__ out) {
  const uint64_t pair = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (pair >= (uint64_t)nq * n) return;
  const uint32_t q = (uint32_t)(pair / n), v = (uint32_t)(pair % n);
  float d = warp_metric_distance(queries + (size_t)q * dim, base + (size_t)v * dim, dim, lane, metric);
  if (lane == 0) out[pair] = d;
}

__global__ void __launch_bounds__(256) bitonic_test_kernel(const float* __restrict__ kin, const uint32_t* __restrict__ vin,
                                                           float* __restrict__ kout, uint32_t* __restrict__ vout,
                                                           uint32_t n, uint32_t pow2) {
  extern __shared__ uint64_t keys[];
  for (uint32_t i = threadIdx.x; i < pow2; i += blockDim.x)
    keys[i] = i < n ? ((uint64_t)float_order(kin[i]) << 32) | vin[i] : kSentinelKey;
  __syncthreads();
  block_bitonic_sort(keys, pow2);
  for (uint32_t i = threadIdx.x; i < n; i += blockDim.x) {
    kout[i] = order_float((uint32_t)(keys[i] >> 32));
    vout[i] = (uint32_t)keys[i];
  }
}

__global__ void fill_sentinel_kernel(GpuSearchResult* out, size_t count) {
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < count; i += (size_t)gridDim.x * blockDim.x)
    out[i] = GpuSearchResult{kInvalidId, kSentinelDist};
}

}  // namespace

int launch_fill_sentinel(GpuSearchResult* out, size_t count, cudaStream_t stream) {
  if (count == 0) return 0;
  const size_t blocks = std::min<size_t>((count + 255) / 256, 4096);
  fill_sentinel_kernel<<<(unsigned)blocks, 256, 0, stream>>>(out, count);
  note_launch();
  return (int)cudaGetLastError();
}

int launch_distance_matrix(const float* queries, const float* base, uint32_t nq, uint32_t n, uint32_t dim,
                           MetricType metric, float* out, cudaStream_t stream) {
  const uint64_t pairs = (uint64_t)nq * n;
  if (pairs == 0) return 0;
  const uint64_t blocks = (pairs + 7) / 8;
  if (blocks > 0x7FFFFFFFull) return -2;
  distance_matrix_kernel<<<(unsigned)blocks, 256, 0, stream>>>(queries, base, nq, n, dim, metric, out);
  note_launch();
  return (int)cudaGetLastError();
}

int launch_bitonic_test(const float* kin, const uint32_t* vin, float* kout, uint32_t* vout, uint32_t n,
                        cudaStream_t stream) {
  if (n == 0) return 0;
  if (n > 4096) return -2;
  const uint32_t pow2 = next_pow2(n);
  bitonic_test_kernel<<<1, 256, pow2 * 8, stream>>>(kin, vin, kout, vout, n, pow2);
  note_launch();
  return (int)cudaGetLastError();
}

}  // namespace fv
