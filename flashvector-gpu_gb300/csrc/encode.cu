// encode.cu -- device-side encoders of the reduced-precision flat tables.
//
//  * fp16: the reference's host encoder encode_fp16_padded / f32_to_f16_bits
//    (crates/engine/src/quant.rs:239-274, 306-327) restated for the GPU:
//    mantissa rounded half-up (not round-to-even), subnormals truncated,
//    rows zero-padded to padded_dim, ||x||^2 as the sequential fp32 sum of
//    the squares (separately rounded multiply and add, as Rust evaluates).
//  * fp8 (no reference counterpart): per-row scale s = max|x| / 448 (1 for a
//    zero row), codes = e4m3(x / s) round-to-nearest-even with saturation,
//    rows zero-padded, ||x||^2 by compensated (Neumaier) fp32 summation.
#include <cuda_fp8.h>

#include "common.cuh"
#include "kernels.h"

namespace fv {

namespace {

__device__ __forceinline__ uint16_t f32_to_f16_halfup(float x) {
  const uint32_t bits = __float_as_uint(x);
  const uint16_t sign = (uint16_t)((bits >> 16) & 0x8000u);
  const int32_t exp = (int32_t)((bits >> 23) & 0xffu);
  const uint32_t mant = bits & 0x007fffffu;
  if (exp == 255) return (uint16_t)(sign | (mant == 0 ? 0x7c00u : 0x7e00u));
  const int32_t e = exp - 127 + 15;
  if (e >= 31) return (uint16_t)(sign | 0x7c00u);
  if (e <= 0) {
    if (e < -10) return sign;
    return (uint16_t)(sign | (uint16_t)((mant | 0x00800000u) >> (14 - e)));
  }
  const uint32_t r = mant + 0x1000u;
  if (r & 0x00800000u) return (uint16_t)(e + 1 >= 31 ? (sign | 0x7c00u) : (sign | (uint16_t)((e + 1) << 10)));
  return (uint16_t)(sign | (uint16_t)(e << 10) | (uint16_t)(r >> 13));
}

__global__ void __launch_bounds__(256) encode_fp16_kernel(const float* __restrict__ x, uint32_t n, uint32_t dim,
                                                          uint32_t pd, uint16_t* __restrict__ out,
                                                          float* __restrict__ norms) {
  const uint64_t row = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (row >= n) return;
  const float* src = x + row * dim;
  uint16_t* dst = out + row * pd;
  for (uint32_t d = lane; d < pd; d += 32) dst[d] = d < dim ? f32_to_f16_halfup(__ldg(src + d)) : (uint16_t)0;
  if (lane == 0 && norms) {
    float s = 0.f;
    for (uint32_t d = 0; d < dim; ++d) {
      const float v = __ldg(src + d);
      s = __fadd_rn(s, __fmul_rn(v, v));
    }
    norms[row] = s;
  }
}

// Neumaier accumulation of one term.
__device__ __forceinline__ void neumaier_add(float& sum, float& comp, float v) {
  const float t = sum + v;
  if (fabsf(sum) >= fabsf(v))
    comp += (sum - t) + v;
  else
    comp += (v - t) + sum;
  sum = t;
}

__global__ void __launch_bounds__(256) encode_fp8_kernel(const float* __restrict__ x, uint32_t n, uint32_t dim,
                                                         uint32_t pd, uint8_t* __restrict__ out,
                                                         float* __restrict__ scales, float* __restrict__ norms) {
  const uint64_t row = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (row >= n) return;
  const float* src = x + row * dim;
  float amax = 0.f, sum = 0.f, comp = 0.f;
  for (uint32_t d = lane; d < dim; d += 32) {
    const float v = __ldg(src + d);
    amax = fmaxf(amax, fabsf(v));
    neumaier_add(sum, comp, __fmul_rn(v, v));
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    amax = fmaxf(amax, __shfl_xor_sync(0xffffffffu, amax, o));
    const float os = __shfl_xor_sync(0xffffffffu, sum, o);
    const float oc = __shfl_xor_sync(0xffffffffu, comp, o);
    neumaier_add(sum, comp, os);
    comp += oc;
  }
  const float scale = amax > 0.f ? amax / 448.0f : 1.0f;
  uint8_t* dst = out + row * pd;
  for (uint32_t d = lane; d < pd; d += 32)
    dst[d] = d < dim ? (uint8_t)__nv_cvt_float_to_fp8(__ldg(src + d) / scale, __NV_SATFINITE, __NV_E4M3) : (uint8_t)0;
  if (lane == 0) {
    scales[row] = scale;
    if (norms) norms[row] = sum + comp;
  }
}

}  // namespace

int launch_encode_fp16(const float* x, uint32_t n, uint32_t dim, uint32_t pd, uint16_t* out, float* norms,
                       cudaStream_t stream) {
  if (n == 0) return 0;
  const uint64_t blocks = ((uint64_t)n * 32 + 255) / 256;
  encode_fp16_kernel<<<(unsigned)blocks, 256, 0, stream>>>(x, n, dim, pd, out, norms);
  note_launch();
  return (int)cudaGetLastError();
}

int launch_encode_fp8(const float* x, uint32_t n, uint32_t dim, uint32_t pd, uint8_t* out, float* scales,
                      float* norms, cudaStream_t stream) {
  if (n == 0) return 0;
  const uint64_t blocks = ((uint64_t)n * 32 + 255) / 256;
  encode_fp8_kernel<<<(unsigned)blocks, 256, 0, stream>>>(x, n, dim, pd, out, scales, norms);
  note_launch();
  return (int)cudaGetLastError();
}

}  // namespace fv
