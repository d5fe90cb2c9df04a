// encode.cu -- device-side encoders of the reduced-precision flat tables.
//
//  * fp16: the reference's host encoder encode_fp16_padded / f32_to_f16_bits
//    (crates/engine/src/quant.rs:239-274, 306-327) restated for the GPU:
//    mantissa rounded half-up (not round-to-even), subnormals truncated,
//    rows zero-padded to padded_dim, ||x||^2 as the sequential fp32 sum of
//    the squares (separately rounded multiply and add, as Rust evaluates).
//  * fp8 (no reference counterpart): one power-of-two scale s = 2^b for the
//    whole table, the smallest with max_v ||x_v||^2 <= 896 s^2 (so every
//    code is below 30 in magnitude, far inside e4m3's range: the relative
//    precision of a normal e4m3 code does not depend on the scale, so this
//    equals per-row power-of-two scaling for every code that stays normal);
//    codes = e4m3(x / s) round-to-nearest-even; columns dim, dim + 1,
//    dim + 2 hold three e4m3 "norm digits" n1 + n2 + n3 ~ ||x||^2 / (2 s^2)
//    (each the round-to-nearest-even e4m3 value of what the previous ones
//    left, residual <= 2^-12 relative), so that a query row carrying
//    -s / s_q in those columns makes the tensor-core dot product equal
//    <q, x> / (s s_q) - ||x||^2 / (2 s s_q) -- the L2 ranking value up to
//    the per-query factor -2 s s_q and the query's norm; remaining columns
//    zero; ||x||^2 by compensated (Neumaier) fp32 summation; every entry of
//    the scale array holds s.
//  * fp8, per-row scales (the other layout, selected by the table's
//    scale_mode): s_v = max|x_v| / 448, codes e4m3(x / s_v), no digits.
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

// smallest b in [-62, 62] with mx <= 896 * 4^b (0 for an all-zero table)
__device__ __forceinline__ int fp8_table_exponent(float mx) {
  if (!(mx > 0.f)) return 0;
  int b = max(-62, min(62, (ilogbf(mx) - 9) / 2));
  while (b < 62 && ldexpf(896.0f, 2 * b) < mx) ++b;
  while (b > -62 && ldexpf(896.0f, 2 * (b - 1)) >= mx) --b;
  return b;
}

// ||x||^2 of each row (compensated), and the largest of them as ordered
// bits in *max_bits (norms are >= 0, so the bit patterns order like the values).
__global__ void __launch_bounds__(256) fp8_norms_kernel(const float* __restrict__ x, uint32_t n, uint32_t dim,
                                                        float* __restrict__ norms, uint32_t* __restrict__ max_bits) {
  const uint64_t row = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (row >= n) return;
  const float* src = x + row * dim;
  float sum = 0.f, comp = 0.f;
  for (uint32_t d = lane; d < dim; d += 32) {
    const float v = __ldg(src + d);
    neumaier_add(sum, comp, __fmul_rn(v, v));
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    const float os = __shfl_xor_sync(0xffffffffu, sum, o);
    const float oc = __shfl_xor_sync(0xffffffffu, comp, o);
    neumaier_add(sum, comp, os);
    comp += oc;
  }
  if (lane == 0) {
    const float nrm = sum + comp;
    norms[row] = nrm;
    if (nrm > 0.f) atomicMax(max_bits, __float_as_uint(nrm));
  }
}

// The table's scale exponent b from the largest norm (written over the
// same word, which from here on holds the scale 2^b as a float).
__global__ void fp8_table_scale_kernel(uint32_t* __restrict__ word) {
  const float mx = __uint_as_float(*word);
  *word = __float_as_uint(ldexpf(1.0f, fp8_table_exponent(mx)));
}

// e4m3 code of v (round to nearest even, saturating) and its value.
__device__ __forceinline__ uint8_t e4m3_code(float v) {
  return (uint8_t)__nv_cvt_float_to_fp8(v, __NV_SATFINITE, __NV_E4M3);
}
__device__ __forceinline__ float e4m3_value(uint8_t c) {
  const uint32_t e = (c >> 3) & 15u, m = c & 7u;
  const float mag = e ? ldexpf((float)(8u + m), (int)e - 10) : ldexpf((float)m, -9);
  return (c & 0x80u) ? -mag : mag;
}

__global__ void __launch_bounds__(256) encode_fp8_kernel(const float* __restrict__ x, uint32_t n, uint32_t dim,
                                                         uint32_t pd, uint8_t* __restrict__ out,
                                                         float* __restrict__ scales,
                                                         const float* __restrict__ norms) {
  const uint64_t row = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (row >= n) return;
  // scales[0] holds the table scale (row 0 rewrites it with the same value)
  const float s = scales[0];
  const int b = ilogbf(s);
  const float* src = x + row * dim;
  uint8_t* dst = out + row * pd;
  for (uint32_t d = lane; d < dim; d += 32) dst[d] = e4m3_code(ldexpf(__ldg(src + d), -b));
  if (lane == 0) {
    float r = ldexpf(norms[row], -1 - 2 * b);
    for (int i = 0; i < 3; ++i) {
      const uint8_t c = e4m3_code(r);
      dst[dim + i] = c;
      r -= e4m3_value(c);
    }
  }
  for (uint32_t d = dim + 3 + lane; d < pd; d += 32) dst[d] = 0;
  if (lane == 0) scales[row] = s;
}

// Per-row-scale table (the other fp8 layout): s_v = max|x_v| / 448 (1 for a
// zero row), codes e4m3(x / s_v) round-to-nearest-even with saturation, zero
// padding, ||x||^2 by compensated fp32 summation.
__global__ void __launch_bounds__(256) encode_fp8_per_vector_kernel(const float* __restrict__ x, uint32_t n,
                                                                    uint32_t dim, uint32_t pd, uint8_t* __restrict__ out,
                                                                    float* __restrict__ scales,
                                                                    float* __restrict__ norms) {
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
  for (uint32_t d = lane; d < pd; d += 32) dst[d] = d < dim ? e4m3_code(__ldg(src + d) / scale) : (uint8_t)0;
  if (lane == 0) {
    scales[row] = scale;
    norms[row] = sum + comp;
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
  uint32_t* word = reinterpret_cast<uint32_t*>(scales);
  cudaError_t e = cudaMemsetAsync(word, 0, sizeof(uint32_t), stream);
  if (e != cudaSuccess) return (int)e;
  fp8_norms_kernel<<<(unsigned)blocks, 256, 0, stream>>>(x, n, dim, norms, word);
  fp8_table_scale_kernel<<<1, 1, 0, stream>>>(word);
  encode_fp8_kernel<<<(unsigned)blocks, 256, 0, stream>>>(x, n, dim, pd, out, scales, norms);
  note_launch(3);
  return (int)cudaGetLastError();
}

}  // namespace fv

namespace fv {

int launch_encode_fp8_per_vector(const float* x, uint32_t n, uint32_t dim, uint32_t pd, uint8_t* out, float* scales,
                                 float* norms, cudaStream_t stream) {
  if (n == 0) return 0;
  const uint64_t blocks = ((uint64_t)n * 32 + 255) / 256;
  encode_fp8_per_vector_kernel<<<(unsigned)blocks, 256, 0, stream>>>(x, n, dim, pd, out, scales, norms);
  note_launch();
  return (int)cudaGetLastError();
}

}  // namespace fv
