// index_build.cu -- GPU kernels of the IVF index build.
//
// The reference builds its IVF tables on the host (crates/engine/src/
// cluster.rs:28-287, quant.rs:14-75, index.rs:405-458): k-means++ seeding,
// Lloyd iterations, residuals, PQ codebooks by per-sub-space k-means, PQ
// nearest-codeword encode, SQ8 min/max fit and encode, posting lists. At 10M
// rows and 16,384 lists that is hours of host time, so the build runs here
// on the GPU:
//   * assignment: nearest centroid through the exact flat scan (k = 1);
//   * centroid update: per-centroid sums in fp64 (atomics), divided once;
//     an empty cluster keeps its previous centroid;
//   * posting lists: counts, exclusive scan, scatter (ids within a list are
//     in no particular order -- search results do not depend on it, they
//     are ordered by (distance, id));
//   * PQ encode: one thread per (row, sub-space), the 256 codewords of the
//     sub-space in shared memory, nearest by the sequential fp32 squared
//     distance with strict `<` (cluster.rs:257-282);
//   * SQ8: per-dimension min / max (fp32 bit-pattern atomics), scale =
//     range / 255 or 0 when range <= 1e-12, code = round-half-away(
//     (r - min) / scale) clamped to [0, 255] (quant.rs:14-75);
//   * RaBitQ: one warp per row, the row's residual rotated in shared memory
//     (three rounds of sign flip, Walsh-Hadamard butterflies, 1/sqrt(P)
//     scale), sign bits by warp ballot, |r|^2, |x|^2 and sum |rot r| summed
//     sequentially by single lanes in the reference's order
//     (quant.rs:156-234), so the tables equal the host encoder's bit for bit.
#include <algorithm>
#include <cmath>

#include "../../include/fv_bridge.h"
#include "common.cuh"
#include "kernels.h"

namespace fv {

namespace {

__global__ void zero_f64_kernel(double* p, size_t n) {
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) p[i] = 0.0;
}

__global__ void kmeans_accumulate_kernel(const float* __restrict__ x, uint32_t n, uint32_t dim,
                                         const GpuSearchResult* __restrict__ assign, double* __restrict__ sums,
                                         uint32_t* __restrict__ counts, uint32_t k) {
  const uint64_t total = (uint64_t)n * dim;
  for (uint64_t e = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; e < total; e += (uint64_t)gridDim.x * blockDim.x) {
    const uint32_t i = (uint32_t)(e / dim), d = (uint32_t)(e % dim);
    const uint32_t c = assign[i].id;
    if (c >= k) continue;
    atomicAdd(sums + (size_t)c * dim + d, (double)x[e]);
    if (d == 0) atomicAdd(counts + c, 1u);
  }
}

__global__ void kmeans_finish_kernel(const double* __restrict__ sums, const uint32_t* __restrict__ counts, uint32_t k,
                                     uint32_t dim, float* __restrict__ centroids) {
  const uint64_t total = (uint64_t)k * dim;
  for (uint64_t e = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; e < total; e += (uint64_t)gridDim.x * blockDim.x) {
    const uint32_t c = (uint32_t)(e / dim);
    const uint32_t cnt = counts[c];
    if (cnt > 0) centroids[e] = (float)(sums[e] / (double)cnt);
  }
}

__global__ void count_lists_kernel(const GpuSearchResult* __restrict__ assign, uint32_t n, uint32_t nlist,
                                   uint32_t* __restrict__ counts) {
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const uint32_t c = assign[i].id;
    if (c < nlist) atomicAdd(counts + c, 1u);
  }
}

// exclusive scan of counts[0..m) into offsets[0..m] by one block
__global__ void __launch_bounds__(1024) scan_offsets_kernel(const uint32_t* __restrict__ counts, uint32_t m,
                                                            uint32_t* __restrict__ offsets) {
  __shared__ uint32_t part[1024];
  const uint32_t per = (m + 1023) / 1024;
  const uint32_t b = threadIdx.x * per, e = min(b + per, m);
  uint32_t s = 0;
  for (uint32_t i = b; i < e; ++i) s += counts[i];
  part[threadIdx.x] = s;
  __syncthreads();
  for (uint32_t off = 1; off < 1024; off <<= 1) {
    const uint32_t v = threadIdx.x >= off ? part[threadIdx.x - off] : 0u;
    __syncthreads();
    part[threadIdx.x] += v;
    __syncthreads();
  }
  uint32_t run = part[threadIdx.x] - s;  // exclusive prefix of this thread's range
  for (uint32_t i = b; i < e; ++i) {
    offsets[i] = run;
    run += counts[i];
  }
  if (threadIdx.x == 1023) offsets[m] = part[1023];
}

__global__ void scatter_lists_kernel(const GpuSearchResult* __restrict__ assign, uint32_t n, uint32_t nlist,
                                     uint32_t* __restrict__ cursor, uint32_t* __restrict__ vec_ids) {
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const uint32_t c = assign[i].id;
    if (c < nlist) vec_ids[atomicAdd(cursor + c, 1u)] = i;
  }
}

__global__ void residuals_kernel(const float* __restrict__ x, uint32_t n, uint32_t dim,
                                 const float* __restrict__ centroids, const GpuSearchResult* __restrict__ assign,
                                 float* __restrict__ out) {
  const uint64_t total = (uint64_t)n * dim;
  for (uint64_t e = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; e < total; e += (uint64_t)gridDim.x * blockDim.x) {
    const uint32_t i = (uint32_t)(e / dim), d = (uint32_t)(e % dim);
    out[e] = x[e] - centroids[(size_t)assign[i].id * dim + d];
  }
}

__global__ void extract_subspace_kernel(const float* __restrict__ x, uint32_t n, uint32_t dim, uint32_t off,
                                        uint32_t sub, float* __restrict__ out) {
  const uint64_t total = (uint64_t)n * sub;
  for (uint64_t e = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; e < total; e += (uint64_t)gridDim.x * blockDim.x) {
    const uint64_t i = e / sub, s = e % sub;
    out[e] = x[i * dim + off + s];
  }
}

// One thread per (row, sub-space); the sub-space's 256 codewords staged in
// shared memory (grid.y = sub-space).
__global__ void __launch_bounds__(256) pq_encode_kernel(const float* __restrict__ x, uint32_t n, uint32_t dim,
                                                        uint32_t m_pq, uint32_t sub,
                                                        const float* __restrict__ codebooks,
                                                        uint8_t* __restrict__ codes) {
  extern __shared__ float cb[];  // [256][sub]
  const uint32_t m = blockIdx.y;
  for (uint32_t e = threadIdx.x; e < 256 * sub; e += blockDim.x) cb[e] = codebooks[(size_t)m * 256 * sub + e];
  __syncthreads();
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const float* v = x + (size_t)i * dim + m * sub;
    float best = __int_as_float(0x7f800000);
    uint32_t bc = 0;
    for (uint32_t c = 0; c < 256; ++c) {
      float s = 0.f;
      for (uint32_t d = 0; d < sub; ++d) {
        const float t = __fsub_rn(v[d], cb[c * sub + d]);
        s = __fadd_rn(s, __fmul_rn(t, t));
      }
      if (s < best) {
        best = s;
        bc = c;
      }
    }
    codes[(size_t)i * m_pq + m] = (uint8_t)bc;
  }
}

__device__ __forceinline__ uint32_t f2ord(float f) {
  const uint32_t u = __float_as_uint(f);
  return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}
__device__ __forceinline__ float ord2f(uint32_t o) {
  return __uint_as_float((o & 0x80000000u) ? (o & 0x7FFFFFFFu) : ~o);
}

__global__ void minmax_init_kernel(uint32_t* mn, uint32_t* mx, uint32_t dim) {
  for (uint32_t d = blockIdx.x * blockDim.x + threadIdx.x; d < dim; d += gridDim.x * blockDim.x) {
    mn[d] = 0xFFFFFFFFu;
    mx[d] = 0u;
  }
}

__global__ void minmax_kernel(const float* __restrict__ r, uint32_t n, uint32_t dim, uint32_t* mn, uint32_t* mx) {
  // each thread folds a strided range of rows for one dimension
  const uint32_t d = threadIdx.x % dim;
  uint32_t lo = 0xFFFFFFFFu, hi = 0u;
  const uint32_t rows_per = blockDim.x / dim;
  if (threadIdx.x >= rows_per * dim) return;
  for (uint32_t i = blockIdx.x * rows_per + threadIdx.x / dim; i < n; i += gridDim.x * rows_per) {
    const uint32_t o = f2ord(r[(size_t)i * dim + d]);
    lo = min(lo, o);
    hi = max(hi, o);
  }
  atomicMin(mn + d, lo);
  atomicMax(mx + d, hi);
}

__global__ void sq8_scales_kernel(const uint32_t* mn, const uint32_t* mx, uint32_t dim, uint32_t n,
                                  float* __restrict__ mins, float* __restrict__ scales) {
  for (uint32_t d = blockIdx.x * blockDim.x + threadIdx.x; d < dim; d += gridDim.x * blockDim.x) {
    const float lo = n ? ord2f(mn[d]) : 0.f, hi = n ? ord2f(mx[d]) : 0.f;
    const float range = __fsub_rn(hi, lo);
    mins[d] = lo;
    scales[d] = range > 1e-12f ? __fdiv_rn(range, 255.0f) : 0.f;
  }
}

__global__ void sq8_encode_kernel(const float* __restrict__ r, uint32_t n, uint32_t dim, const float* __restrict__ mins,
                                  const float* __restrict__ scales, uint8_t* __restrict__ codes) {
  const uint64_t total = (uint64_t)n * dim;
  for (uint64_t e = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; e < total; e += (uint64_t)gridDim.x * blockDim.x) {
    const uint32_t d = (uint32_t)(e % dim);
    const float s = scales[d];
    uint8_t c = 0;
    if (s > 0.f) {
      float q = roundf(__fdiv_rn(__fsub_rn(r[e], mins[d]), s));
      q = fminf(fmaxf(q, 0.f), 255.f);
      c = (uint8_t)q;
    }
    codes[e] = c;
  }
}

__global__ void gather_rows_kernel(const float* __restrict__ x, const uint32_t* __restrict__ rows, uint32_t count,
                                   uint32_t dim, float* __restrict__ out) {
  const uint64_t total = (uint64_t)count * dim;
  for (uint64_t e = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; e < total; e += (uint64_t)gridDim.x * blockDim.x) {
    const uint64_t i = e / dim, d = e % dim;
    out[e] = x[(uint64_t)rows[i] * dim + d];
  }
}

// out row i = in row rows[i], or zeros when rows[i] == zero_row; rows of
// `words` 32-bit words (snapshot loads that place slots at logical ids)
__global__ void gather_word_rows_kernel(const uint32_t* __restrict__ in, const uint32_t* __restrict__ rows,
                                        uint32_t count, uint32_t words, uint32_t zero_row,
                                        uint32_t* __restrict__ out) {
  const uint64_t total = (uint64_t)count * words;
  for (uint64_t e = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; e < total; e += (uint64_t)gridDim.x * blockDim.x) {
    const uint64_t i = e / words, w = e % words;
    const uint32_t r = rows[i];
    out[e] = r == zero_row ? 0u : in[(uint64_t)r * words + w];
  }
}

__global__ void gather_byte_rows_kernel(const uint8_t* __restrict__ in, const uint32_t* __restrict__ rows,
                                        uint32_t count, uint32_t row_bytes, uint32_t zero_row,
                                        uint8_t* __restrict__ out) {
  const uint64_t total = (uint64_t)count * row_bytes;
  for (uint64_t e = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; e < total; e += (uint64_t)gridDim.x * blockDim.x) {
    const uint64_t i = e / row_bytes, b = e % row_bytes;
    const uint32_t r = rows[i];
    out[e] = r == zero_row ? (uint8_t)0 : in[(uint64_t)r * row_bytes + b];
  }
}

constexpr int RQ_WARPS = 4;

// RaBitQ encoder. bits == nullptr: rot_out row = rotation of x row (the
// rotated centroids). Otherwise the residual of x row to centroid
// assign[row] is rotated and its sign bits and meta written.
__global__ void __launch_bounds__(RQ_WARPS * 32)
    rabitq_encode_kernel(const float* __restrict__ x, uint32_t n, uint32_t dim, const float* __restrict__ centroids,
                         uint32_t nlist, const GpuSearchResult* __restrict__ assign, const float* __restrict__ signs,
                         uint32_t P, float scale, float* __restrict__ rot_out, uint32_t* __restrict__ bits,
                         float* __restrict__ meta) {
  extern __shared__ float rq_smem[];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const uint32_t W = P / 32;
  float* buf = rq_smem + (size_t)warp * P;
  for (uint32_t row = blockIdx.x * RQ_WARPS + warp; row < n; row += gridDim.x * RQ_WARPS) {
    const float* v = x + (size_t)row * dim;
    const float* ce = nullptr;
    if (bits) {
      const uint32_t c = assign[row].id;
      if (c < nlist) ce = centroids + (size_t)c * dim;
    }
    for (uint32_t d = lane; d < P; d += 32) buf[d] = d < dim ? (ce ? __fsub_rn(__ldg(v + d), __ldg(ce + d)) : __ldg(v + d)) : 0.f;
    __syncwarp();
    float res_sq = 0.f, vec_sq = 0.f, abs_sum = 0.f;
    if (bits) {
      // res_norm_sq += r * r, vec_norm_sq += x * x in dimension order
      if (lane == 0)
        for (uint32_t d = 0; d < dim; ++d) res_sq = __fadd_rn(res_sq, __fmul_rn(buf[d], buf[d]));
      if (lane == 1)
        for (uint32_t d = 0; d < dim; ++d) {
          const float xv = __ldg(v + d);
          vec_sq = __fadd_rn(vec_sq, __fmul_rn(xv, xv));
        }
      __syncwarp();
    }
    for (int st = 0; st < 3; ++st) {
      const float* sg = signs + (size_t)st * P;
      for (uint32_t d = lane; d < P; d += 32) buf[d] = __fmul_rn(buf[d], __ldg(sg + d));
      __syncwarp();
      for (uint32_t h = 1; h < P; h <<= 1) {
        for (uint32_t i = lane; i < P / 2; i += 32) {
          const uint32_t x0 = ((i & ~(h - 1)) << 1) | (i & (h - 1));
          const float a = buf[x0], b = buf[x0 + h];
          buf[x0] = __fadd_rn(a, b);
          buf[x0 + h] = __fsub_rn(a, b);
        }
        __syncwarp();
      }
      for (uint32_t d = lane; d < P; d += 32) buf[d] = __fmul_rn(buf[d], scale);
      __syncwarp();
    }
    if (!bits) {
      for (uint32_t d = lane; d < P; d += 32) rot_out[(size_t)row * P + d] = buf[d];
      __syncwarp();
      continue;
    }
    uint32_t pop = 0;
    for (uint32_t w = 0; w < W; ++w) {
      const uint32_t b = __ballot_sync(0xffffffffu, buf[w * 32 + lane] >= 0.f);
      if (lane == 0) bits[(size_t)row * W + w] = b;
      pop += __popc(b);
    }
    if (lane == 2)
      for (uint32_t d = 0; d < P; ++d) abs_sum = __fadd_rn(abs_sum, fabsf(buf[d]));
    res_sq = __shfl_sync(0xffffffffu, res_sq, 0);
    vec_sq = __shfl_sync(0xffffffffu, vec_sq, 1);
    abs_sum = __shfl_sync(0xffffffffu, abs_sum, 2);
    if (lane == 0) {
      const float rn = __fsqrt_rn(res_sq);
      float* m = meta + (size_t)row * 4;
      m[0] = res_sq;
      m[1] = (rn > 1e-12f && abs_sum > 1e-12f) ? __fdiv_rn(__fmul_rn(rn, rn), abs_sum) : 0.f;
      m[2] = (float)pop;
      m[3] = vec_sq;
    }
    __syncwarp();
  }
}

__global__ void fill_f32_kernel(float* p, size_t n, float v) {
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) p[i] = v;
}

unsigned grid_for(uint64_t work) {
  return (unsigned)std::max<uint64_t>(1, std::min<uint64_t>((work + 255) / 256, 152ull * 64));
}

}  // namespace

int launch_kmeans_update(const float* x, uint32_t n, uint32_t dim, const GpuSearchResult* assign, uint32_t k,
                         float* centroids, uint32_t* counts, double* sums, cudaStream_t stream) {
  zero_f64_kernel<<<grid_for((uint64_t)k * dim), 256, 0, stream>>>(sums, (size_t)k * dim);
  cudaError_t e = cudaMemsetAsync(counts, 0, (size_t)k * 4, stream);
  if (e != cudaSuccess) return (int)e;
  kmeans_accumulate_kernel<<<grid_for((uint64_t)n * dim), 256, 0, stream>>>(x, n, dim, assign, sums, counts, k);
  kmeans_finish_kernel<<<grid_for((uint64_t)k * dim), 256, 0, stream>>>(sums, counts, k, dim, centroids);
  note_launch(3);
  return (int)cudaGetLastError();
}

int launch_build_lists(const GpuSearchResult* assign, uint32_t n, uint32_t nlist, uint32_t* offsets, uint32_t* vec_ids,
                       uint32_t* work, cudaStream_t stream) {
  cudaError_t e = cudaMemsetAsync(work, 0, (size_t)nlist * 4, stream);
  if (e != cudaSuccess) return (int)e;
  count_lists_kernel<<<grid_for(n), 256, 0, stream>>>(assign, n, nlist, work);
  scan_offsets_kernel<<<1, 1024, 0, stream>>>(work, nlist, offsets);
  e = cudaMemcpyAsync(work, offsets, (size_t)nlist * 4, cudaMemcpyDeviceToDevice, stream);
  if (e != cudaSuccess) return (int)e;
  scatter_lists_kernel<<<grid_for(n), 256, 0, stream>>>(assign, n, nlist, work, vec_ids);
  note_launch(3);
  return (int)cudaGetLastError();
}

int launch_residuals(const float* x, uint32_t n, uint32_t dim, const float* centroids, const GpuSearchResult* assign,
                     float* out, cudaStream_t stream) {
  residuals_kernel<<<grid_for((uint64_t)n * dim), 256, 0, stream>>>(x, n, dim, centroids, assign, out);
  note_launch();
  return (int)cudaGetLastError();
}

int launch_extract_subspace(const float* x, uint32_t n, uint32_t dim, uint32_t off, uint32_t sub, float* out,
                            cudaStream_t stream) {
  extract_subspace_kernel<<<grid_for((uint64_t)n * sub), 256, 0, stream>>>(x, n, dim, off, sub, out);
  note_launch();
  return (int)cudaGetLastError();
}

int launch_pq_encode(const float* x, uint32_t n, uint32_t dim, uint32_t m_pq, const float* codebooks, uint8_t* codes,
                     cudaStream_t stream) {
  if (m_pq == 0 || dim % m_pq) return -2;
  const uint32_t sub = dim / m_pq;
  const size_t smem = (size_t)256 * sub * 4;
  if (smem > 200 * 1024) return -2;
  cudaFuncSetAttribute(pq_encode_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  dim3 grid(std::max(1u, std::min<uint32_t>((n + 255) / 256, 2048u)), m_pq);
  pq_encode_kernel<<<grid, 256, smem, stream>>>(x, n, dim, m_pq, sub, codebooks, codes);
  note_launch();
  return (int)cudaGetLastError();
}

int launch_sq8_fit(const float* r, uint32_t n, uint32_t dim, float* mins, float* scales, uint32_t* work,
                   cudaStream_t stream) {
  if (dim == 0 || dim > 1024) return -2;
  minmax_init_kernel<<<grid_for(dim), 256, 0, stream>>>(work, work + dim, dim);
  const uint32_t threads = std::max(dim, 1024u / dim * dim);
  minmax_kernel<<<std::max(1u, std::min<uint32_t>(n, 2048u)), threads, 0, stream>>>(r, n, dim, work, work + dim);
  sq8_scales_kernel<<<grid_for(dim), 256, 0, stream>>>(work, work + dim, dim, n, mins, scales);
  note_launch(3);
  return (int)cudaGetLastError();
}

int launch_sq8_encode(const float* r, uint32_t n, uint32_t dim, const float* mins, const float* scales, uint8_t* codes,
                      cudaStream_t stream) {
  sq8_encode_kernel<<<grid_for((uint64_t)n * dim), 256, 0, stream>>>(r, n, dim, mins, scales, codes);
  note_launch();
  return (int)cudaGetLastError();
}

int launch_gather_rows(const float* x, const uint32_t* rows, uint32_t count, uint32_t dim, float* out,
                       cudaStream_t stream) {
  if (count == 0) return 0;
  gather_rows_kernel<<<grid_for((uint64_t)count * dim), 256, 0, stream>>>(x, rows, count, dim, out);
  note_launch();
  return (int)cudaGetLastError();
}

int launch_gather_row_bytes(const void* in, const uint32_t* rows, uint32_t count, uint32_t row_bytes,
                            uint32_t zero_row, void* out, cudaStream_t stream) {
  if (count == 0 || row_bytes == 0) return 0;
  if (row_bytes % 4 == 0 && (uintptr_t)in % 4 == 0 && (uintptr_t)out % 4 == 0) {
    const uint32_t words = row_bytes / 4;
    gather_word_rows_kernel<<<grid_for((uint64_t)count * words), 256, 0, stream>>>(
        static_cast<const uint32_t*>(in), rows, count, words, zero_row, static_cast<uint32_t*>(out));
  } else {
    gather_byte_rows_kernel<<<grid_for((uint64_t)count * row_bytes), 256, 0, stream>>>(
        static_cast<const uint8_t*>(in), rows, count, row_bytes, zero_row, static_cast<uint8_t*>(out));
  }
  note_launch();
  return (int)cudaGetLastError();
}

uint32_t rabitq_padded_dim(uint32_t dim) {
  uint32_t p = 32;
  while (p < dim) p <<= 1;
  return p;
}

float rabitq_inv_sqrt(uint32_t padded_dim) { return 1.0f / std::sqrt((float)padded_dim); }

// The reference's seeded sign generator (quant.rs:100-116): a splitmix64
// stream whose state starts at seed ^ 0x9e3779b97f4a7c15; sign = -1 when
// the output's low bit is set.
void rabitq_rot_signs(uint32_t padded_dim, uint64_t seed, float* out) {
  const uint64_t inc = 0x9e3779b97f4a7c15ull;
  uint64_t st = seed ^ inc;
  for (uint32_t i = 0; i < 3u * padded_dim; ++i) {
    st += inc;
    uint64_t z = st;
    z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
    z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
    z ^= z >> 31;
    out[i] = (z & 1u) ? -1.0f : 1.0f;
  }
}

int launch_rabitq_encode(const float* x, uint32_t n, uint32_t dim, const float* centroids, uint32_t nlist,
                         const GpuSearchResult* assign, const float* signs, uint32_t padded_dim, float* rot_centroids,
                         uint32_t* bits, float* meta, cudaStream_t stream) {
  const uint32_t P = padded_dim;
  if (P < 32 || P > 4096 || (P & (P - 1)) || P < dim) return FV_ERR_ARG;
  const size_t smem = (size_t)RQ_WARPS * P * 4;
  cudaError_t e = cudaFuncSetAttribute(rabitq_encode_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return (int)e;
  const float scale = rabitq_inv_sqrt(P);
  const uint32_t cap = (uint32_t)device_sm_count() * 16;
  if (nlist) {
    const uint32_t blocks = std::max(1u, std::min(cap, (nlist + RQ_WARPS - 1) / RQ_WARPS));
    rabitq_encode_kernel<<<blocks, RQ_WARPS * 32, smem, stream>>>(centroids, nlist, dim, nullptr, 0, nullptr, signs, P,
                                                                   scale, rot_centroids, nullptr, nullptr);
    note_launch();
  }
  if (n) {
    const uint32_t blocks = std::max(1u, std::min(cap, (n + RQ_WARPS - 1) / RQ_WARPS));
    rabitq_encode_kernel<<<blocks, RQ_WARPS * 32, smem, stream>>>(x, n, dim, centroids, nlist, assign, signs, P, scale,
                                                                   nullptr, bits, meta);
    note_launch();
  }
  return (int)cudaGetLastError();
}

int launch_fill_f32(float* p, size_t n, float v, cudaStream_t stream) {
  if (n == 0) return 0;
  fill_f32_kernel<<<grid_for(n), 256, 0, stream>>>(p, n, v);
  note_launch();
  return (int)cudaGetLastError();
}

}  // namespace fv
