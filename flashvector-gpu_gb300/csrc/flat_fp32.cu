// flat_fp32.cu -- exact fp32 flat scan fused with top-k.
//
// Replaces the reference's flat_scan_kernel / launch_flat_scan
// (sparse_hybrid.cu:13-107). Same contract, different machine mapping:
//
//  * a CTA owns 64 queries and a contiguous range of base tiles (128 rows);
//    every base tile is staged once in shared memory and scored against all
//    64 queries (the reference re-streams the whole base set per query);
//  * each thread accumulates a 4 x 8 block of (query, row) distances,
//    walking the dimensions in ascending order with separately rounded
//    subtract / multiply / add -- the order of the reference's own exact
//    search RecallEvaluator::exact_knn (metrics.rs:103-135), so distances
//    are bit-identical to it;
//  * per query a max-heap of (distance, slot) keys in shared memory keeps
//    the running top-k (ties -> lower slot, as the reference's strict `<`
//    insertion in slot order); after each tile every thread tests its own
//    4 x 8 block against the queries' current k-th keys and appends only
//    the keys that can enter to a per-query candidate list, so the
//    per-query heap work touches a few keys instead of the whole tile;
//  * when the base range is split over several CTAs the per-split heaps go
//    to scratch and a second kernel merges them.
#include <mutex>

#include "../../include/fv_bridge.h"
#include "common.cuh"
#include "kernels.h"
#include "topk.cuh"

namespace fv {

namespace {

constexpr int QT = 64;    // queries per CTA
constexpr int VT = 128;   // base rows per tile
constexpr int DK = 32;    // dimensions per staged chunk
constexpr int NT = 256;   // threads per CTA
// padded row strides of the staged chunks: multiples of 4 floats so that
// every operand read of the inner loop is one 16-byte shared load
constexpr int QS = QT + 4;
constexpr int VS = VT + 4;

struct FlatArgs {
  const float* vectors;
  const uint32_t* vec_ids;
  uint32_t n, dim;
  const float* queries;
  uint32_t nq, k;
  const uint32_t* mask;
  GpuSearchResult* out;   // written directly when splits == 1
  uint64_t* partial;      // [nq][splits][k] heap dumps when splits > 1
  uint32_t splits, tiles_per_split;
  const QueryFilter* filters;  // per-query filters over logical ids (vec_ids[slot], or slot), or null
};

__device__ __forceinline__ void heap_replace_root(uint64_t* heap, int k, int lane_stride, uint64_t key) {
  // max-heap stored interleaved: element i of this query at heap[i * lane_stride]
  int i = 0;
  while (true) {
    int l = 2 * i + 1;
    if (l >= k) break;
    uint64_t cv = heap[l * lane_stride];
    int c = l;
    if (l + 1 < k) {
      uint64_t rv = heap[(l + 1) * lane_stride];
      if (rv > cv) { cv = rv; c = l + 1; }
    }
    if (cv <= key) break;
    heap[i * lane_stride] = cv;
    i = c;
  }
  heap[i * lane_stride] = key;
}

// In-place heapsort of a max-heap (ascending result).
__device__ void heap_sort_ascending(uint64_t* heap, int k, int s) {
  for (int end = k - 1; end > 0; --end) {
    uint64_t top = heap[0];
    uint64_t last = heap[end * s];
    heap[end * s] = top;
    // sift `last` down from the root within [0, end)
    int i = 0;
    while (true) {
      int l = 2 * i + 1;
      if (l >= end) break;
      uint64_t cv = heap[l * s];
      int c = l;
      if (l + 1 < end) {
        uint64_t rv = heap[(l + 1) * s];
        if (rv > cv) { cv = rv; c = l + 1; }
      }
      if (cv <= last) break;
      heap[i * s] = cv;
      i = c;
    }
    heap[i * s] = last;
  }
}

// FUSED = false: separately rounded sub/mul/add in dimension order (the
// reference's exact search). FUSED = true: fmaf(diff, diff, acc) in
// dimension order (the reference's coarse quantizer, ivf_rerank.cuh:80-84).
template <int METRIC, bool VEC4, bool FUSED = false>
__global__ void __launch_bounds__(NT) flat_f32_scan_kernel(FlatArgs a) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  float* qs = reinterpret_cast<float*>(smem_raw);  // [DK][QS]
  float* xs = qs + DK * QS;                          // [DK][VS]
  float* cd = xs + DK * VS;                          // [QT][VT] candidate distances of a tile
  float* qn = cd + QT * VT;                          // [QT]
  float* xn = qn + QT;                               // [VT]
  uint64_t* heap = reinterpret_cast<uint64_t*>(xn + VT);  // [k][QT], 8B aligned (see smem size)
  uint64_t* wq = heap + (size_t)a.k * QT;                 // [QT] current k-th key per query
  uint32_t* cnt = reinterpret_cast<uint32_t*>(wq + QT);   // [QT] candidates of the tile per query
  uint8_t* cr = reinterpret_cast<uint8_t*>(cnt + QT);     // [QT][VT] their rows within the tile

  const int tid = threadIdx.x;
  const int ty = tid >> 4, tx = tid & 15;
  const uint32_t q0 = blockIdx.x * QT;
  const uint32_t k = a.k;
  const uint32_t ntiles = (a.n + VT - 1) / VT;
  const uint32_t t_begin = blockIdx.y * a.tiles_per_split;
  const uint32_t t_end = min(t_begin + a.tiles_per_split, ntiles);

  for (uint32_t i = tid; i < k * QT; i += NT) heap[i] = kSentinelKey;
  if (tid < QT) {
    wq[tid] = kSentinelKey;
    cnt[tid] = 0;
  }
  if (METRIC == METRIC_COSINE && tid < QT) {
    float s = 0.f;
    if (q0 + tid < a.nq) {
      const float* q = a.queries + (size_t)(q0 + tid) * a.dim;
      for (uint32_t d = 0; d < a.dim; ++d) s = __fadd_rn(s, __fmul_rn(q[d], q[d]));
    }
    qn[tid] = s;
  }
  __syncthreads();

  uint64_t worst = kSentinelKey;  // cached heap root of query `tid` (tid < QT)
  QueryFilter qf[4];              // filters of this thread's four queries
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    const uint32_t q = q0 + ty * 4 + i;
    qf[i] = (a.filters && q < a.nq) ? load_filter(a.filters, q) : QueryFilter{nullptr, 0u, 0u};
  }

  for (uint32_t t = t_begin; t < t_end; ++t) {
    const uint32_t v0 = t * VT;
    float acc[4][8];
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
      for (int j = 0; j < 8; ++j) acc[i][j] = 0.f;
    float xnorm = 0.f;

    for (uint32_t d0 = 0; d0 < a.dim; d0 += DK) {
      const uint32_t dk = min((uint32_t)DK, a.dim - d0);
      __syncthreads();  // previous chunk fully consumed
      if (VEC4) {
        // 64 queries x 32 dims = 512 float4; 128 rows x 32 dims = 1024 float4
#pragma unroll
        for (int r = 0; r < 2; ++r) {
          int e = tid + NT * r;
          int qi = e >> 3, dd = (e & 7) * 4;
          float4 v = make_float4(0.f, 0.f, 0.f, 0.f);
          if (q0 + qi < a.nq && d0 + dd < a.dim)
            v = __ldg(reinterpret_cast<const float4*>(a.queries + (size_t)(q0 + qi) * a.dim + d0 + dd));
          qs[(dd + 0) * QS + qi] = v.x;
          qs[(dd + 1) * QS + qi] = v.y;
          qs[(dd + 2) * QS + qi] = v.z;
          qs[(dd + 3) * QS + qi] = v.w;
        }
#pragma unroll
        for (int r = 0; r < 4; ++r) {
          int e = tid + NT * r;
          int vi = e >> 3, dd = (e & 7) * 4;
          float4 v = make_float4(0.f, 0.f, 0.f, 0.f);
          if (v0 + vi < a.n && d0 + dd < a.dim)
            v = __ldg(reinterpret_cast<const float4*>(a.vectors + (size_t)(v0 + vi) * a.dim + d0 + dd));
          xs[(dd + 0) * VS + vi] = v.x;
          xs[(dd + 1) * VS + vi] = v.y;
          xs[(dd + 2) * VS + vi] = v.z;
          xs[(dd + 3) * VS + vi] = v.w;
        }
      } else {
#pragma unroll
        for (int r = 0; r < (QT * DK) / NT; ++r) {
          int e = tid + NT * r;
          int qi = e / DK, dd = e % DK;
          float v = 0.f;
          if (q0 + qi < a.nq && d0 + dd < a.dim) v = __ldg(a.queries + (size_t)(q0 + qi) * a.dim + d0 + dd);
          qs[dd * QS + qi] = v;
        }
#pragma unroll
        for (int r = 0; r < (VT * DK) / NT; ++r) {
          int e = tid + NT * r;
          int vi = e / DK, dd = e % DK;
          float v = 0.f;
          if (v0 + vi < a.n && d0 + dd < a.dim) v = __ldg(a.vectors + (size_t)(v0 + vi) * a.dim + d0 + dd);
          xs[dd * VS + vi] = v;
        }
      }
      __syncthreads();

      if (METRIC == METRIC_COSINE && tid < VT) {
        for (uint32_t dd = 0; dd < dk; ++dd) {
          float x = xs[dd * VS + tid];
          xnorm = __fadd_rn(xnorm, __fmul_rn(x, x));
        }
      }

      auto step = [&](int dd) {
        // this thread's 4 queries and 8 rows (columns 4 tx.. and 64 + 4 tx..)
        // of dimension dd: three 16-byte loads
        const float4 q4 = *reinterpret_cast<const float4*>(qs + dd * QS + ty * 4);
        const float4 xa = *reinterpret_cast<const float4*>(xs + dd * VS + 4 * tx);
        const float4 xb = *reinterpret_cast<const float4*>(xs + dd * VS + 64 + 4 * tx);
        const float qv[4] = {q4.x, q4.y, q4.z, q4.w};
        const float xv[8] = {xa.x, xa.y, xa.z, xa.w, xb.x, xb.y, xb.z, xb.w};
#pragma unroll
        for (int i = 0; i < 4; ++i)
#pragma unroll
          for (int j = 0; j < 8; ++j) {
            if (METRIC == METRIC_L2 && FUSED) {
              float diff = __fsub_rn(qv[i], xv[j]);
              acc[i][j] = fmaf(diff, diff, acc[i][j]);
            } else if (METRIC == METRIC_L2) {
              float diff = __fsub_rn(qv[i], xv[j]);
              acc[i][j] = __fadd_rn(acc[i][j], __fmul_rn(diff, diff));
            } else {
              acc[i][j] = __fadd_rn(acc[i][j], __fmul_rn(qv[i], xv[j]));
            }
          }
      };
      if (dk == DK) {
#pragma unroll 8
        for (int dd = 0; dd < DK; ++dd) step(dd);
      } else {
        for (uint32_t dd = 0; dd < dk; ++dd) step((int)dd);
      }
    }

    if (METRIC == METRIC_COSINE && tid < VT) xn[tid] = xnorm;
    __syncthreads();  // xn visible; the previous selection has finished (wq, cnt)

#pragma unroll
    for (int i = 0; i < 4; ++i) {
      const int qi = ty * 4 + i;
      const uint64_t wk = wq[qi];
#pragma unroll
      for (int j = 0; j < 8; ++j) {
        const int vi = (j < 4 ? 0 : 64) + 4 * tx + (j & 3);  // the row of acc[.][j] (see step)
        float dist;
        if (METRIC == METRIC_L2) {
          dist = acc[i][j];
        } else if (METRIC == METRIC_INNER_PRODUCT) {
          dist = -acc[i][j];
        } else {
          float denom = __fadd_rn(__fmul_rn(sqrtf(qn[qi]), sqrtf(xn[vi])), 1e-8f);
          dist = __fsub_rn(1.0f, __fdiv_rn(acc[i][j], denom));
        }
        const uint32_t slot = v0 + vi;
        // a key that cannot beat the query's current k-th key never enters
        // (the k-th key only decreases, so testing against an older one
        // admits a superset); NaN fails `<`
        if (dist < kSentinelDist && make_key(dist, slot) < wk && slot < a.n && mask_allows(a.mask, slot) &&
            (!a.filters || filter_allows(qf[i], a.vec_ids ? __ldg(a.vec_ids + slot) : slot))) {
          const uint32_t pos = atomicAdd(cnt + qi, 1u);
          cd[qi * VT + pos] = dist;
          cr[qi * VT + pos] = (uint8_t)vi;
        }
      }
    }
    __syncthreads();

    if (tid < QT) {
      // the tile's candidates of query tid, inserted in row order (the kept
      // set does not depend on the order; keys are unique by slot)
      const uint32_t m = cnt[tid];
      if (m > 0 && q0 + tid < a.nq) {
        uint64_t* h = heap + tid;
        for (uint32_t c = 0; c < m; ++c) {
          const uint64_t key = make_key(cd[tid * VT + c], v0 + cr[tid * VT + c]);
          if (key < worst) {
            heap_replace_root(h, (int)k, QT, key);
            worst = h[0];
          }
        }
        wq[tid] = worst;
      }
      cnt[tid] = 0;
    }
  }
  __syncthreads();

  if (tid < QT && q0 + tid < a.nq) {
    uint64_t* h = heap + tid;
    const uint32_t q = q0 + tid;
    if (a.splits == 1) {
      heap_sort_ascending(h, (int)k, QT);
      for (uint32_t r = 0; r < k; ++r) a.out[(size_t)q * k + r] = key_to_result(h[r * QT], a.vec_ids);
    } else {
      uint64_t* dst = a.partial + ((size_t)q * a.splits + blockIdx.y) * k;
      for (uint32_t r = 0; r < k; ++r) dst[r] = h[r * QT];
    }
  }
}

}  // namespace

// Merges `lists` unsorted candidate lists of `k` keys per query into the
// ascending top-k; one CTA per query, bitonic sort in shared memory.
__global__ void __launch_bounds__(256) merge_partial_topk_kernel(const uint64_t* __restrict__ partial, uint32_t lists,
                                                                 uint32_t k, uint32_t pow2, const uint32_t* vec_ids,
                                                                 GpuSearchResult* __restrict__ out, uint32_t out_k) {
  extern __shared__ uint64_t keys[];
  const uint32_t q = blockIdx.x;
  const uint32_t total = lists * k;
  const uint64_t* src = partial + (size_t)q * total;
  for (uint32_t i = threadIdx.x; i < pow2; i += blockDim.x) keys[i] = i < total ? src[i] : kSentinelKey;
  __syncthreads();
  block_bitonic_sort(keys, pow2);
  for (uint32_t r = threadIdx.x; r < out_k; r += blockDim.x) out[(size_t)q * out_k + r] = key_to_result(keys[r], vec_ids);
}

size_t flat_f32_smem_bytes(uint32_t k) {
  size_t floats = (size_t)DK * QS + (size_t)DK * VS + (size_t)QT * VT + QT + VT;
  size_t bytes = floats * 4;
  bytes = (bytes + 7) & ~(size_t)7;
  // heaps | k-th keys | candidate counts | candidate rows
  return bytes + (size_t)k * QT * 8 + QT * 8 + QT * 4 + (size_t)QT * VT;
}

FlatPlan plan_flat_f32(uint32_t n, uint32_t nq, uint32_t k, uint32_t forced_splits) {
  const uint32_t nqb = (nq + QT - 1) / QT;
  const uint32_t ntiles = (n + VT - 1) / VT;
  int sms = device_sm_count();
  const uint32_t pow2k = next_pow2(k);
  const uint32_t smax = std::max(1u, std::min(ntiles, 8192u / pow2k));  // merge sorts splits * k keys
  uint32_t splits = forced_splits;
  if (!splits) {
    // two CTAs per SM: the fewest splits that give every slot a CTA, or a
    // few more when that fills the last wave better (a query block count
    // just above the slot count otherwise leaves a nearly empty wave)
    const uint64_t slots = 2ull * (uint64_t)sms;
    const uint32_t s0 = (uint32_t)std::max<uint64_t>(1, (slots + nqb - 1) / nqb);
    auto fullness = [&](uint32_t sp) {
      const uint64_t ctas = (uint64_t)nqb * sp, waves = (ctas + slots - 1) / slots;
      return (double)ctas / (double)(waves * slots);
    };
    splits = std::min(s0, smax);
    double best = fullness(splits);
    for (uint32_t sp = splits + 1; sp <= std::min(std::max(2 * s0, 8u), smax); ++sp) {
      const double f = fullness(sp);
      if (f > best + 0.01) {
        best = f;
        splits = sp;
      }
    }
  }
  splits = std::max(1u, std::min(splits, smax));
  uint32_t tps = (ntiles + splits - 1) / splits;
  splits = (ntiles + tps - 1) / tps;
  FlatPlan p;
  p.splits = splits;
  p.tiles_per_split = tps;
  p.scratch_bytes = splits > 1 ? (size_t)nq * splits * k * 8 : 0;
  return p;
}

int launch_flat_f32(const float* vectors, const uint32_t* vec_ids, uint32_t n, uint32_t dim, const float* queries,
                    uint32_t nq, uint32_t k, MetricType metric, const uint32_t* mask, GpuSearchResult* out,
                    uint32_t forced_splits, cudaStream_t stream, const QueryFilter* filters) {
  const FlatPlan p = plan_flat_f32(n, nq, k, forced_splits);
  void* scratch = nullptr;
  if (p.scratch_bytes) {
    scratch = scratch_get(stream, p.scratch_bytes);
    if (!scratch) return (int)cudaErrorMemoryAllocation;
  }
  return launch_flat_f32_planned(p, vectors, vec_ids, n, dim, queries, nq, k, metric, mask, out, false, scratch,
                                 stream, filters);
}

int launch_flat_f32_planned(const FlatPlan& p, const float* vectors, const uint32_t* vec_ids, uint32_t n,
                            uint32_t dim, const float* queries, uint32_t nq, uint32_t k, MetricType metric,
                            const uint32_t* mask, GpuSearchResult* out, bool fused, void* scratch,
                            cudaStream_t stream, const QueryFilter* filters) {
  const uint32_t nqb = (nq + QT - 1) / QT;
  const uint32_t splits = p.splits, tps = p.tiles_per_split;
  FlatArgs a{vectors, vec_ids, n, dim, queries, nq, k, mask, out, static_cast<uint64_t*>(scratch), splits, tps,
             filters};
  if (splits > 1 && !a.partial) return (int)cudaErrorMemoryAllocation;

  const size_t smem = flat_f32_smem_bytes(k);
  const bool vec4 = (dim % 4 == 0) && ((uintptr_t)vectors % 16 == 0) && ((uintptr_t)queries % 16 == 0);
  dim3 grid(nqb, splits);
  auto go = [&](auto kern) {
    cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    kern<<<grid, NT, smem, stream>>>(a);
  };
  ProfScope ps(fused ? "coarse_f32_scan" : "flat_f32_scan", stream);
  if (fused) {
    vec4 ? go(flat_f32_scan_kernel<METRIC_L2, true, true>) : go(flat_f32_scan_kernel<METRIC_L2, false, true>);
  } else {
    switch (metric) {
      case METRIC_INNER_PRODUCT:
        vec4 ? go(flat_f32_scan_kernel<METRIC_INNER_PRODUCT, true>)
             : go(flat_f32_scan_kernel<METRIC_INNER_PRODUCT, false>);
        break;
      case METRIC_COSINE:
        vec4 ? go(flat_f32_scan_kernel<METRIC_COSINE, true>) : go(flat_f32_scan_kernel<METRIC_COSINE, false>);
        break;
      default:
        vec4 ? go(flat_f32_scan_kernel<METRIC_L2, true>) : go(flat_f32_scan_kernel<METRIC_L2, false>);
        break;
    }
  }
  note_launch();
  if (splits > 1) {
    const uint32_t pow2 = next_pow2(splits * k);
    const size_t msmem = (size_t)pow2 * 8;
    cudaFuncSetAttribute(merge_partial_topk_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)msmem);
    merge_partial_topk_kernel<<<nq, 256, msmem, stream>>>(a.partial, splits, k, pow2, vec_ids, out, k);
    note_launch();
  }
  return (int)cudaGetLastError();
}


// ===========================================================================
// Allocation-free variant of the exact flat scan.
//
// Some callers of this library cannot call cudaMalloc: code that runs while
// another thread is capturing a CUDA graph in global capture mode (where an
// allocation is an illegal call), latency-critical serving threads that
// must not take the allocator's locks or risk its implicit device
// synchronisation, and hosts that hand all device memory to one pool of
// their own. For them fv_flat_scan_batch_noalloc keeps the per-split heaps
// of the scan in the fixed array below instead of the per-stream arena.
//
// The array is a file-scope device variable: every GPU that loads this
// library holds its kNoAllocScratchBytes until the process exits. In host
// code its name is only a host-side stand-in, not a device address, so the
// address handed to the kernels is looked up once per device with
// cudaGetSymbolAddress (with that device current) on the first call made
// on the device; make that first call before any stream capture begins.
// The looked-up address is kept for the life of the process: after a
// cudaDeviceReset the array may sit elsewhere in the new context, so a
// process that resets a device must not call this entry point on it again.
// All calls share the one array and it keeps whatever the last call wrote;
// the scan writes every slot it later reads, so nothing needs clearing, but
// calls whose work overlaps on the GPU (different streams, or host threads
// racing on one device) overwrite each other's heaps -- serialise them.
// ===========================================================================
namespace {
constexpr size_t kNoAllocScratchBytes = 8u << 20;  // 8 MiB per device
static __device__ __align__(256) uint64_t g_flat_noalloc_scratch[kNoAllocScratchBytes / 8];

constexpr int kMaxDevices = 64;
std::mutex g_noalloc_mu;
uint64_t* g_noalloc_addr[kMaxDevices] = {};

cudaError_t noalloc_scratch_address(uint64_t** out) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  if (dev < 0 || dev >= kMaxDevices) return cudaErrorInvalidDevice;
  std::lock_guard<std::mutex> lk(g_noalloc_mu);
  if (!g_noalloc_addr[dev]) {
    void* p = nullptr;
    e = cudaGetSymbolAddress(&p, g_flat_noalloc_scratch);
    if (e != cudaSuccess) return e;
    g_noalloc_addr[dev] = static_cast<uint64_t*>(p);
  }
  *out = g_noalloc_addr[dev];
  return cudaSuccess;
}
}  // namespace

// Same work split and kernels as launch_flat_f32, with the per-split heaps
// in the fixed array; refuses (FV_ERR_SCRATCH_LIMIT) a call whose heaps
// would not fit instead of allocating.
int launch_flat_f32_noalloc(const float* vectors, const uint32_t* vec_ids, uint32_t n, uint32_t dim,
                            const float* queries, uint32_t nq, uint32_t k, MetricType metric, const uint32_t* mask,
                            GpuSearchResult* out, cudaStream_t stream) {
  const FlatPlan p = plan_flat_f32(n, nq, k, 0);
  if (p.scratch_bytes > kNoAllocScratchBytes) return FV_ERR_SCRATCH_LIMIT;
  uint64_t* heaps = nullptr;
  if (p.scratch_bytes) {
    cudaError_t e = noalloc_scratch_address(&heaps);
    if (e != cudaSuccess) return (int)e;
  }
  return launch_flat_f32_planned(p, vectors, vec_ids, n, dim, queries, nq, k, metric, mask, out, false, heaps,
                                 stream);
}

}  // namespace fv

extern "C" int fv_flat_scan_batch_noalloc(const float* d_vectors, const uint32_t* d_vec_ids, uint32_t num_vectors,
                                          uint32_t dim, const float* d_queries, uint32_t num_queries, uint32_t top_k,
                                          MetricType metric, const uint32_t* d_valid_mask,
                                          GpuSearchResult* d_out_results, void* stream) {
  if (!d_queries || !d_out_results) return -1;
  if (num_vectors > 0 && !d_vectors) return -1;
  if (num_queries == 0 || top_k == 0) return 0;
  if (top_k > (uint32_t)fv::kMaxTopK) top_k = fv::kMaxTopK;
  cudaStream_t s = (cudaStream_t)stream;
  if (num_vectors == 0)
    return (int)cudaMemsetAsync(d_out_results, 0xFF, (size_t)num_queries * top_k * sizeof(GpuSearchResult), s);
  if (dim == 0) return -2;
  return fv::launch_flat_f32_noalloc(d_vectors, d_vec_ids, num_vectors, dim, d_queries, num_queries, top_k, metric,
                                     d_valid_mask, d_out_results, s);
}

