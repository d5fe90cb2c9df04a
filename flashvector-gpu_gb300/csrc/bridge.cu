// bridge.cu -- the C ABI of libfvgb300: device / memory / stream plumbing,
// argument validation and clamps of the drop-in search entry points, the
// per-stream scratch arena, the device status word and the launch counter.
//
// Plumbing functions replace hnsw_traverse.cu:525-637 one for one (same
// CUDA calls, same null/zero-size handling); the search entry points keep
// the reference's validation order and clamps (sparse_hybrid.cu:96-101,
// 517-518).
#include <atomic>
#include <map>
#include <mutex>
#include <string>
#include <unordered_map>
#include <vector>
#include <cstdio>
#include <cstring>

#include "../../include/fv_bridge.h"
#include "common.cuh"
#include "kernels.h"

namespace fv {

// ------------------------------------------------------------- tuning
namespace {
struct Knob {
  const char* key;
  std::atomic<int64_t> value;
};
Knob g_knobs[] = {{"tc.prepass", {-1}}, {"tc.prepass_stride", {0}}, {"tc.prepass_margin", {0}}, {"tc.pair", {-1}},
                  {"tc.table", {1}}, {"ivf.pipeline", {-1}}, {"ivf.split", {-1}}, {"ivf.compact", {1}},
                  {"ivf.tc_coarse", {-1}}, {"tc.wait_limit_ns", {0}}, {"tc.groups", {-1}}};
}  // namespace

bool tune_set(const char* key, int64_t value) {
  for (auto& k : g_knobs)
    if (std::strcmp(k.key, key) == 0) {
      k.value.store(value, std::memory_order_relaxed);
      return true;
    }
  return false;
}

bool tune_get(const char* key, int64_t* value) {
  for (auto& k : g_knobs)
    if (std::strcmp(k.key, key) == 0) {
      *value = k.value.load(std::memory_order_relaxed);
      return true;
    }
  return false;
}

int64_t tune_value(const char* key, int64_t dflt) {
  int64_t v = dflt;
  return tune_get(key, &v) ? v : dflt;
}

}  // namespace fv

namespace fv {

namespace {
std::atomic<uint64_t> g_launches{0};

struct Arena {
  void* ptr = nullptr;
  size_t bytes = 0;
  bool owned = true;
};
std::mutex g_arena_mu;
// keyed by (device, stream)
std::unordered_map<uint64_t, Arena> g_arenas;

uint64_t arena_key(cudaStream_t s) {
  int dev = 0;
  cudaGetDevice(&dev);
  return (uint64_t)(uintptr_t)s * 64u + (uint64_t)dev;
}

std::mutex g_dev_mu;
std::vector<int> g_sm_counts;
std::vector<uint32_t*> g_status;
}  // namespace

void note_launch(uint32_t n) { g_launches.fetch_add(n, std::memory_order_relaxed); }

namespace {
std::atomic<bool> g_prof_on{false};
std::mutex g_prof_mu;
std::vector<cudaEvent_t> g_prof_free;
struct ProfRec {
  std::string name;
  cudaEvent_t a, b;
};
std::vector<ProfRec> g_prof_pending;
}  // namespace

bool profiling_enabled() { return g_prof_on.load(std::memory_order_relaxed); }

cudaEvent_t profile_event() {
  std::lock_guard<std::mutex> lk(g_prof_mu);
  if (!g_prof_free.empty()) {
    cudaEvent_t e = g_prof_free.back();
    g_prof_free.pop_back();
    return e;
  }
  cudaEvent_t e = nullptr;
  cudaEventCreate(&e);
  return e;
}

void profile_record(const char* name, cudaEvent_t a, cudaEvent_t b) {
  std::lock_guard<std::mutex> lk(g_prof_mu);
  g_prof_pending.push_back({name, a, b});
}

int device_sm_count() {
  int dev = 0;
  cudaGetDevice(&dev);
  std::lock_guard<std::mutex> lk(g_dev_mu);
  if ((int)g_sm_counts.size() <= dev) g_sm_counts.resize(dev + 1, 0);
  if (g_sm_counts[dev] == 0) {
    int n = 0;
    cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
    g_sm_counts[dev] = n > 0 ? n : 1;
  }
  return g_sm_counts[dev];
}

uint32_t* status_word() {
  int dev = 0;
  cudaGetDevice(&dev);
  std::lock_guard<std::mutex> lk(g_dev_mu);
  if ((int)g_status.size() <= dev) g_status.resize(dev + 1, nullptr);
  if (!g_status[dev]) {
    uint32_t* p = nullptr;
    if (cudaMalloc(&p, sizeof(uint32_t)) != cudaSuccess) return nullptr;
    cudaMemset(p, 0, sizeof(uint32_t));
    g_status[dev] = p;
  }
  return g_status[dev];
}

void* scratch_get(cudaStream_t stream, size_t bytes) {
  if (bytes == 0) bytes = 256;
  bytes = (bytes + 255) & ~(size_t)255;
  std::lock_guard<std::mutex> lk(g_arena_mu);
  Arena& a = g_arenas[arena_key(stream)];
  if (a.bytes >= bytes) return a.ptr;
  if (!a.owned) return nullptr;  // caller-provided arena too small: refuse
  if (a.ptr) cudaFreeAsync(a.ptr, stream);
  a.ptr = nullptr;
  a.bytes = 0;
  size_t grow = bytes + bytes / 4;
  if (cudaMallocAsync(&a.ptr, grow, stream) != cudaSuccess) {
    cudaGetLastError();
    a.ptr = nullptr;
    return nullptr;
  }
  a.bytes = grow;
  return a.ptr;
}

}  // namespace fv

using fv::note_launch;

extern "C" {

// ---------------------------------------------------------------- plumbing
int cuda_init_device(int device_id) {
  cudaError_t e = cudaSetDevice(device_id);
  if (e != cudaSuccess) return (int)e;
  return (int)cudaFree(0);
}
int cuda_set_device(int device_id) { return (int)cudaSetDevice(device_id); }
int cuda_get_device_count(int* count) {
  if (!count) return FV_ERR_NULL;
  return (int)cudaGetDeviceCount(count);
}
int cuda_get_device_memory(size_t* free_bytes, size_t* total_bytes) {
  if (!free_bytes || !total_bytes) return FV_ERR_NULL;
  return (int)cudaMemGetInfo(free_bytes, total_bytes);
}
int cuda_device_synchronize(void) { return (int)cudaDeviceSynchronize(); }
int cuda_malloc_device(void** ptr, size_t bytes) {
  if (!ptr || bytes == 0) return FV_ERR_NULL;
  return (int)cudaMalloc(ptr, bytes);
}
int cuda_free_device(void* ptr) { return ptr ? (int)cudaFree(ptr) : 0; }
int cuda_malloc_host(void** ptr, size_t bytes) {
  if (!ptr || bytes == 0) return FV_ERR_NULL;
  return (int)cudaHostAlloc(ptr, bytes, cudaHostAllocMapped);
}
int cuda_free_host(void* ptr) { return ptr ? (int)cudaFreeHost(ptr) : 0; }
int cuda_memcpy_h2d_async(void* dst, const void* src, size_t bytes, void* stream) {
  if (!dst || !src) return FV_ERR_NULL;
  if (bytes == 0) return 0;
  return (int)cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, (cudaStream_t)stream);
}
int cuda_memcpy_d2h_async(void* dst, const void* src, size_t bytes, void* stream) {
  if (!dst || !src) return FV_ERR_NULL;
  if (bytes == 0) return 0;
  return (int)cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToHost, (cudaStream_t)stream);
}
int cuda_memset_device_async(void* dst, int value, size_t bytes, void* stream) {
  if (!dst) return FV_ERR_NULL;
  if (bytes == 0) return 0;
  return (int)cudaMemsetAsync(dst, value, bytes, (cudaStream_t)stream);
}
int cuda_host_get_device_pointer(void** dev_ptr, void* host_ptr) {
  if (!dev_ptr || !host_ptr) return FV_ERR_NULL;
  return (int)cudaHostGetDevicePointer(dev_ptr, host_ptr, 0);
}
int cuda_create_stream(void** stream) {
  if (!stream) return FV_ERR_NULL;
  return (int)cudaStreamCreateWithFlags((cudaStream_t*)stream, cudaStreamNonBlocking);
}
int cuda_destroy_stream(void* stream) {
  if (!stream) return 0;
  {
    std::lock_guard<std::mutex> lk(fv::g_arena_mu);
    auto it = fv::g_arenas.find(fv::arena_key((cudaStream_t)stream));
    if (it != fv::g_arenas.end()) {
      if (it->second.owned && it->second.ptr) cudaFreeAsync(it->second.ptr, (cudaStream_t)stream);
      fv::g_arenas.erase(it);
    }
  }
  return (int)cudaStreamDestroy((cudaStream_t)stream);
}
int cuda_sync_stream(void* stream) {
  if (!stream) return (int)cudaDeviceSynchronize();
  return (int)cudaStreamSynchronize((cudaStream_t)stream);
}

// ------------------------------------------------------------ flat scan
int cuda_flat_scan_batch(const float* d_vectors, const uint32_t* d_vec_ids, uint32_t num_vectors, uint32_t dim,
                         const float* d_queries, uint32_t num_queries, uint32_t top_k, MetricType metric,
                         const uint32_t* d_valid_mask, GpuSearchResult* d_out_results, void* stream) {
  if (!d_queries || !d_out_results) return FV_ERR_NULL;
  if (num_vectors > 0 && !d_vectors) return FV_ERR_NULL;
  if (num_queries == 0 || top_k == 0) return 0;
  if (top_k > (uint32_t)fv::kMaxTopK) top_k = fv::kMaxTopK;
  cudaStream_t s = (cudaStream_t)stream;
  if (num_vectors == 0) {
    // the reference fills the outputs with 0xFF bytes here (ids 0xFFFFFFFF,
    // distance bits 0xFFFFFFFF), not with the 1e30 sentinel
    return (int)cudaMemsetAsync(d_out_results, 0xFF, (size_t)num_queries * top_k * sizeof(GpuSearchResult), s);
  }
  if (dim == 0) return FV_ERR_ARG;
  return fv::launch_flat_f32(d_vectors, d_vec_ids, num_vectors, dim, d_queries, num_queries, top_k, metric,
                             d_valid_mask, d_out_results, 0, s);
}

// -------------------------------------------------- tensor-core scans
namespace {
int tc_common(const fv::TcTables& t, const float* q, uint32_t nq, uint32_t top_k, MetricType metric,
              const uint32_t* mask, const FvScanOptions* opt, GpuSearchResult* out, void* stream) {
  if (nq == 0 || top_k == 0) return 0;
  if (top_k > (uint32_t)fv::kMaxTopK) top_k = fv::kMaxTopK;
  cudaStream_t s = (cudaStream_t)stream;
  if (t.n == 0) {
    // no rows: every slot is the {0xFFFFFFFF, 1e30} sentinel
    return fv::launch_fill_sentinel(out, (size_t)nq * top_k, s);
  }
  if (!t.base) return FV_ERR_NULL;
  if (t.dim == 0 || t.padded_dim < t.dim || t.padded_dim % 16 != 0) return FV_ERR_ARG;
  if ((uintptr_t)t.base % 16 != 0) return FV_ERR_ARG;
  if (metric != METRIC_INNER_PRODUCT && !t.norms) return FV_ERR_NULL;
  if (t.fp8 && !t.scales) return FV_ERR_NULL;
  if (t.fp8 && t.fp8_table_scale && t.padded_dim < t.dim + 3) return FV_ERR_ARG;  // room for the norm digits
  if (t.fp8 && !t.fp8_table_scale && metric != METRIC_INNER_PRODUCT && !t.norms) return FV_ERR_NULL;
  FvScanOptions o{};
  if (opt) o = *opt;
  else o.boundary_fp64 = 1;
  return fv::launch_tc_scan(t, q, nq, top_k, metric, mask, out, o, s);
}
}  // namespace

int cuda_fp16_tc_search_batch(const Fp16GpuTables* tables, const float* d_queries, uint32_t num_queries,
                              uint32_t top_k, MetricType metric, const uint32_t* d_valid_mask,
                              GpuSearchResult* d_out_results, void* stream) {
  if (!tables || !d_queries || !d_out_results) return FV_ERR_NULL;
  fv::TcTables t{false, tables->d_vectors_fp16, tables->d_vec_norms_sq, nullptr, tables->d_vectors,
                 tables->num_vectors, tables->dim, tables->padded_dim};
  return tc_common(t, d_queries, num_queries, top_k, metric, d_valid_mask, nullptr, d_out_results, stream);
}

int fv_fp16_search_batch_ex(const Fp16GpuTables* tables, const float* d_queries, uint32_t num_queries,
                            uint32_t top_k, MetricType metric, const uint32_t* d_valid_mask,
                            const FvScanOptions* options, GpuSearchResult* d_out_results, void* stream) {
  if (!tables || !d_queries || !d_out_results) return FV_ERR_NULL;
  fv::TcTables t{false, tables->d_vectors_fp16, tables->d_vec_norms_sq, nullptr, tables->d_vectors,
                 tables->num_vectors, tables->dim, tables->padded_dim};
  return tc_common(t, d_queries, num_queries, top_k, metric, d_valid_mask, options, d_out_results, stream);
}

int fv_fp8_search_batch(const FvFp8GpuTables* tables, const float* d_queries, uint32_t num_queries, uint32_t top_k,
                        MetricType metric, const uint32_t* d_valid_mask, const FvScanOptions* options,
                        GpuSearchResult* d_out_results, void* stream) {
  if (!tables || !d_queries || !d_out_results) return FV_ERR_NULL;
  if (tables->scale_mode > 1u) return FV_ERR_ARG;
  fv::TcTables t{true, tables->d_vectors_fp8, tables->d_vec_norms_sq, tables->d_scales, tables->d_vectors,
                 tables->num_vectors, tables->dim, tables->padded_dim, tables->scale_mode == 0u};
  return tc_common(t, d_queries, num_queries, top_k, metric, d_valid_mask, options, d_out_results, stream);
}

int fv_encode_fp16_padded(const float* d_vectors, uint32_t num_vectors, uint32_t dim, uint32_t padded_dim,
                          uint16_t* d_out_fp16, float* d_out_norms_sq, void* stream) {
  if (num_vectors && (!d_vectors || !d_out_fp16)) return FV_ERR_NULL;
  if (padded_dim < dim || padded_dim % 16) return FV_ERR_ARG;
  return fv::launch_encode_fp16(d_vectors, num_vectors, dim, padded_dim, d_out_fp16, d_out_norms_sq,
                                (cudaStream_t)stream);
}

int fv_encode_fp8(const float* d_vectors, uint32_t num_vectors, uint32_t dim, uint32_t padded_dim,
                  uint8_t* d_out_fp8, float* d_out_scales, float* d_out_norms_sq, void* stream) {
  if (num_vectors && (!d_vectors || !d_out_fp8 || !d_out_scales || !d_out_norms_sq)) return FV_ERR_NULL;
  if (padded_dim < dim + 3 || padded_dim % 16) return FV_ERR_ARG;
  return fv::launch_encode_fp8(d_vectors, num_vectors, dim, padded_dim, d_out_fp8, d_out_scales, d_out_norms_sq,
                               (cudaStream_t)stream);
}

int fv_encode_fp8_per_vector(const float* d_vectors, uint32_t num_vectors, uint32_t dim, uint32_t padded_dim,
                             uint8_t* d_out_fp8, float* d_out_scales, float* d_out_norms_sq, void* stream) {
  if (num_vectors && (!d_vectors || !d_out_fp8 || !d_out_scales || !d_out_norms_sq)) return FV_ERR_NULL;
  if (padded_dim < dim || padded_dim % 16) return FV_ERR_ARG;
  return fv::launch_encode_fp8_per_vector(d_vectors, num_vectors, dim, padded_dim, d_out_fp8, d_out_scales,
                                          d_out_norms_sq, (cudaStream_t)stream);
}

// ------------------------------------------------------------------ IVF
namespace {
int ivf_pq(const IvfPqGpuTables* t, const FvIvfOptions* o, const float* q, uint32_t nq, uint32_t top_k,
           uint32_t nprobe, uint32_t rerank_k, MetricType metric, const uint32_t* mask, GpuSearchResult* out,
           void* stream) {
  if (!t || !q || !out) return FV_ERR_NULL;
  if (nq == 0 || top_k == 0 || t->m_pq == 0 || t->nlist == 0) return 0;
  if (!t->d_centroids || !t->d_pq_codebooks || !t->d_pq_codes || !t->d_ivf_offsets || !t->d_ivf_vec_ids)
    return FV_ERR_NULL;
  fv::IvfLaunch L{t->d_centroids, t->d_pq_codebooks, nullptr, nullptr, t->d_pq_codes, t->d_ivf_offsets,
                  t->d_ivf_vec_ids, t->d_vectors, t->num_vectors, t->dim, t->nlist, t->m_pq, t->sub_dim,
                  o && o->codes_list_major, q, nq, top_k, nprobe, rerank_k, metric, mask, out};
  return fv::launch_ivf_search(0, L, (cudaStream_t)stream);
}
int ivf_sq(const IvfSqGpuTables* t, const FvIvfOptions* o, const float* q, uint32_t nq, uint32_t top_k,
           uint32_t nprobe, uint32_t rerank_k, MetricType metric, const uint32_t* mask, GpuSearchResult* out,
           void* stream) {
  if (!t || !q || !out) return FV_ERR_NULL;
  if (nq == 0 || top_k == 0 || t->nlist == 0 || t->dim == 0) return 0;
  if (!t->d_centroids || !t->d_sq_mins || !t->d_sq_scales || !t->d_sq_codes || !t->d_ivf_offsets ||
      !t->d_ivf_vec_ids)
    return FV_ERR_NULL;
  fv::IvfLaunch L{t->d_centroids, nullptr, t->d_sq_mins, t->d_sq_scales, t->d_sq_codes, t->d_ivf_offsets,
                  t->d_ivf_vec_ids, t->d_vectors, t->num_vectors, t->dim, t->nlist, 0, 0,
                  o && o->codes_list_major, q, nq, top_k, nprobe, rerank_k, metric, mask, out};
  return fv::launch_ivf_search(1, L, (cudaStream_t)stream);
}
}  // namespace

int cuda_ivf_pq_search_batch(const IvfPqGpuTables* tables, const float* d_queries, uint32_t num_queries,
                             uint32_t top_k, uint32_t nprobe, uint32_t rerank_k, MetricType metric,
                             const uint32_t* d_valid_mask, GpuSearchResult* d_out_results, void* stream) {
  return ivf_pq(tables, nullptr, d_queries, num_queries, top_k, nprobe, rerank_k, metric, d_valid_mask,
                d_out_results, stream);
}
int cuda_ivf_sq_search_batch(const IvfSqGpuTables* tables, const float* d_queries, uint32_t num_queries,
                             uint32_t top_k, uint32_t nprobe, uint32_t rerank_k, MetricType metric,
                             const uint32_t* d_valid_mask, GpuSearchResult* d_out_results, void* stream) {
  return ivf_sq(tables, nullptr, d_queries, num_queries, top_k, nprobe, rerank_k, metric, d_valid_mask,
                d_out_results, stream);
}
int fv_ivf_pq_search_ex(const IvfPqGpuTables* tables, const FvIvfOptions* options, const float* d_queries,
                        uint32_t num_queries, uint32_t top_k, uint32_t nprobe, uint32_t rerank_k, MetricType metric,
                        const uint32_t* d_valid_mask, GpuSearchResult* d_out_results, void* stream) {
  return ivf_pq(tables, options, d_queries, num_queries, top_k, nprobe, rerank_k, metric, d_valid_mask,
                d_out_results, stream);
}
int fv_ivf_sq_search_ex(const IvfSqGpuTables* tables, const FvIvfOptions* options, const float* d_queries,
                        uint32_t num_queries, uint32_t top_k, uint32_t nprobe, uint32_t rerank_k, MetricType metric,
                        const uint32_t* d_valid_mask, GpuSearchResult* d_out_results, void* stream) {
  return ivf_sq(tables, options, d_queries, num_queries, top_k, nprobe, rerank_k, metric, d_valid_mask,
                d_out_results, stream);
}
namespace {
int ivf_rabitq(const IvfRabitqGpuTables* t, const FvIvfOptions* o, const float* q, uint32_t nq, uint32_t top_k,
               uint32_t nprobe, uint32_t rerank_k, MetricType metric, const uint32_t* mask, GpuSearchResult* out,
               void* stream) {
  if (!t || !q || !out) return FV_ERR_NULL;
  if (nq == 0 || top_k == 0 || t->nlist == 0 || t->padded_dim == 0) return 0;
  if (!t->d_centroids || !t->d_rot_centroids || !t->d_rabitq_bits || !t->d_rabitq_meta || !t->d_rot_signs ||
      !t->d_ivf_offsets || !t->d_ivf_vec_ids)
    return FV_ERR_NULL;
  if (t->words_per_vec * 32 != t->padded_dim) return FV_ERR_ARG;
  fv::IvfLaunch L{};
  L.centroids = t->d_centroids;
  L.offsets = t->d_ivf_offsets;
  L.vec_ids = t->d_ivf_vec_ids;
  L.vectors = t->d_vectors;
  L.num_vectors = t->num_vectors;
  L.dim = t->dim;
  L.nlist = t->nlist;
  L.list_major = o && o->codes_list_major;
  L.queries = q;
  L.nq = nq;
  L.top_k = top_k;
  L.nprobe = nprobe;
  L.rerank_k = rerank_k;
  L.metric = metric;
  L.mask = mask;
  L.out = out;
  L.rot_centroids = t->d_rot_centroids;
  L.rq_bits = t->d_rabitq_bits;
  L.rq_meta = t->d_rabitq_meta;
  L.rot_signs = t->d_rot_signs;
  L.padded_dim = t->padded_dim;
  return fv::launch_ivf_search(fv::IVF_MODE_RABITQ, L, (cudaStream_t)stream);
}
}  // namespace

int cuda_ivf_rabitq_search_batch(const IvfRabitqGpuTables* tables, const float* d_queries, uint32_t num_queries,
                                 uint32_t top_k, uint32_t nprobe, uint32_t rerank_k, MetricType metric,
                                 const uint32_t* d_valid_mask, GpuSearchResult* d_out_results, void* stream) {
  return ivf_rabitq(tables, nullptr, d_queries, num_queries, top_k, nprobe, rerank_k, metric, d_valid_mask,
                    d_out_results, stream);
}
int fv_ivf_rabitq_search_ex(const IvfRabitqGpuTables* tables, const FvIvfOptions* options, const float* d_queries,
                            uint32_t num_queries, uint32_t top_k, uint32_t nprobe, uint32_t rerank_k,
                            MetricType metric, const uint32_t* d_valid_mask, GpuSearchResult* d_out_results,
                            void* stream) {
  return ivf_rabitq(tables, options, d_queries, num_queries, top_k, nprobe, rerank_k, metric, d_valid_mask,
                    d_out_results, stream);
}
int fv_ivf_relayout_codes(const uint8_t* d_codes_by_id, const uint32_t* d_ivf_vec_ids, uint32_t num_vectors,
                          uint32_t row_bytes, uint8_t* d_out_by_list, void* stream) {
  if (num_vectors && (!d_codes_by_id || !d_ivf_vec_ids || !d_out_by_list)) return FV_ERR_NULL;
  return fv::launch_relayout_codes(d_codes_by_id, d_ivf_vec_ids, num_vectors, row_bytes, d_out_by_list,
                                   (cudaStream_t)stream);
}

// ---------------------------------------------------------- index build
int fv_build_pq_encode(const float* d_residuals, uint32_t num_vectors, uint32_t dim, uint32_t m_pq,
                       const float* d_codebooks, uint8_t* d_out_codes, void* stream) {
  if (num_vectors && (!d_residuals || !d_codebooks || !d_out_codes)) return FV_ERR_NULL;
  if (num_vectors == 0) return 0;
  return fv::launch_pq_encode(d_residuals, num_vectors, dim, m_pq, d_codebooks, d_out_codes, (cudaStream_t)stream);
}
int fv_build_sq8(const float* d_residuals, uint32_t num_vectors, uint32_t dim, float* d_out_mins,
                 float* d_out_scales, uint8_t* d_out_codes, void* stream) {
  if (!d_residuals || !d_out_mins || !d_out_scales || (num_vectors && !d_out_codes)) return FV_ERR_NULL;
  cudaStream_t s = (cudaStream_t)stream;
  uint32_t* work = static_cast<uint32_t*>(fv::scratch_get(s, (size_t)dim * 8));
  if (!work) return (int)cudaErrorMemoryAllocation;
  int rc = fv::launch_sq8_fit(d_residuals, num_vectors, dim, d_out_mins, d_out_scales, work, s);
  if (rc || num_vectors == 0) return rc;
  return fv::launch_sq8_encode(d_residuals, num_vectors, dim, d_out_mins, d_out_scales, d_out_codes, s);
}
int fv_build_ivf_lists(const GpuSearchResult* d_assign, uint32_t num_vectors, uint32_t nlist, uint32_t* d_out_offsets,
                       uint32_t* d_out_vec_ids, void* stream) {
  if (!d_out_offsets || (num_vectors && (!d_assign || !d_out_vec_ids))) return FV_ERR_NULL;
  if (nlist == 0) return FV_ERR_ARG;
  cudaStream_t s = (cudaStream_t)stream;
  uint32_t* work = static_cast<uint32_t*>(fv::scratch_get(s, (size_t)nlist * 4));
  if (!work) return (int)cudaErrorMemoryAllocation;
  return fv::launch_build_lists(d_assign, num_vectors, nlist, d_out_offsets, d_out_vec_ids, work, s);
}

uint32_t fv_rabitq_padded_dim(uint32_t dim) { return fv::rabitq_padded_dim(dim); }

void fv_rabitq_rot_signs(uint32_t padded_dim, uint64_t seed, float* host_out) {
  if (host_out) fv::rabitq_rot_signs(padded_dim, seed, host_out);
}

int fv_build_rabitq(const float* d_vectors, uint32_t num_vectors, uint32_t dim, const float* d_centroids,
                    uint32_t nlist, const GpuSearchResult* d_assign, const float* d_rot_signs, uint32_t padded_dim,
                    float* d_out_rot_centroids, uint32_t* d_out_bits, float* d_out_meta, void* stream) {
  if (!d_rot_signs || (nlist && (!d_centroids || !d_out_rot_centroids)) ||
      (num_vectors && (!d_vectors || !d_assign || !d_out_bits || !d_out_meta)))
    return FV_ERR_NULL;
  if (dim == 0) return FV_ERR_ARG;
  return fv::launch_rabitq_encode(d_vectors, num_vectors, dim, d_centroids, nlist, d_assign, d_rot_signs, padded_dim,
                                  d_out_rot_centroids, d_out_bits, d_out_meta, (cudaStream_t)stream);
}

// ------------------------------------------------------------ CUDA graphs
// A captured sequence of this library's calls on one stream, replayed with
// one launch. The captured calls keep their pointers: refill the same input
// buffers (queries, masks) before each replay. Scratch must already be large
// enough when capture starts (make the same call once before capturing), so
// that nothing is allocated inside the capture.
}  // extern "C"

struct FvGraph {
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  size_t kernels = 0;
};

extern "C" {

int fv_graph_begin(void* stream) {
  if (!stream) return FV_ERR_NULL;  // the legacy stream cannot be captured
  return (int)cudaStreamBeginCapture((cudaStream_t)stream, cudaStreamCaptureModeThreadLocal);
}

int fv_graph_end(void* stream, FvGraph** out) {
  if (!stream || !out) return FV_ERR_NULL;
  FvGraph* g = new FvGraph();
  cudaError_t e = cudaStreamEndCapture((cudaStream_t)stream, &g->graph);
  if (e == cudaSuccess) e = cudaGraphInstantiate(&g->exec, g->graph, 0);
  if (e != cudaSuccess) {
    if (g->graph) cudaGraphDestroy(g->graph);
    delete g;
    *out = nullptr;
    return (int)e;
  }
  size_t n = 0;
  cudaGraphGetNodes(g->graph, nullptr, &n);
  std::vector<cudaGraphNode_t> nodes(n);
  if (n) cudaGraphGetNodes(g->graph, nodes.data(), &n);
  for (auto nd : nodes) {
    cudaGraphNodeType t;
    if (cudaGraphNodeGetType(nd, &t) == cudaSuccess && t == cudaGraphNodeTypeKernel) ++g->kernels;
  }
  *out = g;
  return 0;
}

int fv_graph_launch(FvGraph* graph, void* stream) {
  if (!graph) return FV_ERR_NULL;
  cudaError_t e = cudaGraphLaunch(graph->exec, (cudaStream_t)stream);
  if (e == cudaSuccess) fv::note_launch((uint32_t)graph->kernels);
  return (int)e;
}

uint64_t fv_graph_kernel_count(const FvGraph* graph) { return graph ? graph->kernels : 0; }

int fv_graph_destroy(FvGraph* graph) {
  if (!graph) return 0;
  if (graph->exec) cudaGraphExecDestroy(graph->exec);
  if (graph->graph) cudaGraphDestroy(graph->graph);
  delete graph;
  return 0;
}

// ------------------------------------------------------------- fixtures
int cuda_compute_distances_warp(const float* d_queries, const float* d_dataset, uint32_t num_queries,
                                uint32_t num_vectors, uint32_t dim, MetricType metric, float* d_out_distances,
                                void* stream) {
  if (!d_queries || !d_dataset || !d_out_distances) return FV_ERR_NULL;
  return fv::launch_distance_matrix(d_queries, d_dataset, num_queries, num_vectors, dim, metric, d_out_distances,
                                    (cudaStream_t)stream);
}

int cuda_bitonic_sort_test(const float* d_keys_in, const uint32_t* d_vals_in, float* d_keys_out, uint32_t* d_vals_out,
                           uint32_t n, void* stream) {
  if (!d_keys_in || !d_vals_in || !d_keys_out || !d_vals_out) return FV_ERR_NULL;
  return fv::launch_bitonic_test(d_keys_in, d_vals_in, d_keys_out, d_vals_out, n, (cudaStream_t)stream);
}

// ----------------------------------------------------------- extensions
const char* fv_version(void) { return "fvgb300 0.1 sm_103a"; }

int fv_tune_set(const char* key, int64_t value) {
  if (!key) return FV_ERR_NULL;
  return fv::tune_set(key, value) ? 0 : FV_ERR_ARG;
}

int fv_tune_get(const char* key, int64_t* value) {
  if (!key || !value) return FV_ERR_NULL;
  return fv::tune_get(key, value) ? 0 : FV_ERR_ARG;
}

int fv_read_device_status(uint32_t* status) {
  if (!status) return FV_ERR_NULL;
  uint32_t* w = fv::status_word();
  if (!w) return (int)cudaErrorMemoryAllocation;
  cudaError_t e = cudaDeviceSynchronize();
  if (e != cudaSuccess) return (int)e;
  e = cudaMemcpy(status, w, sizeof(uint32_t), cudaMemcpyDeviceToHost);
  if (e != cudaSuccess) return (int)e;
  return (int)cudaMemset(w, 0, sizeof(uint32_t));
}

uint64_t fv_launch_count(void) { return fv::g_launches.load(std::memory_order_relaxed); }

int fv_profile_enable(int on) {
  fv::g_prof_on.store(on != 0);
  return 0;
}

int fv_profile_summary(char* buf, size_t len) {
  if (!buf || len == 0) return FV_ERR_NULL;
  std::vector<fv::ProfRec> recs;
  {
    std::lock_guard<std::mutex> lk(fv::g_prof_mu);
    recs.swap(fv::g_prof_pending);
  }
  std::map<std::string, std::pair<uint64_t, double>> agg;
  int rc = 0;
  for (auto& r : recs) {
    float ms = 0.f;
    cudaError_t e = cudaEventSynchronize(r.b);
    if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, r.a, r.b);
    if (e != cudaSuccess) rc = (int)e;
    auto& slot = agg[r.name];
    slot.first += 1;
    slot.second += ms;
    std::lock_guard<std::mutex> lk(fv::g_prof_mu);
    fv::g_prof_free.push_back(r.a);
    fv::g_prof_free.push_back(r.b);
  }
  std::string out = "{";
  bool first = true;
  for (auto& kv : agg) {
    char item[256];
    snprintf(item, sizeof(item), "%s\"%s\": {\"launches\": %llu, \"ms\": %.6f}", first ? "" : ", ", kv.first.c_str(),
             (unsigned long long)kv.second.first, kv.second.second);
    out += item;
    first = false;
  }
  out += "}";
  if (out.size() + 1 > len) return FV_ERR_ARG;
  memcpy(buf, out.c_str(), out.size() + 1);
  return rc;
}

int fv_set_stream_scratch(void* stream, void* d_ptr, size_t bytes) {
  std::lock_guard<std::mutex> lk(fv::g_arena_mu);
  fv::Arena& a = fv::g_arenas[fv::arena_key((cudaStream_t)stream)];
  if (a.owned && a.ptr) cudaFreeAsync(a.ptr, (cudaStream_t)stream);
  if (d_ptr) {
    a.ptr = d_ptr;
    a.bytes = bytes;
    a.owned = false;
  } else {
    a = fv::Arena{};
  }
  return 0;
}

int fv_release_stream_scratch(void* stream) { return fv_set_stream_scratch(stream, nullptr, 0); }

}  // extern "C"
