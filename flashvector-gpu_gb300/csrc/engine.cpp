// engine.cpp -- host orchestration of the scan path: the reference's
// GpuVectorIndex (crates/engine/src/index.rs:131-2634) restated in C++ for the
// scan engines only (exact flat, fp16 / fp8 tensor core, IVF-PQ, IVF-SQ8).
//
// Mirrors, per reference method:
//   build           index.rs:328-576   (cosine rows normalised on the host,
//                                       normalize_slice_in_place :30-38;
//                                       tables built on the GPU: fp16 / fp8
//                                       encoders, k-means, PQ, SQ8, lists)
//   add_vectors     index.rs:647-694   (live-insert ("delta") buffer, logical
//                                       ids from next_logical_id, device copy
//                                       regrown to the next power of two >= 256)
//   delete_ids      index.rs:583-643   (tombstones; main slots cleared in the
//                                       validity words)
//   batch_search_*  index.rs:1979-2237 (query prep, slot mask = user mask AND
//                                       live, main search on a pooled stream,
//                                       delta flat scan concurrently on the
//                                       delta stream, D2H, stable merge)
//   finish_delta_merge index.rs:1353-1387, build_slot_mask_words :1264-1292,
//   build_delta_mask_words :1294-1316, MetricsTracker metrics.rs:21-97.
// Differences: the batch size is not capped at 1024 and masks are not capped
// at 2M ids (streams.rs:12-20); k-means seeds from a seeded sample rather than
// k-means++, and an empty cluster keeps its centroid.
#include <algorithm>
#include <atomic>
#include <chrono>
#include <cmath>
#include <condition_variable>
#include <cstring>
#include <memory>
#include <mutex>
#include <shared_mutex>
#include <string>
#include <type_traits>
#include <unordered_set>
#include <vector>

#include "../../include/fv_bridge.h"
#include "engine.h"
#include "kernels.h"
#include "snapshot.h"

namespace fv {

namespace {

template <class T>
struct DevBuf {
  T* p = nullptr;
  size_t n = 0;
  DevBuf() = default;
  DevBuf(const DevBuf&) = delete;
  DevBuf& operator=(const DevBuf&) = delete;
  ~DevBuf() { release(); }
  void release() {
    if (p) cudaFree(p);
    p = nullptr;
    n = 0;
  }
  int alloc(size_t count) {
    release();
    if (count == 0) return 0;
    cudaError_t e = cudaMalloc(&p, count * sizeof(T));
    if (e != cudaSuccess) {
      p = nullptr;
      return (int)e;
    }
    n = count;
    return 0;
  }
  int ensure(size_t count) { return count <= n ? 0 : alloc(count); }
  size_t bytes() const { return n * sizeof(T); }
};

template <class T>
struct PinnedBuf {
  T* p = nullptr;
  size_t n = 0;
  ~PinnedBuf() {
    if (p) cudaFreeHost(p);
  }
  int ensure(size_t count) {
    if (count <= n) return 0;
    if (p) cudaFreeHost(p);
    p = nullptr;
    n = 0;
    if (cudaMallocHost(&p, std::max<size_t>(count, 1) * sizeof(T)) != cudaSuccess) return (int)cudaErrorMemoryAllocation;
    n = count;
    return 0;
  }
};

uint64_t splitmix(uint64_t& s) {
  uint64_t z = (s += 0x9E3779B97F4A7C15ull);
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

// the reference's build: fp16 rows and the IVF-PQ, IVF-SQ8 and RaBitQ
// tables (index.rs:404-445)
constexpr uint32_t kDefaultBuild = FV_BUILD_FP16 | FV_BUILD_IVF_PQ | FV_BUILD_IVF_SQ8 | FV_BUILD_IVF_RABITQ;
// RabitqEncoder::encode seed of the engine build (index.rs:435-441)
constexpr uint64_t kRabitqSeed = 0x5F3759DFCAFEBABEull;

// `count` distinct indices of [0, n) (Floyd's algorithm), ascending.
std::vector<uint32_t> sample_rows(uint32_t n, uint32_t count, uint64_t seed) {
  count = std::min(count, n);
  std::unordered_set<uint32_t> pick;
  uint64_t s = seed ^ 0xA5A5A5A5DEADBEEFull;
  for (uint32_t j = n - count; j < n; ++j) {
    const uint32_t t = (uint32_t)(splitmix(s) % ((uint64_t)j + 1));
    if (!pick.insert(t).second) pick.insert(j);
  }
  std::vector<uint32_t> out(pick.begin(), pick.end());
  std::sort(out.begin(), out.end());
  return out;
}

// normalize_slice_in_place (index.rs:30-38)
void normalize_rows(float* v, size_t n, uint32_t dim) {
  for (size_t i = 0; i < n; ++i) {
    float* r = v + i * dim;
    float s = 0.f;
    for (uint32_t d = 0; d < dim; ++d) s = s + r[d] * r[d];
    float norm = std::sqrt(s);
    if (norm < 1e-8f) norm = 1e-8f;
    const float inv = 1.0f / norm;
    for (uint32_t d = 0; d < dim; ++d) r[d] = r[d] * inv;
  }
}

struct Stream {
  cudaStream_t s = nullptr;
  std::mutex mu;
  DevBuf<float> q;
  DevBuf<GpuSearchResult> res;
  DevBuf<uint32_t> mask;
  PinnedBuf<float> hq;
  PinnedBuf<GpuSearchResult> hres;
  cudaEvent_t ready = nullptr;  // queries resident on the device
};

struct Delta {
  std::vector<float> vectors;
  std::vector<uint32_t> ids;
  DevBuf<float> d_vectors;
  DevBuf<uint32_t> d_ids;
  DevBuf<uint32_t> d_mask;
  DevBuf<GpuSearchResult> d_res;
  PinnedBuf<GpuSearchResult> h_res;
  std::vector<uint32_t> live;  // validity words over delta slots (tombstones cleared)
  DevBuf<uint32_t> d_live;
  size_t capacity = 0;
  uint32_t len() const { return (uint32_t)ids.size(); }
};

}  // namespace

class Index {
 public:
  explicit Index(const FvIndexConfig& c) : cfg_(c), start_(std::chrono::steady_clock::now()) {
    if (cfg_.build_flags == 0) cfg_.build_flags = kDefaultBuild;
    if (cfg_.kmeans_iters == 0) cfg_.kmeans_iters = 10;
    if (cfg_.pq_iters == 0) cfg_.pq_iters = 10;
    const uint32_t ns = cfg_.streams ? cfg_.streams : 4;
    streams_.resize(ns);
    // blocking streams: work the caller queued on the legacy default stream
    // (device queries, device rows of a build) is ordered before the
    // engine's work, as with the reference's pool streams
    for (auto& st : streams_) {
      st = std::make_unique<Stream>();
      cudaStreamCreateWithFlags(&st->s, cudaStreamDefault);
      cudaEventCreateWithFlags(&st->ready, cudaEventDisableTiming);
    }
    cudaStreamCreateWithFlags(&delta_stream_, cudaStreamDefault);
  }
  ~Index() {
    cudaDeviceSynchronize();
    for (auto& st : streams_) {
      fv_release_stream_scratch(st->s);
      cudaEventDestroy(st->ready);
      cudaStreamDestroy(st->s);
    }
    fv_release_stream_scratch(delta_stream_);
    cudaStreamDestroy(delta_stream_);
  }

  int build(const float* host, uint32_t n) { return build_from(host, n, false, nullptr); }
  int build_device(const float* d_vectors, uint32_t n, const float* d_init_centroids) {
    return build_from(d_vectors, n, true, d_init_centroids);
  }
  int add(const float* host, uint32_t n, uint32_t* out_ids);
  int remove(const uint32_t* ids, uint32_t n, uint32_t* out_deleted);
  int search(const FvSearchParams& p, const float* q, uint32_t nq, bool device_queries, const uint32_t* user_mask,
             uint32_t mask_words, GpuSearchResult* out);
  void stats(FvLatencyStats* s);
  void info(FvIndexInfo* i);
  int export_ivf(uint32_t what, void* host_out, size_t bytes);
  int tables(IvfPqGpuTables* pq, IvfSqGpuTables* sq, FvIvfOptions* opt);
  int rabitq_tables(IvfRabitqGpuTables* t, FvIvfOptions* opt);

  // served batches (serve.cpp)
  void pin() {
    std::shared_lock<std::shared_mutex> lk(state_mu_);
    pins_.fetch_add(1);
  }
  void unpin() {
    if (pins_.fetch_sub(1) == 1) {
      std::lock_guard<std::mutex> g(pin_mu_);
      pin_cv_.notify_all();
    }
  }
  int launch_batch(const BatchLaunch& b, cudaStream_t s);
  size_t batch_scratch_bytes(const BatchLaunch& b) const;
  int load_snapshot(const snap::File& f, std::string* error);
  int save_snapshot(const char* path, std::string* error);
  uint32_t dim() const { return cfg_.dim; }
  int metric() const { return (int)cfg_.metric; }
  bool built() const { return built_; }
  uint32_t nlist() const { return nlist_; }

 private:
  // called by writers holding state_mu_ exclusively: no new pin can start,
  // wait for the batches in flight to release theirs
  void wait_unpinned() {
    std::unique_lock<std::mutex> g(pin_mu_);
    pin_cv_.wait(g, [&] { return pins_.load() == 0; });
  }
  int upload_delta_live(cudaStream_t s);
  int build_from(const float* src, uint32_t n, bool device, const float* d_init_centroids);
  int build_ivf(cudaStream_t s, const float* d_init_centroids);
  int build_rabitq(const GpuSearchResult* assign, cudaStream_t s);
  // list-major copies of the id-indexed bits / meta (`entries` list positions)
  int rabitq_list_major(uint32_t P, uint32_t entries, cudaStream_t s) {
    int rc = rq_bits_lm_.alloc((size_t)entries * (P / 32));
    if (!rc) rc = rq_meta_lm_.alloc((size_t)entries * 4);
    if (!rc)
      rc = launch_relayout_codes(reinterpret_cast<const uint8_t*>(rq_bits_.p), vec_ids_.p, entries, P / 8,
                                 reinterpret_cast<uint8_t*>(rq_bits_lm_.p), s);
    if (!rc)
      rc = launch_relayout_codes(reinterpret_cast<const uint8_t*>(rq_meta_.p), vec_ids_.p, entries, 16,
                                 reinterpret_cast<uint8_t*>(rq_meta_lm_.p), s);
    return rc;
  }
  int kmeans(const float* d_x, uint32_t n, uint32_t dim, uint32_t k, uint32_t iters, uint64_t seed, float* d_cent,
             cudaStream_t s, const float* d_init = nullptr);
  int assign_rows(const float* d_x, uint32_t n, uint32_t dim, const float* d_cent, uint32_t k, GpuSearchResult* out,
                  cudaStream_t s);
  void slot_mask(const uint32_t* user, uint32_t words, std::vector<uint32_t>& out, bool& use) const;
  void delta_mask(const uint32_t* user, uint32_t words, std::vector<uint32_t>& out, bool& use) const;
  void record(double seconds, uint32_t nq);
  IvfLaunch batch_ivf_launch(const BatchLaunch& b, GpuSearchResult* out) const;
  TcTables tc_tables(bool fp8) const;

  FvIndexConfig cfg_;
  std::vector<std::unique_ptr<Stream>> streams_;
  std::atomic<uint32_t> rr_{0};
  cudaStream_t delta_stream_ = nullptr;
  std::mutex delta_mu_;
  mutable std::shared_mutex state_mu_;  // searches shared; build / add / delete exclusive

  bool built_ = false;
  uint32_t n_ = 0;
  uint32_t pd16_ = 0, pd8_ = 0, nlist_ = 0;
  DevBuf<float> vectors_, norms16_, fp8_scales_, fp8_norms_;
  DevBuf<uint16_t> fp16_;
  DevBuf<uint8_t> fp8_;
  DevBuf<float> centroids_, codebooks_, sq_mins_, sq_scales_;
  DevBuf<uint8_t> pq_codes_, pq_codes_lm_, sq_codes_, sq_codes_lm_;
  DevBuf<uint32_t> offsets_, vec_ids_;
  // RaBitQ: padded dimension, rotation signs [3P], rotated centroids
  // [nlist][P], sign bits [n][P/32] and meta [n][4] by id and list-major
  uint32_t rq_pd_ = 0;
  uint32_t list_entries_ = 0;  // posting-list entries (offsets[nlist])
  DevBuf<float> rq_signs_, rq_cent_, rq_meta_, rq_meta_lm_;
  DevBuf<uint32_t> rq_bits_, rq_bits_lm_;
  DevBuf<uint32_t> valid_words_;
  std::vector<uint32_t> main_valid_;
  std::unordered_set<uint32_t> tombstones_;
  uint32_t next_id_ = 0;
  Delta delta_;

  std::atomic<int> pins_{0};
  std::mutex pin_mu_;
  std::condition_variable pin_cv_;

  std::mutex metrics_mu_;
  std::vector<double> lat_us_;
  uint64_t total_queries_ = 0;
  std::chrono::steady_clock::time_point start_;
};

// ------------------------------------------------------------------ build
int Index::assign_rows(const float* d_x, uint32_t n, uint32_t dim, const float* d_cent, uint32_t k,
                       GpuSearchResult* out, cudaStream_t s) {
  // nearest centroid of every row: the exact flat scan with k = 1, in
  // chunks so that the per-stream scratch stays small
  const uint32_t chunk = 1u << 20;
  for (uint32_t b = 0; b < n; b += chunk) {
    const uint32_t cnt = std::min(chunk, n - b);
    int rc = launch_flat_f32(d_cent, nullptr, k, dim, d_x + (size_t)b * dim, cnt, 1, METRIC_L2, nullptr, out + b, 0,
                             s);
    if (rc) return rc;
  }
  return 0;
}

int Index::kmeans(const float* d_x, uint32_t n, uint32_t dim, uint32_t k, uint32_t iters, uint64_t seed,
                  float* d_cent, cudaStream_t s, const float* d_init) {
  DevBuf<uint32_t> rows;
  DevBuf<GpuSearchResult> assign;
  DevBuf<uint32_t> counts;
  DevBuf<double> sums;
  int rc = assign.alloc(n);
  if (!rc) rc = counts.alloc(k);
  if (!rc) rc = sums.alloc((size_t)k * dim);
  if (rc) return rc;
  if (d_init) {
    rc = (int)cudaMemcpyAsync(d_cent, d_init, (size_t)k * dim * 4, cudaMemcpyDeviceToDevice, s);
  } else {
    std::vector<uint32_t> init = sample_rows(n, k, seed);
    rc = rows.alloc(init.size());
    if (!rc) rc = (int)cudaMemcpyAsync(rows.p, init.data(), init.size() * 4, cudaMemcpyHostToDevice, s);
    if (!rc) rc = launch_gather_rows(d_x, rows.p, (uint32_t)init.size(), dim, d_cent, s);
  }
  if (rc) return rc;
  for (uint32_t it = 0; it < iters; ++it) {
    rc = assign_rows(d_x, n, dim, d_cent, k, assign.p, s);
    if (!rc) rc = launch_kmeans_update(d_x, n, dim, assign.p, k, d_cent, counts.p, sums.p, s);
    if (rc) return rc;
  }
  return (int)cudaStreamSynchronize(s);
}

int Index::build_ivf(cudaStream_t s, const float* d_init_centroids) {
  const uint32_t dim = cfg_.dim;
  nlist_ = std::max(1u, std::min(cfg_.nlist, n_));
  list_entries_ = n_;
  if (d_init_centroids && nlist_ != cfg_.nlist) return FV_ERR_ARG;
  uint32_t train = cfg_.train_rows ? cfg_.train_rows : (uint32_t)std::min<uint64_t>(n_, 256ull * nlist_);
  train = std::max(std::min(train, n_), nlist_);
  int rc = centroids_.alloc((size_t)nlist_ * dim);
  if (rc) return rc;
  {
    // coarse centroids trained on a sample, then every row assigned
    std::vector<uint32_t> rows = sample_rows(n_, train, cfg_.seed + 1);
    DevBuf<uint32_t> d_rows;
    DevBuf<float> sample;
    rc = d_rows.alloc(rows.size());
    if (!rc) rc = sample.alloc((size_t)rows.size() * dim);
    if (rc) return rc;
    cudaMemcpyAsync(d_rows.p, rows.data(), rows.size() * 4, cudaMemcpyHostToDevice, s);
    rc = launch_gather_rows(vectors_.p, d_rows.p, (uint32_t)rows.size(), dim, sample.p, s);
    if (!rc)
      rc = kmeans(sample.p, (uint32_t)rows.size(), dim, nlist_, d_init_centroids ? cfg_.kmeans_iters_given : cfg_.kmeans_iters,
                  cfg_.seed + 2, centroids_.p, s, d_init_centroids);
    if (rc) return rc;
  }
  DevBuf<GpuSearchResult> assign;
  DevBuf<float> residuals;
  DevBuf<uint32_t> work;
  rc = assign.alloc(n_);
  if (!rc) rc = residuals.alloc((size_t)n_ * dim);
  if (!rc) rc = work.alloc(std::max<size_t>(nlist_, 2 * dim));
  if (!rc) rc = offsets_.alloc(nlist_ + 1);
  if (!rc) rc = vec_ids_.alloc(n_);
  if (rc) return rc;
  rc = assign_rows(vectors_.p, n_, dim, centroids_.p, nlist_, assign.p, s);
  if (!rc) rc = launch_build_lists(assign.p, n_, nlist_, offsets_.p, vec_ids_.p, work.p, s);
  if (!rc) rc = launch_residuals(vectors_.p, n_, dim, centroids_.p, assign.p, residuals.p, s);
  if (rc) return rc;

  if ((cfg_.build_flags & FV_BUILD_IVF_PQ) && cfg_.m_pq && dim % cfg_.m_pq == 0) {
    const uint32_t m = cfg_.m_pq, sub = dim / m;
    rc = codebooks_.alloc((size_t)m * 256 * sub);
    if (rc) return rc;
    const uint32_t kk = std::min(n_, 256u);
    std::vector<uint32_t> rows = sample_rows(n_, std::min(n_, std::max(65536u, kk)), cfg_.seed + 3);
    DevBuf<uint32_t> d_rows;
    DevBuf<float> sample, subv, cb;
    rc = d_rows.alloc(rows.size());
    if (!rc) rc = sample.alloc((size_t)rows.size() * dim);
    if (!rc) rc = subv.alloc((size_t)rows.size() * sub);
    if (!rc) rc = cb.alloc((size_t)256 * sub);
    if (rc) return rc;
    cudaMemcpyAsync(d_rows.p, rows.data(), rows.size() * 4, cudaMemcpyHostToDevice, s);
    rc = launch_gather_rows(residuals.p, d_rows.p, (uint32_t)rows.size(), dim, sample.p, s);
    if (!rc) rc = launch_fill_f32(codebooks_.p, codebooks_.n, 3.4028234663852886e38f, s);  // unused codewords: FLT_MAX
    for (uint32_t mm = 0; !rc && mm < m; ++mm) {
      rc = launch_extract_subspace(sample.p, (uint32_t)rows.size(), dim, mm * sub, sub, subv.p, s);
      if (!rc) rc = kmeans(subv.p, (uint32_t)rows.size(), sub, kk, cfg_.pq_iters, cfg_.seed + 100 + mm, cb.p, s);
      if (!rc)
        rc = (int)cudaMemcpyAsync(codebooks_.p + (size_t)mm * 256 * sub, cb.p, (size_t)kk * sub * 4,
                                  cudaMemcpyDeviceToDevice, s);
    }
    if (!rc) rc = pq_codes_.alloc((size_t)n_ * m);
    if (!rc) rc = launch_pq_encode(residuals.p, n_, dim, m, codebooks_.p, pq_codes_.p, s);
    if (!rc) rc = pq_codes_lm_.alloc((size_t)n_ * m);
    if (!rc) rc = launch_relayout_codes(pq_codes_.p, vec_ids_.p, n_, m, pq_codes_lm_.p, s);
    if (rc) return rc;
  }
  if (cfg_.build_flags & FV_BUILD_IVF_SQ8) {
    rc = sq_mins_.alloc(dim);
    if (!rc) rc = sq_scales_.alloc(dim);
    if (!rc) rc = sq_codes_.alloc((size_t)n_ * dim);
    if (!rc) rc = launch_sq8_fit(residuals.p, n_, dim, sq_mins_.p, sq_scales_.p, work.p, s);
    if (!rc) rc = launch_sq8_encode(residuals.p, n_, dim, sq_mins_.p, sq_scales_.p, sq_codes_.p, s);
    if (!rc) rc = sq_codes_lm_.alloc((size_t)n_ * dim);
    if (!rc) rc = launch_relayout_codes(sq_codes_.p, vec_ids_.p, n_, dim, sq_codes_lm_.p, s);
    if (rc) return rc;
  }
  if (cfg_.build_flags & FV_BUILD_IVF_RABITQ) {
    rc = build_rabitq(assign.p, s);
    if (rc) return rc;
  }
  return (int)cudaStreamSynchronize(s);
}

// RaBitQ tables of the built rows (index.rs:435-441: the engine's seed, the
// rows' own coarse assignment), plus list-major copies of bits and meta.
int Index::build_rabitq(const GpuSearchResult* assign, cudaStream_t s) {
  const uint32_t dim = cfg_.dim, P = rabitq_padded_dim(dim), W = P / 32;
  if (P > 4096) return 0;
  std::vector<float> signs(3 * (size_t)P);
  rabitq_rot_signs(P, kRabitqSeed, signs.data());
  int rc = rq_signs_.alloc(signs.size());
  if (!rc) rc = rq_cent_.alloc((size_t)nlist_ * P);
  if (!rc) rc = rq_bits_.alloc((size_t)n_ * W);
  if (!rc) rc = rq_meta_.alloc((size_t)n_ * 4);
  if (!rc) rc = (int)cudaMemcpyAsync(rq_signs_.p, signs.data(), signs.size() * 4, cudaMemcpyHostToDevice, s);
  if (!rc)
    rc = launch_rabitq_encode(vectors_.p, n_, dim, centroids_.p, nlist_, assign, rq_signs_.p, P, rq_cent_.p,
                              rq_bits_.p, rq_meta_.p, s);
  if (!rc) rc = rabitq_list_major(P, list_entries_, s);
  if (!rc) rc = (int)cudaStreamSynchronize(s);  // `signs` is freed on return
  if (rc) return rc;
  rq_pd_ = P;
  return 0;
}

int Index::build_from(const float* host, uint32_t n, bool device, const float* d_init_centroids) {
  if (!host) return FV_ERR_NULL;
  if (n == 0 || cfg_.dim == 0 || cfg_.dim > 4096) return FV_ERR_ARG;
  std::unique_lock<std::shared_mutex> lk(state_mu_);
  wait_unpinned();
  const uint32_t dim = cfg_.dim;
  cudaStream_t s = streams_[0]->s;
  if (device) {
    // device rows may still be in production on any stream of the caller
    const int rc = (int)cudaDeviceSynchronize();
    if (rc) return rc;
  }
  std::vector<float> staged;
  const float* src = host;
  if (device && cfg_.metric == METRIC_COSINE) {
    staged.resize((size_t)n * dim);
    int rc = (int)cudaMemcpy(staged.data(), host, staged.size() * 4, cudaMemcpyDeviceToHost);
    if (rc) return rc;
    device = false;
    host = staged.data();
  }
  if (!device && cfg_.metric == METRIC_COSINE) {
    if (staged.empty()) staged.assign(host, host + (size_t)n * dim);
    normalize_rows(staged.data(), n, dim);
    src = staged.data();
  } else {
    src = host;
  }
  n_ = n;
  rq_pd_ = 0;
  int rc = vectors_.alloc((size_t)n * dim);
  if (rc) return rc;
  rc = (int)cudaMemcpyAsync(vectors_.p, src, (size_t)n * dim * 4,
                            device ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice, s);
  if (rc) return rc;
  if (cfg_.build_flags & FV_BUILD_FP16) {
    pd16_ = (dim + 15) / 16 * 16;
    rc = fp16_.alloc((size_t)n * pd16_);
    if (!rc) rc = norms16_.alloc(n);
    if (!rc) rc = launch_encode_fp16(vectors_.p, n, dim, pd16_, fp16_.p, norms16_.p, s);
    if (rc) return rc;
  }
  if (cfg_.build_flags & FV_BUILD_FP8) {
    pd8_ = (dim + 3 + 15) / 16 * 16;  // three norm-digit columns
    rc = fp8_.alloc((size_t)n * pd8_);
    if (!rc) rc = fp8_scales_.alloc(n);
    if (!rc) rc = fp8_norms_.alloc(n);
    if (!rc) rc = launch_encode_fp8(vectors_.p, n, dim, pd8_, fp8_.p, fp8_scales_.p, fp8_norms_.p, s);
    if (rc) return rc;
  }
  if (cfg_.nlist && (cfg_.build_flags & (FV_BUILD_IVF_PQ | FV_BUILD_IVF_SQ8 | FV_BUILD_IVF_RABITQ))) {
    rc = build_ivf(s, d_init_centroids);
    if (rc) return rc;
  }
  // validity words: every main slot live (index.rs:505-511)
  main_valid_.assign((n + 31) / 32, 0xFFFFFFFFu);
  if (n % 32) main_valid_.back() = (1u << (n % 32)) - 1u;
  rc = valid_words_.alloc(main_valid_.size());
  if (!rc) rc = (int)cudaMemcpyAsync(valid_words_.p, main_valid_.data(), main_valid_.size() * 4,
                                     cudaMemcpyHostToDevice, s);
  if (!rc) rc = (int)cudaStreamSynchronize(s);
  if (rc) return rc;
  tombstones_.clear();
  delta_.vectors.clear();
  delta_.ids.clear();
  delta_.live.clear();
  next_id_ = n;
  built_ = true;
  return 0;
}

// --------------------------------------------------------- add / delete
int Index::add(const float* host, uint32_t n, uint32_t* out_ids) {
  if (n == 0) return 0;
  if (!host || !out_ids) return FV_ERR_NULL;
  {
    std::shared_lock<std::shared_mutex> rl(state_mu_);
    if (!built_) {
      rl.unlock();
      int rc = build(host, n);
      if (rc) return rc;
      for (uint32_t i = 0; i < n; ++i) out_ids[i] = i;
      return 0;
    }
  }
  std::unique_lock<std::shared_mutex> lk(state_mu_);
  wait_unpinned();
  const uint32_t dim = cfg_.dim;
  const size_t off = delta_.vectors.size();
  delta_.vectors.insert(delta_.vectors.end(), host, host + (size_t)n * dim);
  if (cfg_.metric == METRIC_COSINE) normalize_rows(delta_.vectors.data() + off, n, dim);
  for (uint32_t i = 0; i < n; ++i) {
    out_ids[i] = next_id_ + i;
    delta_.ids.push_back(next_id_ + i);
  }
  next_id_ += n;
  const size_t len = delta_.ids.size();
  int rc = 0;
  if (len > delta_.capacity) {
    size_t cap = 256;
    while (cap < len) cap <<= 1;
    rc = delta_.d_vectors.alloc(cap * dim);
    if (!rc) rc = delta_.d_ids.alloc(cap);
    if (!rc) rc = delta_.d_mask.alloc((cap + 31) / 32);
    if (!rc) rc = delta_.d_live.alloc((cap + 31) / 32);
    if (rc) return rc;
    delta_.capacity = cap;
  }
  delta_.live.resize((len + 31) / 32, 0u);
  for (size_t i = len - n; i < len; ++i) delta_.live[i >> 5] |= 1u << (i & 31);
  rc = (int)cudaMemcpyAsync(delta_.d_vectors.p, delta_.vectors.data(), delta_.vectors.size() * 4,
                            cudaMemcpyHostToDevice, delta_stream_);
  if (!rc)
    rc = (int)cudaMemcpyAsync(delta_.d_ids.p, delta_.ids.data(), len * 4, cudaMemcpyHostToDevice, delta_stream_);
  if (!rc) rc = upload_delta_live(delta_stream_);
  if (!rc) rc = (int)cudaStreamSynchronize(delta_stream_);
  return rc;
}

int Index::upload_delta_live(cudaStream_t s) {
  if (delta_.live.empty()) return 0;
  return (int)cudaMemcpyAsync(delta_.d_live.p, delta_.live.data(), delta_.live.size() * 4, cudaMemcpyHostToDevice, s);
}

int Index::remove(const uint32_t* ids, uint32_t n, uint32_t* out_deleted) {
  if (!out_deleted) return FV_ERR_NULL;
  *out_deleted = 0;
  if (n == 0) return 0;
  if (!ids) return FV_ERR_NULL;
  std::unique_lock<std::shared_mutex> lk(state_mu_);
  wait_unpinned();
  if (!built_) return 0;
  std::unordered_set<uint32_t> in_delta(delta_.ids.begin(), delta_.ids.end());
  uint32_t deleted = 0;
  bool main_dirty = false, delta_dirty = false;
  for (uint32_t i = 0; i < n; ++i) {
    const uint32_t lid = ids[i];
    if (tombstones_.count(lid)) continue;
    if (in_delta.count(lid)) {
      tombstones_.insert(lid);
      // delta ids are assigned in increasing order: the slot is the rank
      const size_t pos = (size_t)(std::lower_bound(delta_.ids.begin(), delta_.ids.end(), lid) - delta_.ids.begin());
      delta_.live[pos >> 5] &= ~(1u << (pos & 31));
      delta_dirty = true;
      ++deleted;
      continue;
    }
    if (lid < n_) {  // slot == logical id (the index is never compacted here)
      tombstones_.insert(lid);
      main_valid_[lid >> 5] &= ~(1u << (lid & 31));
      main_dirty = true;
      ++deleted;
    }
  }
  if (main_dirty) {
    cudaStream_t s = streams_[0]->s;
    int rc = (int)cudaMemcpyAsync(valid_words_.p, main_valid_.data(), main_valid_.size() * 4, cudaMemcpyHostToDevice,
                                  s);
    if (!rc) rc = (int)cudaStreamSynchronize(s);
    if (rc) return rc;
  }
  if (delta_dirty) {
    int rc = upload_delta_live(delta_stream_);
    if (!rc) rc = (int)cudaStreamSynchronize(delta_stream_);
    if (rc) return rc;
  }
  *out_deleted = deleted;
  return 0;
}

// --------------------------------------------------------------- masks
// build_slot_mask_words (index.rs:1264-1292): user mask over logical ids AND
// the live words; words beyond the user mask count as 0.
void Index::slot_mask(const uint32_t* user, uint32_t words, std::vector<uint32_t>& out, bool& use) const {
  use = user != nullptr || !tombstones_.empty();
  if (!use) return;
  const uint32_t nw = (n_ + 31) / 32;
  out.resize(nw);
  for (uint32_t w = 0; w < nw; ++w) out[w] = main_valid_[w] & (user ? (w < words ? user[w] : 0u) : 0xFFFFFFFFu);
}

// build_delta_mask_words (index.rs:1294-1316)
void Index::delta_mask(const uint32_t* user, uint32_t words, std::vector<uint32_t>& out, bool& use) const {
  use = delta_.len() > 0 && (user != nullptr || !tombstones_.empty());
  if (!use) return;
  out.assign((delta_.len() + 31) / 32, 0u);
  for (uint32_t i = 0; i < delta_.len(); ++i) {
    const uint32_t lid = delta_.ids[i];
    if (tombstones_.count(lid)) continue;
    bool allow = true;
    if (user) {
      const uint32_t w = (lid >> 5) < words ? user[lid >> 5] : 0u;
      allow = (w >> (lid & 31)) & 1u;
    }
    if (allow) out[i >> 5] |= 1u << (i & 31);
  }
}

// -------------------------------------------------------------- search
int Index::search(const FvSearchParams& p, const float* q, uint32_t nq, bool device_queries, const uint32_t* user_mask,
                  uint32_t mask_words, GpuSearchResult* out) {
  if (!q || !out) return FV_ERR_NULL;
  std::shared_lock<std::shared_mutex> lk(state_mu_);
  if (!built_) return FV_ERR_ARG;
  if (nq == 0 || p.top_k == 0) return 0;
  const uint32_t dim = cfg_.dim;
  if (p.top_k > 256) return FV_ERR_ARG;  // validate_search_shape (index.rs:309-326)
  const auto t0 = std::chrono::steady_clock::now();
  const uint32_t k = p.top_k;
  Stream& st = *streams_[rr_.fetch_add(1) % streams_.size()];
  std::lock_guard<std::mutex> sl(st.mu);
  int rc = st.q.ensure((size_t)nq * dim);
  if (!rc) rc = st.res.ensure((size_t)nq * k);
  if (!rc) rc = st.hres.ensure((size_t)nq * k);
  if (rc) return rc;

  // queries (prepare_queries, index.rs:1473-1483)
  const float* d_q = q;
  if (!device_queries) {
    rc = st.hq.ensure((size_t)nq * dim);
    if (rc) return rc;
    memcpy(st.hq.p, q, (size_t)nq * dim * 4);
    if (cfg_.metric == METRIC_COSINE) normalize_rows(st.hq.p, nq, dim);
    rc = (int)cudaMemcpyAsync(st.q.p, st.hq.p, (size_t)nq * dim * 4, cudaMemcpyHostToDevice, st.s);
    if (rc) return rc;
    d_q = st.q.p;
  }
  cudaEventRecord(st.ready, st.s);

  std::vector<uint32_t> words;
  bool use_mask = false;
  slot_mask(user_mask, mask_words, words, use_mask);
  const uint32_t* d_mask = nullptr;
  if (use_mask) {
    rc = st.mask.ensure(words.size());
    if (!rc) rc = (int)cudaMemcpyAsync(st.mask.p, words.data(), words.size() * 4, cudaMemcpyHostToDevice, st.s);
    if (rc) return rc;
    d_mask = st.mask.p;
  }

  switch (p.engine) {
    case FV_ENGINE_FLAT:
      rc = cuda_flat_scan_batch(vectors_.p, nullptr, n_, dim, d_q, nq, k, (MetricType)cfg_.metric, d_mask, st.res.p,
                                st.s);
      break;
    case FV_ENGINE_FP16: {
      if (!fp16_.p) return FV_ERR_ARG;
      Fp16GpuTables t{fp16_.p, norms16_.p, vectors_.p, n_, dim, pd16_};
      rc = fv_fp16_search_batch_ex(&t, d_q, nq, k, (MetricType)cfg_.metric, d_mask, &p.scan, st.res.p, st.s);
      break;
    }
    case FV_ENGINE_FP8: {
      if (!fp8_.p) return FV_ERR_ARG;
      FvFp8GpuTables t{fp8_.p, fp8_scales_.p, fp8_norms_.p, vectors_.p, n_, dim, pd8_};
      rc = fv_fp8_search_batch(&t, d_q, nq, k, (MetricType)cfg_.metric, d_mask, &p.scan, st.res.p, st.s);
      break;
    }
    case FV_ENGINE_IVF_PQ: {
      if (!pq_codes_.p) return FV_ERR_ARG;
      IvfPqGpuTables t{centroids_.p, codebooks_.p, pq_codes_lm_.p, offsets_.p, vec_ids_.p, vectors_.p, n_, dim,
                       nlist_,       cfg_.m_pq,    dim / cfg_.m_pq};
      FvIvfOptions o{1, {0, 0, 0}};
      rc = fv_ivf_pq_search_ex(&t, &o, d_q, nq, k, p.nprobe, p.rerank_k, (MetricType)cfg_.metric, d_mask, st.res.p,
                               st.s);
      break;
    }
    case FV_ENGINE_IVF_SQ8: {
      if (!sq_codes_.p) return FV_ERR_ARG;
      IvfSqGpuTables t{centroids_.p, sq_mins_.p, sq_scales_.p, sq_codes_lm_.p, offsets_.p, vec_ids_.p, vectors_.p,
                       n_,           dim,        nlist_};
      FvIvfOptions o{1, {0, 0, 0}};
      rc = fv_ivf_sq_search_ex(&t, &o, d_q, nq, k, p.nprobe, p.rerank_k, (MetricType)cfg_.metric, d_mask, st.res.p,
                               st.s);
      break;
    }
    case FV_ENGINE_IVF_RABITQ: {
      if (!rq_pd_) return FV_ERR_ARG;
      IvfRabitqGpuTables t{centroids_.p, rq_cent_.p, rq_bits_lm_.p, rq_meta_lm_.p, rq_signs_.p, offsets_.p,
                           vec_ids_.p,   vectors_.p, n_,          dim,           rq_pd_,      rq_pd_ / 32,
                           nlist_};
      FvIvfOptions o{1, {0, 0, 0}};
      rc = fv_ivf_rabitq_search_ex(&t, &o, d_q, nq, k, p.nprobe, p.rerank_k, (MetricType)cfg_.metric, d_mask,
                                   st.res.p, st.s);
      break;
    }
    default:
      return FV_ERR_ARG;
  }
  if (rc) return rc;

  // concurrent delta scan (launch_delta_scan_inner, index.rs:1424-1471)
  std::unique_lock<std::mutex> dl(delta_mu_, std::defer_lock);
  const bool has_delta = delta_.len() > 0;
  if (has_delta) {
    dl.lock();
    rc = delta_.d_res.ensure((size_t)nq * k);
    if (!rc) rc = delta_.h_res.ensure((size_t)nq * k);
    if (rc) return rc;
    cudaStreamWaitEvent(delta_stream_, st.ready, 0);
    std::vector<uint32_t> dw;
    bool use_dmask = false;
    delta_mask(user_mask, mask_words, dw, use_dmask);
    if (use_dmask) {
      rc = (int)cudaMemcpyAsync(delta_.d_mask.p, dw.data(), dw.size() * 4, cudaMemcpyHostToDevice, delta_stream_);
      if (rc) return rc;
    }
    rc = cuda_flat_scan_batch(delta_.d_vectors.p, delta_.d_ids.p, delta_.len(), dim, d_q, nq, k,
                              (MetricType)cfg_.metric, use_dmask ? delta_.d_mask.p : nullptr, delta_.d_res.p,
                              delta_stream_);
    if (!rc)
      rc = (int)cudaMemcpyAsync(delta_.h_res.p, delta_.d_res.p, (size_t)nq * k * sizeof(GpuSearchResult),
                                cudaMemcpyDeviceToHost, delta_stream_);
    if (rc) return rc;
  }
  rc = (int)cudaMemcpyAsync(st.hres.p, st.res.p, (size_t)nq * k * sizeof(GpuSearchResult), cudaMemcpyDeviceToHost,
                            st.s);
  if (!rc) rc = (int)cudaStreamSynchronize(st.s);
  if (!rc && has_delta) rc = (int)cudaStreamSynchronize(delta_stream_);
  if (rc) return rc;

  if (!has_delta) {
    memcpy(out, st.hres.p, (size_t)nq * k * sizeof(GpuSearchResult));
  } else {
    // finish_delta_merge (index.rs:1353-1387): main then delta, invalid ids
    // dropped, stable sort by distance, truncate, pad with {u32::MAX, +inf}
    std::vector<GpuSearchResult> comb;
    for (uint32_t qi = 0; qi < nq; ++qi) {
      comb.clear();
      for (uint32_t r = 0; r < k; ++r)
        if (st.hres.p[(size_t)qi * k + r].id != 0xFFFFFFFFu) comb.push_back(st.hres.p[(size_t)qi * k + r]);
      for (uint32_t r = 0; r < k; ++r)
        if (delta_.h_res.p[(size_t)qi * k + r].id != 0xFFFFFFFFu) comb.push_back(delta_.h_res.p[(size_t)qi * k + r]);
      std::stable_sort(comb.begin(), comb.end(),
                       [](const GpuSearchResult& a, const GpuSearchResult& b) { return a.distance < b.distance; });
      for (uint32_t r = 0; r < k; ++r)
        out[(size_t)qi * k + r] = r < comb.size() ? comb[r] : GpuSearchResult{0xFFFFFFFFu, INFINITY};
    }
  }
  record(std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count(), nq);
  return 0;
}

// ------------------------------------------------------------ snapshots
// The reference's FLSHVEC1 file (persistence.rs, index.rs:845-1260) read
// into the engine's device tables, and written from them.
//
// Load: sections are copied to the GPU straight from the read-only mapping
// (page-locked in place when the driver allows, so the copies are DMA from
// the page cache). Slots whose logical id differs from the slot index
// (logical_ids not the identity) are placed at their logical ids, so the
// engine keeps slot == logical id; never-assigned ids in between become
// invalid slots. Tables the file lacks or that this engine adds are built on
// the GPU: fp16 rows when the file has none of this padding, fp8 rows, and
// the list-major IVF code copies.
//
// Save: every section the reference's loader requires is written, the
// graph and RaBitQ ones (outside this engine) empty, so the reference can
// open the file and serve the flat / fp16 / IVF paths from it.
namespace {
// Page-locks the mapping for the duration of a load (copies from it are then
// DMA); on destruction waits for the stream's copies before unlocking.
struct HostRegistration {
  void* p = nullptr;
  cudaStream_t s = nullptr;
  bool ok = false;
  HostRegistration(const void* ptr, size_t bytes, cudaStream_t stream) : s(stream) {
    if (bytes == 0) return;
    p = const_cast<void*>(ptr);
    ok = cudaHostRegister(p, bytes, cudaHostRegisterReadOnly) == cudaSuccess;
    if (!ok) cudaGetLastError();  // clear: the copies fall back to staged transfers
  }
  ~HostRegistration() {
    cudaStreamSynchronize(s);
    if (ok) cudaHostUnregister(p);
  }
};

template <class T>
int upload(DevBuf<T>& dst, const uint8_t* src, uint64_t bytes, cudaStream_t s) {
  int rc = dst.alloc(bytes / sizeof(T));
  if (!rc && bytes) rc = (int)cudaMemcpyAsync(dst.p, src, bytes, cudaMemcpyHostToDevice, s);
  return rc;
}
}  // namespace

int Index::load_snapshot(const snap::File& f, std::string* error) {
  std::unique_lock<std::shared_mutex> lk(state_mu_);
  wait_unpinned();
  const snap::Manifest& m = f.manifest();
  auto fail = [&](const std::string& why) {
    if (error) *error = why;
    return FV_ERR_ARG;
  };
  const uint32_t dim = cfg_.dim;
  const uint64_t n = m.num_vectors;
  if (n == 0 || n >= 0xFFFFFFFFull) return fail("snapshot holds no vectors (or more than 2^32 - 1)");
  uint64_t b = 0;
  const uint8_t* vecs = f.section("vectors", &b);
  if (!vecs || b != n * dim * 4) return fail("vectors section missing or not num_vectors x dim f32");
  cudaStream_t s = streams_[0]->s;
  HostRegistration reg(f.base(), f.size(), s);

  // logical ids: slot -> logical id (identity when absent)
  std::vector<uint32_t> lid;
  uint64_t lb = 0;
  if (const uint8_t* p = f.section("logical_ids", &lb)) {
    if (lb != n * 4) return fail("logical_ids section is not num_vectors u32");
    lid.assign(reinterpret_cast<const uint32_t*>(p), reinterpret_cast<const uint32_t*>(p) + n);
  }
  bool identity = true;
  uint64_t nslots = n;
  for (uint64_t i = 0; i < lid.size(); ++i) {
    identity = identity && lid[i] == i;
    nslots = std::max<uint64_t>(nslots, (uint64_t)lid[i] + 1);
  }
  if (!identity && nslots > std::max<uint64_t>(4 * n, n + 4096))
    return fail("logical ids too sparse to place at their own slots (more than 4x the row count)");
  // inv[logical] = slot, n = no row (zero / invalid)
  std::vector<uint32_t> inv;
  DevBuf<uint32_t> d_inv;
  if (!identity) {
    inv.assign(nslots, (uint32_t)n);
    for (uint64_t i = 0; i < n; ++i) {
      if (inv[lid[i]] != (uint32_t)n) return fail("duplicate logical id in logical_ids");
      inv[lid[i]] = (uint32_t)i;
    }
    int rc = d_inv.alloc(nslots);
    if (!rc) rc = (int)cudaMemcpyAsync(d_inv.p, inv.data(), nslots * 4, cudaMemcpyHostToDevice, s);
    if (rc) return rc;
  }
  // a table of n rows -> the engine's nslots rows at logical positions
  auto place_rows = [&](const uint8_t* src, uint64_t row_bytes, auto& dst) -> int {
    using T = typename std::remove_reference<decltype(*dst.p)>::type;
    if (identity) return upload(dst, src, n * row_bytes, s);
    DevBuf<uint8_t> tmp;
    int rc = upload(tmp, src, n * row_bytes, s);
    if (!rc) rc = dst.alloc(nslots * row_bytes / sizeof(T));
    if (!rc) rc = launch_gather_row_bytes(tmp.p, d_inv.p, (uint32_t)nslots, (uint32_t)row_bytes, (uint32_t)n, dst.p, s);
    if (!rc) rc = (int)cudaStreamSynchronize(s);  // tmp is freed on return
    return rc;
  };
  int rc = place_rows(vecs, (uint64_t)dim * 4, vectors_);
  if (rc) return rc;
  n_ = (uint32_t)nslots;

  // validity words over slots -> over logical ids (tombstoned and unassigned
  // ids invalid)
  std::vector<uint32_t> slot_valid((n + 31) / 32, 0xFFFFFFFFu);
  uint64_t vb = 0;
  if (const uint8_t* p = f.section("main_valid_words", &vb)) {
    if (vb < slot_valid.size() * 4) return fail("main_valid_words shorter than num_vectors bits");
    std::memcpy(slot_valid.data(), p, slot_valid.size() * 4);
  }
  main_valid_.assign((nslots + 31) / 32, 0u);
  tombstones_.clear();
  for (uint64_t i = 0; i < n; ++i) {
    const uint32_t l = identity ? (uint32_t)i : lid[i];
    if ((slot_valid[i >> 5] >> (i & 31)) & 1u)
      main_valid_[l >> 5] |= 1u << (l & 31);
    else
      tombstones_.insert(l);
  }
  uint64_t tb = 0;
  if (const uint8_t* p = f.section("tombstones", &tb)) {
    const uint32_t* t = reinterpret_cast<const uint32_t*>(p);
    for (uint64_t i = 0; i < tb / 4; ++i) tombstones_.insert(t[i]);
  }
  rc = valid_words_.alloc(main_valid_.size());
  if (!rc) rc = (int)cudaMemcpyAsync(valid_words_.p, main_valid_.data(), main_valid_.size() * 4,
                                     cudaMemcpyHostToDevice, s);
  if (rc) return rc;

  // fp16 rows: the file's when padded as this engine pads, else encoded here
  pd16_ = pd8_ = 0;
  if (cfg_.build_flags & FV_BUILD_FP16) {
    const uint32_t pd = (dim + 15) / 16 * 16;
    uint64_t hb = 0, nb = 0;
    const uint8_t* h = f.section("vectors_fp16", &hb);
    const uint8_t* nr = f.section("vec_norms_sq", &nb);
    pd16_ = pd;
    if (h && nr && m.fp16_padded_dim == pd && hb == n * pd * 2 && nb == n * 4) {
      rc = place_rows(h, (uint64_t)pd * 2, fp16_);
      if (!rc) rc = place_rows(nr, 4, norms16_);
    } else {
      rc = fp16_.alloc((size_t)n_ * pd);
      if (!rc) rc = norms16_.alloc(n_);
      if (!rc) rc = launch_encode_fp16(vectors_.p, n_, dim, pd, fp16_.p, norms16_.p, s);
    }
    if (rc) return rc;
  }
  if (cfg_.build_flags & FV_BUILD_FP8) {
    pd8_ = (dim + 3 + 15) / 16 * 16;  // three norm-digit columns
    rc = fp8_.alloc((size_t)n_ * pd8_);
    if (!rc) rc = fp8_scales_.alloc(n_);
    if (!rc) rc = fp8_norms_.alloc(n_);
    if (!rc) rc = launch_encode_fp8(vectors_.p, n_, dim, pd8_, fp8_.p, fp8_scales_.p, fp8_norms_.p, s);
    if (rc) return rc;
  }

  // IVF tables (ids in the lists are slots: mapped to logical ids)
  nlist_ = 0;
  rq_pd_ = 0;
  uint64_t cb = 0, ob = 0, ib = 0;
  const uint8_t* cent = f.section("ivf_centroids", &cb);
  const uint8_t* offs = f.section("ivf_offsets", &ob);
  const uint8_t* vids = f.section("ivf_vec_ids", &ib);
  if (m.nlist && cent && offs && vids && cb == (uint64_t)m.nlist * dim * 4 && ob == ((uint64_t)m.nlist + 1) * 4 &&
      ib == n * 4) {
    nlist_ = m.nlist;
    rc = upload(centroids_, cent, cb, s);
    if (!rc) rc = upload(offsets_, offs, ob, s);
    DevBuf<uint32_t> slot_ids;  // list order, slots (for the list-major copies)
    if (!rc) rc = upload(slot_ids, vids, ib, s);
    std::vector<uint32_t> mapped(reinterpret_cast<const uint32_t*>(vids), reinterpret_cast<const uint32_t*>(vids) + n);
    for (auto& v : mapped) {
      if (v >= n) return fail("ivf_vec_ids holds a slot beyond num_vectors");
      if (!identity) v = lid[v];
    }
    if (!rc) rc = vec_ids_.alloc(n);
    if (!rc) rc = (int)cudaMemcpyAsync(vec_ids_.p, mapped.data(), n * 4, cudaMemcpyHostToDevice, s);
    if (!rc) rc = (int)cudaStreamSynchronize(s);  // `mapped` is freed on return
    if (rc) return rc;
    uint64_t bb = 0, pb = 0;
    const uint8_t* books = f.section("pq_codebooks", &bb);
    const uint8_t* pcodes = f.section("pq_codes", &pb);
    const uint32_t mq = m.m_pq;
    if (mq && dim % mq == 0 && books && pcodes && bb == (uint64_t)mq * 256 * (dim / mq) * 4 && pb == n * mq) {
      rc = upload(codebooks_, books, bb, s);
      DevBuf<uint8_t> by_slot;
      if (!rc) rc = upload(by_slot, pcodes, pb, s);
      if (!rc) rc = pq_codes_lm_.alloc(n * mq);
      if (!rc) rc = launch_relayout_codes(by_slot.p, slot_ids.p, (uint32_t)n, mq, pq_codes_lm_.p, s);
      if (!rc) rc = place_rows(pcodes, mq, pq_codes_);
      if (!rc) rc = (int)cudaStreamSynchronize(s);
      if (rc) return rc;
    }
    uint64_t mb = 0, sb = 0, qb = 0;
    const uint8_t* mins = f.section("sq_mins", &mb);
    const uint8_t* scales = f.section("sq_scales", &sb);
    const uint8_t* scodes = f.section("sq_codes", &qb);
    if (mins && scales && scodes && mb == (uint64_t)dim * 4 && sb == (uint64_t)dim * 4 && qb == n * dim) {
      rc = upload(sq_mins_, mins, mb, s);
      if (!rc) rc = upload(sq_scales_, scales, sb, s);
      DevBuf<uint8_t> by_slot;
      if (!rc) rc = upload(by_slot, scodes, qb, s);
      if (!rc) rc = sq_codes_lm_.alloc(n * dim);
      if (!rc) rc = launch_relayout_codes(by_slot.p, slot_ids.p, (uint32_t)n, dim, sq_codes_lm_.p, s);
      if (!rc) rc = place_rows(scodes, dim, sq_codes_);
      if (!rc) rc = (int)cudaStreamSynchronize(s);
      if (rc) return rc;
    }
    // RaBitQ: the file's tables when present and consistent, else encoded
    // here from the rows and their lists
    list_entries_ = (uint32_t)n;
    uint64_t rsb = 0, rcb = 0, rbb = 0, rmb = 0;
    const uint8_t* rsig = f.section("rabitq_signs", &rsb);
    const uint8_t* rcen = f.section("rabitq_centroids", &rcb);
    const uint8_t* rbits = f.section("rabitq_bits", &rbb);
    const uint8_t* rmeta = f.section("rabitq_meta", &rmb);
    const uint64_t P = m.rabitq_padded_dim;
    if (P >= 32 && P <= 4096 && (P & (P - 1)) == 0 && P >= dim && rsig && rcen && rbits && rmeta &&
        rsb == 3 * P * 4 && rcb == (uint64_t)m.nlist * P * 4 && rbb == n * (P / 8) && rmb == n * 16) {
      rc = upload(rq_signs_, rsig, rsb, s);
      if (!rc) rc = upload(rq_cent_, rcen, rcb, s);
      if (!rc) rc = place_rows(rbits, P / 8, rq_bits_);
      if (!rc) rc = place_rows(rmeta, 16, rq_meta_);
      if (!rc) rc = rabitq_list_major((uint32_t)P, (uint32_t)n, s);
      if (!rc) rc = (int)cudaStreamSynchronize(s);
      if (rc) return rc;
      rq_pd_ = (uint32_t)P;
    } else if ((cfg_.build_flags & FV_BUILD_IVF_RABITQ) && rabitq_padded_dim(dim) <= 4096) {
      std::vector<GpuSearchResult> assign(nslots, GpuSearchResult{0xFFFFFFFFu, 0.f});
      const uint32_t* o = reinterpret_cast<const uint32_t*>(offs);
      for (uint32_t l = 0; l < m.nlist; ++l)
        for (uint32_t i = o[l]; i < o[l + 1] && i < n; ++i) assign[mapped[i]].id = l;
      DevBuf<GpuSearchResult> d_assign;
      rc = d_assign.alloc(nslots);
      if (!rc)
        rc = (int)cudaMemcpyAsync(d_assign.p, assign.data(), nslots * sizeof(GpuSearchResult), cudaMemcpyHostToDevice, s);
      if (!rc) rc = build_rabitq(d_assign.p, s);
      if (rc) return rc;
    }
  }

  // live-insert buffer
  delta_.vectors.clear();
  delta_.ids.clear();
  delta_.live.clear();
  uint64_t dvb = 0, dib = 0;
  const uint8_t* dv = f.section("delta_vectors", &dvb);
  const uint8_t* di = f.section("delta_ids", &dib);
  uint32_t next = m.next_logical_id;
  next = std::max<uint32_t>(next, (uint32_t)nslots);
  if (dv && di && dib > 0) {
    const uint64_t len = dib / 4;
    if (dvb != len * dim * 4) return fail("delta_vectors does not match delta_ids");
    delta_.vectors.assign(reinterpret_cast<const float*>(dv), reinterpret_cast<const float*>(dv) + len * dim);
    delta_.ids.assign(reinterpret_cast<const uint32_t*>(di), reinterpret_cast<const uint32_t*>(di) + len);
    size_t cap = 256;
    while (cap < len) cap <<= 1;
    rc = delta_.d_vectors.alloc(cap * dim);
    if (!rc) rc = delta_.d_ids.alloc(cap);
    if (!rc) rc = delta_.d_mask.alloc((cap + 31) / 32);
    if (!rc) rc = delta_.d_live.alloc((cap + 31) / 32);
    if (rc) return rc;
    delta_.capacity = cap;
    delta_.live.assign((len + 31) / 32, 0u);
    for (uint64_t i = 0; i < len; ++i) {
      if (!tombstones_.count(delta_.ids[i])) delta_.live[i >> 5] |= 1u << (i & 31);
      next = std::max<uint32_t>(next, delta_.ids[i] + 1);
    }
    rc = (int)cudaMemcpyAsync(delta_.d_vectors.p, delta_.vectors.data(), len * dim * 4, cudaMemcpyHostToDevice, s);
    if (!rc) rc = (int)cudaMemcpyAsync(delta_.d_ids.p, delta_.ids.data(), len * 4, cudaMemcpyHostToDevice, s);
    if (!rc) rc = upload_delta_live(s);
    if (rc) return rc;
  }
  next_id_ = next;
  rc = (int)cudaStreamSynchronize(s);
  if (rc) return rc;
  built_ = true;
  return 0;
}

int Index::save_snapshot(const char* path, std::string* error) {
  std::shared_lock<std::shared_mutex> lk(state_mu_);
  if (!built_) {
    if (error) *error = "index not built";
    return FV_ERR_ARG;
  }
  const uint32_t dim = cfg_.dim;
  auto d2h = [](const auto& buf, auto& host) -> int {
    host.resize(buf.n);
    return buf.n ? (int)cudaMemcpy(host.data(), buf.p, buf.bytes(), cudaMemcpyDeviceToHost) : 0;
  };
  std::vector<float> vecs, cent, books, mins, scales, norms, rsig, rcen, rmeta;
  std::vector<uint16_t> f16;
  std::vector<uint8_t> pq, sq;
  std::vector<uint32_t> offs, vids, rbits;
  int rc = d2h(vectors_, vecs);
  if (!rc) rc = d2h(centroids_, cent);
  if (!rc) rc = d2h(codebooks_, books);
  if (!rc) rc = d2h(pq_codes_, pq);
  if (!rc) rc = d2h(offsets_, offs);
  if (!rc) rc = d2h(vec_ids_, vids);
  if (!rc) rc = d2h(sq_mins_, mins);
  if (!rc) rc = d2h(sq_scales_, scales);
  if (!rc) rc = d2h(sq_codes_, sq);
  if (!rc) rc = d2h(fp16_, f16);
  if (!rc) rc = d2h(norms16_, norms);
  if (!rc && rq_pd_) {
    rc = d2h(rq_signs_, rsig);
    if (!rc) rc = d2h(rq_cent_, rcen);
    if (!rc) rc = d2h(rq_bits_, rbits);
    if (!rc) rc = d2h(rq_meta_, rmeta);
  }
  if (rc) return rc;
  std::vector<uint32_t> ids(n_);
  for (uint32_t i = 0; i < n_; ++i) ids[i] = i;
  std::vector<uint32_t> tomb(tombstones_.begin(), tombstones_.end());
  std::sort(tomb.begin(), tomb.end());

  snap::Manifest m;
  m.version = 1;
  m.dim = dim;
  m.max_elements = n_;
  m.nlist = nlist_;
  m.m_pq = codebooks_.n ? cfg_.m_pq : 0;
  m.metric = cfg_.metric;
  m.num_vectors = n_;
  m.fp16_padded_dim = fp16_.n ? pd16_ : 0;
  m.rabitq_padded_dim = rq_pd_;
  m.next_logical_id = next_id_;
  auto sec = [](const char* name, const char* dtype, const auto& v) {
    using T = typename std::decay<decltype(v[0])>::type;
    return snap::OutSection{name, dtype, (uint64_t)v.size(), v.data(), (uint64_t)v.size() * sizeof(T)};
  };
  const std::vector<uint32_t> none_u32;
  std::vector<snap::OutSection> out = {
      sec("vectors", "f32", vecs),          sec("logical_ids", "u32", ids),
      sec("main_valid_words", "u32", main_valid_), sec("hnsw_adjacency", "u32", none_u32),
      sec("hnsw_degrees", "u32", none_u32), sec("cagra_adjacency", "u32", none_u32),
      sec("ivf_centroids", "f32", cent),    sec("pq_codebooks", "f32", books),
      sec("pq_codes", "u8", pq),            sec("ivf_offsets", "u32", offs),
      sec("ivf_vec_ids", "u32", vids),      sec("sq_mins", "f32", mins),
      sec("sq_scales", "f32", scales),      sec("sq_codes", "u8", sq),
      sec("rabitq_signs", "f32", rsig),     sec("rabitq_centroids", "f32", rcen),
      sec("rabitq_bits", "u32", rbits),     sec("rabitq_meta", "f32", rmeta),
      sec("vectors_fp16", "u16", f16),      sec("vec_norms_sq", "f32", norms)};
  if (!tomb.empty()) out.push_back(sec("tombstones", "u32", tomb));
  if (delta_.len()) {
    out.push_back(sec("delta_vectors", "f32", delta_.vectors));
    out.push_back(sec("delta_ids", "u32", delta_.ids));
  }
  return snap::write(path, m, out, error);
}

// ------------------------------------------------------- served batches
// One heterogeneous batch on the caller's stream, with the semantics of
// search() for every query taken alone: the main scan (shared validity
// words for tombstones, per-query filters over logical ids), the delta
// scan of the live-insert buffer (validity words over delta slots, filters
// through the delta ids) and the stable merge, all stream-ordered.
// The IVF launch of a served batch (list-major tables, the batch's
// per-query parameters and filters), writing `out`.
IvfLaunch Index::batch_ivf_launch(const BatchLaunch& b, GpuSearchResult* out) const {
  const bool pq = b.engine == FV_ENGINE_IVF_PQ, rq = b.engine == FV_ENGINE_IVF_RABITQ;
  IvfLaunch L{};
  L.centroids = centroids_.p;
  L.codebooks = pq ? codebooks_.p : nullptr;
  L.sq_mins = pq ? nullptr : sq_mins_.p;
  L.sq_scales = pq ? nullptr : sq_scales_.p;
  L.codes = pq ? pq_codes_lm_.p : sq_codes_lm_.p;
  L.offsets = offsets_.p;
  L.vec_ids = vec_ids_.p;
  L.vectors = vectors_.p;
  L.num_vectors = n_;
  L.dim = cfg_.dim;
  L.nlist = nlist_;
  L.m_pq = pq ? cfg_.m_pq : 0;
  L.sub_dim = pq ? cfg_.dim / cfg_.m_pq : 0;
  L.list_major = true;
  L.queries = b.d_queries;
  L.nq = b.nq;
  L.top_k = b.top_k;
  L.nprobe = b.nprobe;
  L.rerank_k = b.rerank_k;
  L.metric = (MetricType)cfg_.metric;
  L.mask = tombstones_.empty() ? nullptr : valid_words_.p;
  L.out = out;
  L.q_topk = b.d_topk;
  L.q_nprobe = b.d_nprobe;
  L.q_rerank = b.d_rerank;
  L.filters = b.d_filters;
  if (rq) {
    L.codes = nullptr;
    L.rot_centroids = rq_cent_.p;
    L.rq_bits = rq_bits_lm_.p;
    L.rq_meta = rq_meta_lm_.p;
    L.rot_signs = rq_signs_.p;
    L.padded_dim = rq_pd_;
  }
  return L;
}

TcTables Index::tc_tables(bool fp8) const {
  return fp8 ? TcTables{true, fp8_.p, fp8_norms_.p, fp8_scales_.p, vectors_.p, n_, cfg_.dim, pd8_}
             : TcTables{false, fp16_.p, norms16_.p, nullptr, vectors_.p, n_, cfg_.dim, pd16_};
}

int Index::launch_batch(const BatchLaunch& b, cudaStream_t s) {
  if (!built_) return FV_ERR_ARG;
  if (b.nq == 0 || b.top_k == 0) return 0;
  if (b.top_k > 256) return FV_ERR_ARG;
  if (!b.d_queries || !b.d_out) return FV_ERR_NULL;
  const bool ivf = b.engine == FV_ENGINE_IVF_PQ || b.engine == FV_ENGINE_IVF_SQ8 || b.engine == FV_ENGINE_IVF_RABITQ;
  if (!ivf && (b.d_topk || b.d_nprobe || b.d_rerank)) return FV_ERR_ARG;
  const bool has_delta = delta_.len() > 0;
  if (has_delta && (!b.d_main || !b.d_delta)) return FV_ERR_NULL;
  const uint32_t dim = cfg_.dim, k = b.top_k, nq = b.nq;
  const MetricType metric = (MetricType)cfg_.metric;
  GpuSearchResult* main_out = has_delta ? b.d_main : b.d_out;
  const uint32_t* shared_mask = tombstones_.empty() ? nullptr : valid_words_.p;
  int rc = 0;
  switch (b.engine) {
    case FV_ENGINE_FLAT:
      rc = launch_flat_f32(vectors_.p, nullptr, n_, dim, b.d_queries, nq, k, metric, shared_mask, main_out, 0, s,
                           b.d_filters);
      break;
    case FV_ENGINE_FP16:
    case FV_ENGINE_FP8: {
      const bool fp8 = b.engine == FV_ENGINE_FP8;
      if (fp8 ? !fp8_.p : !fp16_.p) return FV_ERR_ARG;
      rc = launch_tc_scan(tc_tables(fp8), b.d_queries, nq, k, metric, shared_mask, main_out, b.scan, s, b.d_filters);
      break;
    }
    case FV_ENGINE_IVF_PQ:
    case FV_ENGINE_IVF_SQ8:
    case FV_ENGINE_IVF_RABITQ: {
      const bool pq = b.engine == FV_ENGINE_IVF_PQ, rq = b.engine == FV_ENGINE_IVF_RABITQ;
      if (rq ? !rq_pd_ : pq ? !pq_codes_lm_.p : !sq_codes_lm_.p) return FV_ERR_ARG;
      if (nlist_ == 0 || (pq && cfg_.m_pq == 0)) {
        rc = launch_fill_sentinel(main_out, (size_t)nq * k, s);
        break;
      }
      rc = launch_ivf_search(rq ? IVF_MODE_RABITQ : pq ? IVF_MODE_PQ : IVF_MODE_SQ8, batch_ivf_launch(b, main_out), s);
      break;
    }
    default:
      return FV_ERR_ARG;
  }
  if (rc || !has_delta) return rc;
  rc = launch_flat_f32(delta_.d_vectors.p, delta_.d_ids.p, delta_.len(), dim, b.d_queries, nq, k, metric,
                       delta_.d_live.p, b.d_delta, 0, s, b.d_filters);
  if (rc) return rc;
  return launch_merge_main_delta(b.d_main, b.d_delta, nq, k, b.d_topk, k, b.d_out, s);
}

// Scratch that launch_batch takes from its stream's arena for `b`: the
// largest request of its launches (they run in order on one stream, so
// they share one arena). Only b.engine, nq, top_k, nprobe, rerank_k, scan
// and whether the per-query arrays are present are read.
size_t Index::batch_scratch_bytes(const BatchLaunch& b) const {
  if (!built_ || b.nq == 0 || b.top_k == 0) return 0;
  const MetricType metric = (MetricType)cfg_.metric;
  size_t need = 0;
  switch (b.engine) {
    case FV_ENGINE_FLAT:
      need = plan_flat_f32(n_, b.nq, std::min(b.top_k, 256u), 0).scratch_bytes;
      break;
    case FV_ENGINE_FP16:
    case FV_ENGINE_FP8:
      need = tc_scan_scratch_bytes(tc_tables(b.engine == FV_ENGINE_FP8), b.nq, b.top_k, metric, b.scan);
      break;
    case FV_ENGINE_IVF_PQ:
    case FV_ENGINE_IVF_SQ8:
    case FV_ENGINE_IVF_RABITQ: {
      const bool pq = b.engine == FV_ENGINE_IVF_PQ, rq = b.engine == FV_ENGINE_IVF_RABITQ;
      need = ivf_search_scratch_bytes(rq ? IVF_MODE_RABITQ : pq ? IVF_MODE_PQ : IVF_MODE_SQ8,
                                      batch_ivf_launch(b, nullptr));
      break;
    }
    default:
      return 0;
  }
  if (delta_.len() > 0)
    need = std::max(need, plan_flat_f32(delta_.len(), b.nq, std::min(b.top_k, 256u), 0).scratch_bytes);
  return need;
}

// ------------------------------------------------------------- metrics
void Index::record(double seconds, uint32_t nq) {
  std::lock_guard<std::mutex> lk(metrics_mu_);
  const double us = seconds * 1e6 / std::max<uint32_t>(nq, 1);
  if (lat_us_.size() >= 100000) lat_us_.erase(lat_us_.begin(), lat_us_.begin() + 50000);
  lat_us_.push_back(us);
  total_queries_ += nq;
}

void Index::stats(FvLatencyStats* s) {
  std::lock_guard<std::mutex> lk(metrics_mu_);
  *s = FvLatencyStats{};
  s->count = total_queries_;
  const double el = std::max(1e-3, std::chrono::duration<double>(std::chrono::steady_clock::now() - start_).count());
  s->qps = (double)total_queries_ / el;
  if (lat_us_.empty()) return;
  std::vector<double> v = lat_us_;
  std::sort(v.begin(), v.end());
  const size_t n = v.size();
  auto at = [&](double f) { return v[std::min(n - 1, (size_t)((double)n * f))]; };
  s->p50_us = at(0.5);
  s->p90_us = at(0.9);
  s->p99_us = at(0.99);
  s->p999_us = at(0.999);
  s->min_us = v.front();
  s->max_us = v.back();
  double sum = 0;
  for (double x : v) sum += x;
  s->mean_us = sum / (double)n;
}

void Index::info(FvIndexInfo* i) {
  std::shared_lock<std::shared_mutex> lk(state_mu_);
  *i = FvIndexInfo{};
  i->num_vectors = n_;
  i->delta_len = delta_.len();
  i->tombstones = (uint32_t)tombstones_.size();
  i->dim = cfg_.dim;
  i->padded_dim = pd16_;
  i->nlist = nlist_;
  i->m_pq = cfg_.m_pq;
  i->metric = cfg_.metric;
  i->next_id = next_id_;
  i->device_bytes = vectors_.bytes() + fp16_.bytes() + norms16_.bytes() + fp8_.bytes() + fp8_scales_.bytes() +
                    fp8_norms_.bytes() + centroids_.bytes() + codebooks_.bytes() + pq_codes_.bytes() +
                    pq_codes_lm_.bytes() + sq_codes_.bytes() + sq_codes_lm_.bytes() + offsets_.bytes() +
                    vec_ids_.bytes() + rq_signs_.bytes() + rq_cent_.bytes() + rq_bits_.bytes() + rq_bits_lm_.bytes() +
                    rq_meta_.bytes() + rq_meta_lm_.bytes();
}

// Device views of the IVF tables (list-major codes) for direct kernel calls.
int Index::tables(IvfPqGpuTables* pq, IvfSqGpuTables* sq, FvIvfOptions* opt) {
  std::shared_lock<std::shared_mutex> lk(state_mu_);
  if (!built_ || !offsets_.p) return FV_ERR_ARG;
  if (pq) *pq = IvfPqGpuTables{centroids_.p, codebooks_.p, pq_codes_lm_.p, offsets_.p, vec_ids_.p, vectors_.p, n_,
                               cfg_.dim,     nlist_,       cfg_.m_pq,      cfg_.m_pq ? cfg_.dim / cfg_.m_pq : 0};
  if (sq) *sq = IvfSqGpuTables{centroids_.p, sq_mins_.p, sq_scales_.p, sq_codes_lm_.p, offsets_.p, vec_ids_.p,
                               vectors_.p,   n_,         cfg_.dim,     nlist_};
  if (opt) *opt = FvIvfOptions{1, {0, 0, 0}};
  return 0;
}

int Index::rabitq_tables(IvfRabitqGpuTables* t, FvIvfOptions* opt) {
  std::shared_lock<std::shared_mutex> lk(state_mu_);
  if (!built_ || !offsets_.p || !rq_pd_) return FV_ERR_ARG;
  if (t) *t = IvfRabitqGpuTables{centroids_.p, rq_cent_.p, rq_bits_lm_.p, rq_meta_lm_.p, rq_signs_.p, offsets_.p,
                                 vec_ids_.p,   vectors_.p, n_,          cfg_.dim,      rq_pd_,      rq_pd_ / 32,
                                 nlist_};
  if (opt) *opt = FvIvfOptions{1, {0, 0, 0}};
  return 0;
}

// Copies one IVF table to the host (for checking the build against a CPU
// restatement): 0 centroids, 1 codebooks, 2 pq codes (by id), 3 sq mins,
// 4 sq scales, 5 sq codes (by id), 6 offsets, 7 vec ids, 8 RaBitQ signs,
// 9 rotated centroids, 10 RaBitQ bits (by id), 11 RaBitQ meta (by id).
int Index::export_ivf(uint32_t what, void* host_out, size_t bytes) {
  std::shared_lock<std::shared_mutex> lk(state_mu_);
  const void* src = nullptr;
  size_t have = 0;
  switch (what) {
    case 0: src = centroids_.p; have = centroids_.bytes(); break;
    case 1: src = codebooks_.p; have = codebooks_.bytes(); break;
    case 2: src = pq_codes_.p; have = pq_codes_.bytes(); break;
    case 3: src = sq_mins_.p; have = sq_mins_.bytes(); break;
    case 4: src = sq_scales_.p; have = sq_scales_.bytes(); break;
    case 5: src = sq_codes_.p; have = sq_codes_.bytes(); break;
    case 6: src = offsets_.p; have = offsets_.bytes(); break;
    case 7: src = vec_ids_.p; have = vec_ids_.bytes(); break;
    case 8: src = rq_signs_.p; have = rq_signs_.bytes(); break;
    case 9: src = rq_cent_.p; have = rq_cent_.bytes(); break;
    case 10: src = rq_bits_.p; have = rq_bits_.bytes(); break;
    case 11: src = rq_meta_.p; have = rq_meta_.bytes(); break;
    default: return FV_ERR_ARG;
  }
  if (!host_out || bytes < have) return FV_ERR_ARG;
  if (have == 0) return 0;
  return (int)cudaMemcpy(host_out, src, have, cudaMemcpyDeviceToHost);
}

}  // namespace fv

// ------------------------------------------------------------------ C ABI
struct FvIndex {
  fv::Index impl;
  explicit FvIndex(const FvIndexConfig& c) : impl(c) {}
};

namespace fv {
Index* index_of(FvIndex* handle) { return handle ? &handle->impl : nullptr; }
uint32_t index_dim(const Index* index) { return index->dim(); }
int index_metric(const Index* index) { return index->metric(); }
bool index_built(const Index* index) { return index->built(); }
void index_prepare_queries(const Index* index, float* rows, uint32_t n) {
  if (index->metric() == METRIC_COSINE) normalize_rows(rows, n, index->dim());
}
uint32_t index_nlist(const Index* index) { return index->nlist(); }
void index_pin(Index* index) { index->pin(); }
void index_unpin(Index* index) { index->unpin(); }
int index_launch_batch(Index* index, const BatchLaunch& b, cudaStream_t stream) { return index->launch_batch(b, stream); }
size_t index_batch_scratch_bytes(const Index* index, const BatchLaunch& b) { return index->batch_scratch_bytes(b); }
}  // namespace fv

extern "C" {

int fv_index_create(const FvIndexConfig* config, FvIndex** out) {
  if (!config || !out) return FV_ERR_NULL;
  if (config->dim == 0 || config->dim > 4096 || config->metric > 2) return FV_ERR_ARG;
  try {
    *out = new FvIndex(*config);
  } catch (...) {
    return FV_ERR_NOMEM;
  }
  return 0;
}
int fv_index_destroy(FvIndex* index) {
  delete index;
  return 0;
}
int fv_index_build(FvIndex* index, const float* host_vectors, uint32_t num_vectors) {
  if (!index) return FV_ERR_NULL;
  return index->impl.build(host_vectors, num_vectors);
}
int fv_index_build_device(FvIndex* index, const float* d_vectors, uint32_t num_vectors,
                          const float* d_init_centroids) {
  if (!index) return FV_ERR_NULL;
  return index->impl.build_device(d_vectors, num_vectors, d_init_centroids);
}
int fv_index_add(FvIndex* index, const float* host_vectors, uint32_t num_vectors, uint32_t* out_ids) {
  if (!index) return FV_ERR_NULL;
  return index->impl.add(host_vectors, num_vectors, out_ids);
}
int fv_index_delete(FvIndex* index, const uint32_t* ids, uint32_t count, uint32_t* out_deleted) {
  if (!index) return FV_ERR_NULL;
  return index->impl.remove(ids, count, out_deleted);
}
int fv_index_search(FvIndex* index, const FvSearchParams* params, const float* host_queries, uint32_t num_queries,
                    const uint32_t* host_mask_words, uint32_t mask_words, GpuSearchResult* host_out) {
  if (!index || !params) return FV_ERR_NULL;
  return index->impl.search(*params, host_queries, num_queries, false, host_mask_words, mask_words, host_out);
}
int fv_index_search_device(FvIndex* index, const FvSearchParams* params, const float* d_queries, uint32_t num_queries,
                           GpuSearchResult* host_out) {
  if (!index || !params) return FV_ERR_NULL;
  return index->impl.search(*params, d_queries, num_queries, true, nullptr, 0, host_out);
}
int fv_index_stats(FvIndex* index, FvLatencyStats* out) {
  if (!index || !out) return FV_ERR_NULL;
  index->impl.stats(out);
  return 0;
}
int fv_index_info(FvIndex* index, FvIndexInfo* out) {
  if (!index || !out) return FV_ERR_NULL;
  index->impl.info(out);
  return 0;
}
int fv_index_ivf_tables(FvIndex* index, IvfPqGpuTables* pq, IvfSqGpuTables* sq, FvIvfOptions* options) {
  if (!index) return FV_ERR_NULL;
  return index->impl.tables(pq, sq, options);
}
int fv_index_rabitq_tables(FvIndex* index, IvfRabitqGpuTables* rabitq, FvIvfOptions* options) {
  if (!index) return FV_ERR_NULL;
  return index->impl.rabitq_tables(rabitq, options);
}
int fv_index_export_ivf(FvIndex* index, uint32_t table, void* host_out, size_t bytes) {
  if (!index) return FV_ERR_NULL;
  return index->impl.export_ivf(table, host_out, bytes);
}

namespace {
thread_local std::string g_snapshot_error;
}

int fv_index_save_snapshot(FvIndex* index, const char* path) {
  if (!index || !path) return FV_ERR_NULL;
  g_snapshot_error.clear();
  return index->impl.save_snapshot(path, &g_snapshot_error);
}

int fv_index_load_snapshot(const char* path, const FvIndexConfig* config, FvIndex** out) {
  if (!path || !out) return FV_ERR_NULL;
  g_snapshot_error.clear();
  fv::snap::File f;
  int rc = f.open(path, &g_snapshot_error);
  if (rc) return rc;
  const fv::snap::Manifest& m = f.manifest();
  if (m.dim == 0 || m.dim > 4096 || m.metric > 2) {
    g_snapshot_error = "snapshot config out of range";
    return FV_ERR_ARG;
  }
  FvIndexConfig c{};
  if (config) c = *config;
  c.dim = m.dim;
  c.metric = m.metric;
  c.nlist = m.nlist;
  c.m_pq = m.m_pq;
  if (c.build_flags == 0) c.build_flags = fv::kDefaultBuild;
  FvIndex* idx = nullptr;
  try {
    idx = new FvIndex(c);
  } catch (...) {
    return FV_ERR_NOMEM;
  }
  rc = idx->impl.load_snapshot(f, &g_snapshot_error);
  if (rc) {
    delete idx;
    return rc;
  }
  *out = idx;
  return 0;
}

int fv_snapshot_inspect(const char* path, char* manifest_json, size_t len, size_t* needed) {
  if (!path) return FV_ERR_NULL;
  g_snapshot_error.clear();
  fv::snap::File f;
  const int rc = f.open(path, &g_snapshot_error);
  if (rc) return rc;
  const std::string j = fv::snap::manifest_to_json(f.manifest());
  if (needed) *needed = j.size() + 1;
  if (manifest_json && len) {
    const size_t c = std::min(len - 1, j.size());
    std::memcpy(manifest_json, j.data(), c);
    manifest_json[c] = 0;
  }
  return 0;
}

const char* fv_snapshot_error(void) { return g_snapshot_error.c_str(); }

}  // extern "C"
