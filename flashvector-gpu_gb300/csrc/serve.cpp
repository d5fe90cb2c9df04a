// serve.cpp -- continuous-batching request loop (fv_serve_*, include/fv_serve.h).
//
// The reference's SearchBatcher (crates/server/src/batcher.rs:82-259)
// restated for one GPU with several batches in flight:
//
//   submit      -> the request (query copied, cosine rows normalised) joins
//                  the queue of its launch class;
//   batcher     -> one thread; picks the class whose oldest request is
//                  oldest and launches up to max_batch of its requests on a
//                  free stream when the GPU is idle, the class is full, or
//                  the oldest request has waited max_wait_us;
//   launch      -> one pinned staging block (queries, per-query k / nprobe /
//                  rerank_k, per-query filter rows) -> one H2D copy -> the
//                  engine's batch launch (main scan, delta scan, merge) ->
//                  one D2H copy -> a host function that hands the slot to
//                  the completion thread;
//   completion  -> copies each request's results out of the pinned block,
//                  stamps completion, wakes waiters, frees the stream.
//
// Launch classes: (engine, top_k) for the flat and tensor-core engines;
// (engine) for IVF, whose kernel takes per-query k / nprobe / rerank_k;
// (engine, top_k, nprobe, rerank_k) with group_by_params (the reference's
// BatchKey, batcher.rs:55-61). Filters never split a batch: each query
// carries its own filter row.
#include <algorithm>
#include <atomic>
#include <chrono>
#include <cmath>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <new>
#include <thread>
#include <tuple>
#include <unordered_map>
#include <vector>

#include "../../include/fv_serve.h"
#include "engine.h"
#include "kernels.h"

namespace fv {

class Server;

namespace {

constexpr uint32_t kMaxTopK = 256;  // reference clamp (streams.rs:14)
constexpr size_t kDefaultScratchBudget = (size_t)512 << 20;  // FvServeConfig.scratch_budget_kb = 0
constexpr size_t kGraphsPerSlot = 64;  // executable graphs kept per stream (FvServeConfig.graphs)

uint64_t now_ns() {
  return (uint64_t)std::chrono::duration_cast<std::chrono::nanoseconds>(
             std::chrono::steady_clock::now().time_since_epoch())
      .count();
}

std::chrono::steady_clock::time_point at_ns(uint64_t t) {
  return std::chrono::steady_clock::time_point(
      std::chrono::duration_cast<std::chrono::steady_clock::duration>(std::chrono::nanoseconds(t)));
}

size_t align_up(size_t v, size_t a) { return (v + a - 1) / a * a; }

struct Filter {
  std::vector<uint32_t> words;
  uint32_t* d_words = nullptr;  // device copy (index-backed servers)
  ~Filter() {
    if (d_words) cudaFree(d_words);
  }
};

struct Req {
  FvRequest p{};
  uint64_t ticket = 0;
  uint64_t arrival = 0, launch = 0, done = 0;
  std::vector<float> q;
  std::shared_ptr<Filter> filter;
  std::vector<GpuSearchResult> res;
  int status = 0;
  bool finished = false;
};

struct ClassKey {
  uint32_t engine, top_k, nprobe, rerank;
  bool operator<(const ClassKey& o) const {
    return std::tie(engine, top_k, nprobe, rerank) < std::tie(o.engine, o.top_k, o.nprobe, o.rerank);
  }
};

bool is_ivf(uint32_t engine) {
  return engine == FV_ENGINE_IVF_PQ || engine == FV_ENGINE_IVF_SQ8 || engine == FV_ENGINE_IVF_RABITQ;
}

// Staging layout of one batch of nq requests (one contiguous block, so one
// copy each way): queries | top_k | nprobe | rerank_k | filters.
struct Layout {
  size_t q, topk, nprobe, rerank, filt, total;
  Layout(uint32_t nq, uint32_t dim) {
    q = 0;
    topk = align_up((size_t)nq * dim * 4, 256);
    nprobe = topk + align_up((size_t)nq * 4, 256);
    rerank = nprobe + align_up((size_t)nq * 4, 256);
    filt = rerank + align_up((size_t)nq * 4, 256);
    total = filt + align_up((size_t)nq * sizeof(QueryFilter), 256);
  }
};

struct Slot {
  Server* srv = nullptr;
  int idx = 0;
  cudaStream_t stream = nullptr;
  uint8_t* h_in = nullptr;  // pinned staging
  GpuSearchResult* h_out = nullptr;
  uint8_t* d_in = nullptr;
  GpuSearchResult* d_out = nullptr;
  GpuSearchResult* d_main = nullptr;
  GpuSearchResult* d_delta = nullptr;
  std::vector<Req*> reqs;
  uint32_t kstride = 0;
  bool pinned_index = false;
  // this batch's part of the server's scratch pool (index-backed servers)
  size_t scratch_off = 0, scratch_bytes = 0;
  // FvServeConfig.graphs: executable graphs of this stream's batches by
  // launch shape (engine, nq, k, nprobe, rerank_k, filtered)
  std::map<std::tuple<uint32_t, uint32_t, uint32_t, uint32_t, uint32_t, bool>, cudaGraphExec_t> graphs;
  // executor-backed servers: a worker thread per slot
  std::vector<float> x_q;
  std::vector<FvRequest> x_reqs;
  std::vector<GpuSearchResult> x_out;
  std::thread worker;
  std::mutex wmu;
  std::condition_variable wcv;
  bool has_work = false;
  bool quit = false;
};

}  // namespace

class Server {
 public:
  Server(Index* index, uint32_t dim, const FvServeConfig& c, FvServeExecutor ex, void* user)
      : index_(index), dim_(dim), cfg_(c), exec_(ex), user_(user) {
    if (cfg_.max_batch == 0) cfg_.max_batch = 256;
    if (cfg_.inflight == 0) cfg_.inflight = 4;
    max_wait_ns_ = (uint64_t)cfg_.max_wait_us * 1000ull;
    pool_bytes_ = cfg_.scratch_budget_kb ? (size_t)cfg_.scratch_budget_kb * 1024 : kDefaultScratchBudget;
    pool_bytes_ = pool_bytes_ / 256 * 256;
  }

  int init() {
    const Layout lay(cfg_.max_batch, dim_);
    if (index_) {
      // the scratch pool every batch in flight takes its part of
      if (pool_bytes_ < 256) return FV_ERR_ARG;
      cudaError_t e = cudaMalloc(reinterpret_cast<void**>(&pool_), pool_bytes_);
      if (e != cudaSuccess) return (int)e;
      pool_free_[0] = pool_bytes_;
    }
    const size_t out_n = (size_t)cfg_.max_batch * kMaxTopK;
    slots_.resize(cfg_.inflight);
    for (uint32_t i = 0; i < cfg_.inflight; ++i) {
      slots_[i] = std::make_unique<Slot>();
      Slot* s = slots_[i].get();
      s->srv = this;
      s->idx = (int)i;
      if (index_) {
        cudaError_t e = cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking);
        if (e == cudaSuccess) e = cudaMallocHost(reinterpret_cast<void**>(&s->h_in), lay.total);
        if (e == cudaSuccess) e = cudaMallocHost(reinterpret_cast<void**>(&s->h_out), out_n * sizeof(GpuSearchResult));
        if (e == cudaSuccess) e = cudaMalloc(reinterpret_cast<void**>(&s->d_in), lay.total);
        if (e == cudaSuccess) e = cudaMalloc(reinterpret_cast<void**>(&s->d_out), 3 * out_n * sizeof(GpuSearchResult));
        if (e != cudaSuccess) return (int)e;
        s->d_main = s->d_out + out_n;
        s->d_delta = s->d_out + 2 * out_n;
      } else {
        s->worker = std::thread([this, s] { worker_loop(s); });
      }
      free_slots_.push_back((int)i);
    }
    if (index_) completion_ = std::thread([this] { completion_loop(); });
    batcher_ = std::thread([this] { batcher_loop(); });
    return 0;
  }

  ~Server() {
    {
      std::unique_lock<std::mutex> lk(mu_);
      stop_ = true;
      work_cv_.notify_all();
    }
    if (batcher_.joinable()) batcher_.join();
    {
      std::unique_lock<std::mutex> lk(mu_);
      req_cv_.wait(lk, [&] { return inflight_ == 0; });
    }
    {
      std::lock_guard<std::mutex> g(cb_mu_);
      cb_stop_ = true;
      cb_cv_.notify_all();
    }
    if (completion_.joinable()) completion_.join();
    for (auto& sp : slots_) {
      Slot* s = sp.get();
      if (s->worker.joinable()) {
        {
          std::lock_guard<std::mutex> g(s->wmu);
          s->quit = true;
          s->wcv.notify_all();
        }
        s->worker.join();
      }
      if (s->stream) {
        cudaStreamSynchronize(s->stream);
        for (auto& kv : s->graphs) cudaGraphExecDestroy(kv.second);
        fv_release_stream_scratch(s->stream);
        cudaStreamDestroy(s->stream);
      }
      if (s->h_in) cudaFreeHost(s->h_in);
      if (s->h_out) cudaFreeHost(s->h_out);
      if (s->d_in) cudaFree(s->d_in);
      if (s->d_out) cudaFree(s->d_out);
    }
    if (pool_) cudaFree(pool_);
  }

  // The scratch bytes one batch of `nq` requests takes: the plan of the
  // launches index_launch_batch makes (rounded as the stream arena rounds).
  size_t batch_scratch(uint32_t engine, uint32_t nq, uint32_t kmax, uint32_t npmax, uint32_t rrmax) const {
    static const uint32_t kPresent = 0;  // marks the per-query arrays as present; never read
    BatchLaunch b;
    b.engine = engine;
    b.nq = nq;
    b.top_k = kmax;
    b.nprobe = npmax;
    b.rerank_k = rrmax;
    if (is_ivf(engine)) b.d_topk = b.d_nprobe = b.d_rerank = &kPresent;
    const size_t need = index_batch_scratch_bytes(index_, b);
    return (std::max<size_t>(need, 256) + 255) / 256 * 256;
  }

  int scratch_estimate(const FvRequest* rq, uint32_t nq, uint64_t* out) {
    if (!rq || !out) return FV_ERR_NULL;
    if (!index_) {
      *out = 0;
      return 0;
    }
    if (rq->engine > FV_ENGINE_IVF_RABITQ || rq->top_k == 0 || rq->top_k > (uint32_t)kMaxTopK || nq == 0)
      return FV_ERR_ARG;
    index_pin(index_);
    *out = batch_scratch(rq->engine, nq, rq->top_k, rq->nprobe, rq->rerank_k);
    index_unpin(index_);
    return 0;
  }

  // ------------------------------------------------------------ filters
  int add_filter(const uint32_t* words, uint32_t nwords, int32_t* out_id) {
    if (!out_id || (nwords && !words)) return FV_ERR_NULL;
    auto f = std::make_shared<Filter>();
    f->words.assign(words, words + nwords);
    if (index_ && nwords) {
      cudaError_t e = cudaMalloc(reinterpret_cast<void**>(&f->d_words), (size_t)nwords * 4);
      if (e == cudaSuccess) e = cudaMemcpy(f->d_words, words, (size_t)nwords * 4, cudaMemcpyHostToDevice);
      if (e != cudaSuccess) return (int)e;
    }
    std::lock_guard<std::mutex> g(mu_);
    const int32_t id = next_filter_++;
    filters_[id] = std::move(f);
    *out_id = id;
    return 0;
  }

  int remove_filter(int32_t id) {
    std::lock_guard<std::mutex> g(mu_);
    return filters_.erase(id) ? 0 : FV_ERR_ARG;
  }

  // ------------------------------------------------------------- submit
  int submit(const FvRequest* rq, const float* q, uint64_t arrival, uint64_t* ticket) {
    if (!rq || !q || !ticket) return FV_ERR_NULL;
    if (rq->engine > FV_ENGINE_IVF_RABITQ || rq->top_k == 0 || rq->top_k > (uint32_t)kMaxTopK) return FV_ERR_ARG;
    if (index_) {
      if (!index_built(index_)) return FV_ERR_ARG;
      if (is_ivf(rq->engine)) {
        const uint32_t nl = index_nlist(index_);
        const uint32_t np = rq->nprobe == 0 ? 1u : rq->nprobe;
        if (std::min(np, nl) > (uint32_t)kMaxTopK) return FV_ERR_ARG;  // coarse selection keeps <= 256 lists
      }
    }
    auto r = std::make_unique<Req>();
    r->p = *rq;
    r->q.assign(q, q + dim_);
    if (index_) index_prepare_queries(index_, r->q.data(), 1);
    const uint64_t t = arrival ? arrival : now_ns();
    std::lock_guard<std::mutex> g(mu_);
    if (rq->filter_id >= 0) {
      auto it = filters_.find(rq->filter_id);
      if (it == filters_.end()) return FV_ERR_ARG;
      r->filter = it->second;
    }
    if (cfg_.queue_capacity && pending_ >= cfg_.queue_capacity) return FV_ERR_QUEUE_FULL;
    r->arrival = t;
    r->ticket = next_ticket_++;
    classes_[class_of(r->p)].push_back(r.get());
    *ticket = r->ticket;
    tickets_[r->ticket] = std::move(r);
    ++pending_;
    work_cv_.notify_one();
    return 0;
  }

  int wait(uint64_t ticket, GpuSearchResult* out, uint32_t out_len, uint32_t timeout_ms, double* latency_us) {
    std::unique_lock<std::mutex> lk(mu_);
    auto it = tickets_.find(ticket);
    if (it == tickets_.end()) return FV_ERR_ARG;
    Req* r = it->second.get();
    if (timeout_ms) {
      if (!req_cv_.wait_for(lk, std::chrono::milliseconds(timeout_ms), [&] { return r->finished; }))
        return FV_ERR_TIMEOUT;
    } else {
      req_cv_.wait(lk, [&] { return r->finished; });
    }
    const int st = r->status;
    if (out && st == 0) {
      const uint32_t n = std::min<uint32_t>(out_len, (uint32_t)r->res.size());
      std::memcpy(out, r->res.data(), (size_t)n * sizeof(GpuSearchResult));
    }
    if (latency_us) *latency_us = (double)(r->done - r->arrival) / 1e3;
    tickets_.erase(it);
    return st;
  }

  int replay(const FvRequest* reqs, const float* queries, const uint64_t* arrival, uint32_t n, GpuSearchResult* out,
             uint32_t stride, int32_t* status) {
    if (n == 0) return 0;
    if (!reqs || !queries || !arrival || !out) return FV_ERR_NULL;
    for (uint32_t i = 0; i < n; ++i) {
      if (i && arrival[i] < arrival[i - 1]) return FV_ERR_ARG;
      if (reqs[i].top_k > stride) return FV_ERR_ARG;
    }
    std::vector<uint64_t> tickets(n, 0);
    std::vector<int> rc(n, 0);
    const uint64_t start = now_ns() + 200000;  // 0.2 ms lead
    for (uint32_t i = 0; i < n; ++i) {
      const uint64_t t = start + arrival[i];
      for (uint64_t x = now_ns(); x < t; x = now_ns()) {
        if (t - x > 200000) std::this_thread::sleep_for(std::chrono::microseconds(50));
      }
      rc[i] = submit(&reqs[i], queries + (size_t)i * dim_, t, &tickets[i]);
    }
    int first = 0;
    for (uint32_t i = 0; i < n; ++i) {
      if (rc[i] == 0) rc[i] = wait(tickets[i], out + (size_t)i * stride, reqs[i].top_k, 0, nullptr);
      if (status) status[i] = rc[i];
      if (rc[i] && !first) first = rc[i];
    }
    return status ? 0 : first;
  }

  // -------------------------------------------------------------- stats
  void stats(FvServeStats* s) {
    std::lock_guard<std::mutex> g(mu_);
    *s = FvServeStats{};
    s->total_requests = total_requests_;
    s->total_batches = total_batches_;
    s->avg_batch_size = total_batches_ ? (double)total_requests_ / (double)total_batches_ : 0.0;
    s->completed = completed_;
    s->failed = failed_;
    s->max_inflight = max_inflight_;
    s->graph_instantiations = graph_instantiations_.load(std::memory_order_relaxed);
    s->graph_fallbacks = graph_fallbacks_.load(std::memory_order_relaxed);
    if (completed_ && last_done_ > first_arrival_)
      s->qps = (double)completed_ / ((double)(last_done_ - first_arrival_) / 1e9);
    auto pct = [](std::vector<double> v, double* p50, double* p90, double* p99, double* p999, double* mx,
                  double* mean) {
      if (v.empty()) return;
      std::sort(v.begin(), v.end());
      const size_t n = v.size();
      auto at = [&](double f) { return v[std::min(n - 1, (size_t)((double)n * f))]; };
      *p50 = at(0.5);
      if (p90) *p90 = at(0.9);
      *p99 = at(0.99);
      if (p999) *p999 = at(0.999);
      if (mx) *mx = v.back();
      if (mean) {
        double sum = 0;
        for (double x : v) sum += x;
        *mean = sum / (double)n;
      }
    };
    s->scratch_waits = scratch_waits_;
    s->scratch_split = scratch_split_;
    s->scratch_peak_bytes = pool_peak_;
    s->scratch_pool_bytes = index_ ? pool_bytes_ : 0;
    pct(lat_us_, &s->p50_us, &s->p90_us, &s->p99_us, &s->p999_us, &s->max_us, &s->mean_us);
    pct(queue_us_, &s->queue_p50_us, nullptr, &s->queue_p99_us, nullptr, nullptr, nullptr);
  }

  void reset_stats() {
    std::lock_guard<std::mutex> g(mu_);
    total_requests_ = total_batches_ = completed_ = failed_ = 0;
    max_inflight_ = 0;
    scratch_waits_ = scratch_split_ = 0;
    pool_peak_ = pool_used_;
    first_arrival_ = UINT64_MAX;
    last_done_ = 0;
    lat_us_.clear();
    queue_us_.clear();
  }

  void host_done(Slot* s) {
    std::lock_guard<std::mutex> g(cb_mu_);
    done_q_.push_back(s);
    cb_cv_.notify_one();
  }

 private:
  ClassKey class_of(const FvRequest& p) const {
    if (cfg_.group_by_params) return ClassKey{p.engine, p.top_k, p.nprobe, p.rerank_k};
    if (is_ivf(p.engine)) return ClassKey{p.engine, 0, 0, 0};
    return ClassKey{p.engine, p.top_k, 0, 0};
  }

  // First-fit allocator over the scratch pool (offsets and sizes in
  // multiples of 256 bytes); called with mu_ held. SIZE_MAX: no room.
  size_t pool_alloc(size_t bytes) {
    for (auto it = pool_free_.begin(); it != pool_free_.end(); ++it) {
      if (it->second < bytes) continue;
      const size_t off = it->first, left = it->second - bytes;
      pool_free_.erase(it);
      if (left) pool_free_[off + bytes] = left;
      pool_used_ += bytes;
      pool_peak_ = std::max(pool_peak_, pool_used_);
      return off;
    }
    return SIZE_MAX;
  }

  void pool_release(size_t off, size_t bytes) {
    pool_used_ -= bytes;
    auto it = pool_free_.emplace(off, bytes).first;
    auto next = std::next(it);
    if (next != pool_free_.end() && it->first + it->second == next->first) {
      it->second += next->second;
      pool_free_.erase(next);
    }
    if (it != pool_free_.begin()) {
      auto prev = std::prev(it);
      if (prev->first + prev->second == it->first) {
        prev->second += it->second;
        pool_free_.erase(it);
      }
    }
  }

  // Fails the oldest request of a class without launching it; mu_ held.
  void reject_front(std::deque<Req*>* q, int rc) {
    Req* r = q->front();
    q->pop_front();
    --pending_;
    r->status = rc;
    r->done = now_ns();
    r->finished = true;
    ++failed_;
    req_cv_.notify_all();
  }

  void batcher_loop() {
    std::unique_lock<std::mutex> lk(mu_);
    while (true) {
      if (pending_ == 0) {
        if (stop_) break;
        work_cv_.wait(lk);
        continue;
      }
      if (free_slots_.empty()) {
        work_cv_.wait(lk);
        continue;
      }
      // the class with the oldest waiting request, unless one is full
      const uint64_t now = now_ns();
      std::deque<Req*>* pick = nullptr;
      ClassKey key{};
      bool go = false;
      for (auto& kv : classes_) {
        auto& dq = kv.second;
        if (dq.empty()) continue;
        if (dq.size() >= cfg_.max_batch) {
          pick = &dq;
          key = kv.first;
          go = true;
          break;
        }
        if (!pick || dq.front()->arrival < pick->front()->arrival) {
          pick = &dq;
          key = kv.first;
        }
      }
      const uint64_t due = pick->front()->arrival + max_wait_ns_;
      if (!go) go = stop_ || inflight_ == 0 || now >= due;
      if (!go) {
        work_cv_.wait_until(lk, at_ns(due));
        continue;
      }
      size_t n = std::min<size_t>(pick->size(), cfg_.max_batch);
      size_t off = 0, need = 0;
      if (index_) {
        // admission by scratch memory: the batch's exact scratch must fit
        // in the free part of the pool; a batch larger than the whole pool
        // is cut down; a single request larger than it fails
        index_pin(index_);  // the estimate and the launch see one index state
        auto estimate = [&](size_t cnt) {
          uint32_t kmax = 0, npmax = 0, rrmax = 0;
          for (size_t i = 0; i < cnt; ++i) {
            const FvRequest& p = (*pick)[i]->p;
            kmax = std::max(kmax, p.top_k);
            npmax = std::max(npmax, p.nprobe);
            rrmax = std::max(rrmax, p.rerank_k);
          }
          return batch_scratch(key.engine, (uint32_t)cnt, kmax, npmax, rrmax);
        };
        need = estimate(n);
        const size_t asked = n;
        while (need > pool_bytes_ && n > 1) {
          n = (n + 1) / 2;
          need = estimate(n);
        }
        if (n < asked) ++scratch_split_;
        if (need > pool_bytes_) {
          index_unpin(index_);
          reject_front(pick, FV_ERR_SCRATCH_LIMIT);
          continue;
        }
        off = pool_alloc(need);
        if (off == SIZE_MAX) {
          index_unpin(index_);
          ++scratch_waits_;
          work_cv_.wait(lk);  // a finishing batch returns its part of the pool
          continue;
        }
      }
      const int si = free_slots_.back();
      free_slots_.pop_back();
      Slot* s = slots_[si].get();
      s->scratch_off = off;
      s->scratch_bytes = need;
      s->pinned_index = index_ != nullptr;
      s->reqs.assign(pick->begin(), pick->begin() + n);
      pick->erase(pick->begin(), pick->begin() + n);
      pending_ -= n;
      ++inflight_;
      max_inflight_ = std::max<uint32_t>(max_inflight_, inflight_);
      ++total_batches_;
      total_requests_ += n;
      for (Req* r : s->reqs) r->launch = now;
      lk.unlock();
      launch(s, key);
      lk.lock();
    }
  }

  void launch(Slot* s, const ClassKey& key) {
    const uint32_t nq = (uint32_t)s->reqs.size();
    uint32_t kmax = 0, npmax = 0, rrmax = 0;
    for (Req* r : s->reqs) {
      kmax = std::max(kmax, r->p.top_k);
      npmax = std::max(npmax, r->p.nprobe);
      rrmax = std::max(rrmax, r->p.rerank_k);
    }
    s->kstride = kmax;
    if (!index_) {
      std::lock_guard<std::mutex> g(s->wmu);
      s->x_q.resize((size_t)nq * dim_);
      s->x_reqs.resize(nq);
      for (uint32_t i = 0; i < nq; ++i) {
        std::memcpy(s->x_q.data() + (size_t)i * dim_, s->reqs[i]->q.data(), (size_t)dim_ * 4);
        s->x_reqs[i] = s->reqs[i]->p;
      }
      s->x_out.assign((size_t)nq * kmax, GpuSearchResult{0xFFFFFFFFu, 1e30f});
      s->has_work = true;
      s->wcv.notify_one();
      return;
    }
    const Layout lay(nq, dim_);
    float* hq = reinterpret_cast<float*>(s->h_in + lay.q);
    uint32_t* hk = reinterpret_cast<uint32_t*>(s->h_in + lay.topk);
    uint32_t* hn = reinterpret_cast<uint32_t*>(s->h_in + lay.nprobe);
    uint32_t* hr = reinterpret_cast<uint32_t*>(s->h_in + lay.rerank);
    QueryFilter* hf = reinterpret_cast<QueryFilter*>(s->h_in + lay.filt);
    bool any_filter = false;
    for (uint32_t i = 0; i < nq; ++i) {
      const Req* r = s->reqs[i];
      std::memcpy(hq + (size_t)i * dim_, r->q.data(), (size_t)dim_ * 4);
      hk[i] = r->p.top_k;
      hn[i] = r->p.nprobe;
      hr[i] = r->p.rerank_k;
      const Filter* f = r->filter.get();
      // an empty registered filter allows nothing: a non-null row of 0
      // words (the kernels test the word count before any load, so the
      // placeholder address is never dereferenced)
      static const uint32_t kNone = 0;
      hf[i] = f ? QueryFilter{f->d_words ? f->d_words : &kNone, (uint32_t)f->words.size(), 0u}
                : QueryFilter{nullptr, 0u, 0u};
      if (f) any_filter = true;
    }
    BatchLaunch b;
    b.engine = key.engine;
    b.nq = nq;
    b.top_k = kmax;
    b.nprobe = npmax;
    b.rerank_k = rrmax;
    b.d_queries = reinterpret_cast<const float*>(s->d_in + lay.q);
    if (is_ivf(key.engine)) {
      b.d_topk = reinterpret_cast<const uint32_t*>(s->d_in + lay.topk);
      b.d_nprobe = reinterpret_cast<const uint32_t*>(s->d_in + lay.nprobe);
      b.d_rerank = reinterpret_cast<const uint32_t*>(s->d_in + lay.rerank);
    }
    b.d_filters = any_filter ? reinterpret_cast<const QueryFilter*>(s->d_in + lay.filt) : nullptr;
    b.d_out = s->d_out;
    b.d_main = s->d_main;
    b.d_delta = s->d_delta;
    // the batch's part of the pool is the stream's scratch arena for its
    // launches (the batch before it on this stream has completed)
    int rc = fv_set_stream_scratch(s->stream, pool_ + s->scratch_off, s->scratch_bytes);
    if (!rc) rc = (int)cudaMemcpyAsync(s->d_in, s->h_in, lay.total, cudaMemcpyHostToDevice, s->stream);
    if (!rc) rc = cfg_.graphs ? launch_graph(s, b, any_filter) : index_launch_batch(index_, b, s->stream);
    if (!rc)
      rc = (int)cudaMemcpyAsync(s->h_out, s->d_out, (size_t)nq * kmax * sizeof(GpuSearchResult),
                                cudaMemcpyDeviceToHost, s->stream);
    if (!rc) rc = (int)cudaLaunchHostFunc(s->stream, &Server::host_fn, s);
    if (rc) {
      cudaStreamSynchronize(s->stream);  // nothing enqueued may still use the staging
      complete(s, rc);
    }
  }

  // The batch's kernels as one CUDA graph: captured on the slot's stream
  // (thread-local capture: the other threads' CUDA calls are unaffected),
  // then applied to the slot's executable graph of the same launch shape by
  // cudaGraphExecUpdate (same kernels; new pointers, scratch and sizes), or
  // instantiated when the shape is new or the update is refused. The slot's
  // previous batch has completed, so its graphs are idle.
  int launch_graph(Slot* s, const BatchLaunch& b, bool any_filter) {
    cudaGraph_t g = nullptr;
    cudaError_t e = cudaStreamBeginCapture(s->stream, cudaStreamCaptureModeThreadLocal);
    if (e != cudaSuccess) return (int)e;
    const int rc = index_launch_batch(index_, b, s->stream);
    e = cudaStreamEndCapture(s->stream, &g);
    if (rc || e != cudaSuccess) {
      // a capture the driver invalidated (the first launch of a kernel in
      // the process loads its module, which a capture does not allow) runs
      // as plain launches; later batches of the shape are captured
      if (g) cudaGraphDestroy(g);
      (void)cudaGetLastError();
      graph_fallbacks_.fetch_add(1, std::memory_order_relaxed);
      return index_launch_batch(index_, b, s->stream);
    }
    const auto key = std::make_tuple(b.engine, b.nq, b.top_k, b.nprobe, b.rerank_k, any_filter);
    auto it = s->graphs.find(key);
    cudaGraphExec_t ex = nullptr;
    if (it != s->graphs.end()) {
      cudaGraphExecUpdateResultInfo info{};
      if (cudaGraphExecUpdate(it->second, g, &info) == cudaSuccess) {
        ex = it->second;
      } else {
        (void)cudaGetLastError();  // the refused update leaves no sticky error
        cudaGraphExecDestroy(it->second);
        s->graphs.erase(it);
      }
    }
    if (!ex) {
      if (s->graphs.size() >= kGraphsPerSlot) {
        cudaGraphExecDestroy(s->graphs.begin()->second);
        s->graphs.erase(s->graphs.begin());
      }
      e = cudaGraphInstantiate(&ex, g, 0);
      if (e != cudaSuccess) {
        cudaGraphDestroy(g);
        return (int)e;
      }
      s->graphs[key] = ex;
      graph_instantiations_.fetch_add(1, std::memory_order_relaxed);
    }
    cudaGraphDestroy(g);
    return (int)cudaGraphLaunch(ex, s->stream);
  }

  static void CUDART_CB host_fn(void* p) {
    Slot* s = static_cast<Slot*>(p);
    s->srv->host_done(s);
  }

  void completion_loop() {
    std::unique_lock<std::mutex> lk(cb_mu_);
    while (true) {
      cb_cv_.wait(lk, [&] { return cb_stop_ || !done_q_.empty(); });
      if (done_q_.empty()) break;
      Slot* s = done_q_.front();
      done_q_.pop_front();
      lk.unlock();
      complete(s, 0);
      lk.lock();
    }
  }

  void worker_loop(Slot* s) {
    std::unique_lock<std::mutex> lk(s->wmu);
    while (true) {
      s->wcv.wait(lk, [&] { return s->quit || s->has_work; });
      if (!s->has_work) break;
      s->has_work = false;
      const uint32_t nq = (uint32_t)s->x_reqs.size();
      lk.unlock();
      int rc = exec_ ? exec_(user_, s->x_reqs.data(), s->x_q.data(), nq, dim_, s->kstride, s->x_out.data())
                     : FV_ERR_NULL;
      complete(s, rc);
      lk.lock();
    }
  }

  void complete(Slot* s, int rc) {
    const uint64_t t = now_ns();
    if (s->pinned_index) {
      index_unpin(index_);
      s->pinned_index = false;
    }
    const GpuSearchResult* src = index_ ? s->h_out : s->x_out.data();
    for (size_t i = 0; i < s->reqs.size(); ++i) {
      Req* r = s->reqs[i];
      if (rc == 0) r->res.assign(src + i * s->kstride, src + i * s->kstride + r->p.top_k);
      r->status = rc;
      r->done = t;
    }
    {
      std::lock_guard<std::mutex> g(mu_);
      for (Req* r : s->reqs) {
        r->finished = true;
        if (rc) {
          ++failed_;
        } else {
          ++completed_;
          lat_us_.push_back((double)(t - r->arrival) / 1e3);
          queue_us_.push_back((double)(r->launch - r->arrival) / 1e3);
          first_arrival_ = std::min(first_arrival_, r->arrival);
          last_done_ = std::max(last_done_, t);
        }
      }
      s->reqs.clear();
      if (s->scratch_bytes) {
        pool_release(s->scratch_off, s->scratch_bytes);
        s->scratch_bytes = 0;
      }
      free_slots_.push_back(s->idx);
      --inflight_;
    }
    req_cv_.notify_all();
    work_cv_.notify_all();
  }

  Index* index_;
  uint32_t dim_;
  FvServeConfig cfg_;
  FvServeExecutor exec_;
  void* user_;
  uint64_t max_wait_ns_ = 0;

  std::mutex mu_;
  std::condition_variable work_cv_, req_cv_;
  bool stop_ = false;
  std::map<ClassKey, std::deque<Req*>> classes_;
  std::unordered_map<uint64_t, std::unique_ptr<Req>> tickets_;
  std::map<int32_t, std::shared_ptr<Filter>> filters_;
  int32_t next_filter_ = 0;
  uint64_t next_ticket_ = 1;
  size_t pending_ = 0;
  uint32_t inflight_ = 0;
  std::vector<std::unique_ptr<Slot>> slots_;
  std::vector<int> free_slots_;
  // scratch pool (index-backed servers): free ranges by offset
  uint8_t* pool_ = nullptr;
  size_t pool_bytes_ = 0, pool_used_ = 0, pool_peak_ = 0;
  std::map<size_t, size_t> pool_free_;
  uint64_t scratch_waits_ = 0, scratch_split_ = 0;

  uint64_t total_requests_ = 0, total_batches_ = 0, completed_ = 0, failed_ = 0;
  uint32_t max_inflight_ = 0;
  std::atomic<uint32_t> graph_instantiations_{0};
  std::atomic<uint64_t> graph_fallbacks_{0};
  uint64_t first_arrival_ = UINT64_MAX, last_done_ = 0;
  std::vector<double> lat_us_, queue_us_;

  std::mutex cb_mu_;
  std::condition_variable cb_cv_;
  std::deque<Slot*> done_q_;
  bool cb_stop_ = false;

  std::thread batcher_, completion_;
};

}  // namespace fv

struct FvServe {
  std::unique_ptr<fv::Server> impl;
};

extern "C" {

int fv_serve_create(FvIndex* index, const FvServeConfig* config, FvServe** out) {
  if (!index || !out) return FV_ERR_NULL;
  fv::Index* ix = fv::index_of(index);
  FvServeConfig c{};
  if (config) c = *config;
  auto h = new (std::nothrow) FvServe;
  if (!h) return FV_ERR_NOMEM;
  h->impl = std::make_unique<fv::Server>(ix, fv::index_dim(ix), c, nullptr, nullptr);
  const int rc = h->impl->init();
  if (rc) {
    delete h;
    return rc;
  }
  *out = h;
  return 0;
}

int fv_serve_create_with_executor(uint32_t dim, const FvServeConfig* config, FvServeExecutor executor, void* user,
                                  FvServe** out) {
  if (!executor || !out) return FV_ERR_NULL;
  if (dim == 0) return FV_ERR_ARG;
  FvServeConfig c{};
  if (config) c = *config;
  auto h = new (std::nothrow) FvServe;
  if (!h) return FV_ERR_NOMEM;
  h->impl = std::make_unique<fv::Server>(nullptr, dim, c, executor, user);
  const int rc = h->impl->init();
  if (rc) {
    delete h;
    return rc;
  }
  *out = h;
  return 0;
}

int fv_serve_destroy(FvServe* server) {
  delete server;
  return 0;
}

int fv_serve_add_filter(FvServe* server, const uint32_t* words, uint32_t num_words, int32_t* out_id) {
  if (!server) return FV_ERR_NULL;
  return server->impl->add_filter(words, num_words, out_id);
}

int fv_serve_remove_filter(FvServe* server, int32_t id) {
  if (!server) return FV_ERR_NULL;
  return server->impl->remove_filter(id);
}

int fv_serve_submit(FvServe* server, const FvRequest* request, const float* query, uint64_t* out_ticket) {
  if (!server) return FV_ERR_NULL;
  return server->impl->submit(request, query, 0, out_ticket);
}

int fv_serve_wait(FvServe* server, uint64_t ticket, GpuSearchResult* out, uint32_t out_len, uint32_t timeout_ms,
                  double* out_latency_us) {
  if (!server) return FV_ERR_NULL;
  return server->impl->wait(ticket, out, out_len, timeout_ms, out_latency_us);
}

int fv_serve_replay(FvServe* server, const FvRequest* requests, const float* queries, const uint64_t* arrival_ns,
                    uint32_t num_requests, GpuSearchResult* out, uint32_t out_stride, int32_t* out_status) {
  if (!server) return FV_ERR_NULL;
  return server->impl->replay(requests, queries, arrival_ns, num_requests, out, out_stride, out_status);
}

int fv_serve_scratch_estimate(FvServe* server, const FvRequest* request, uint32_t nq, uint64_t* out_bytes) {
  if (!server) return FV_ERR_NULL;
  return server->impl->scratch_estimate(request, nq, out_bytes);
}

int fv_serve_stats(FvServe* server, FvServeStats* out) {
  if (!server || !out) return FV_ERR_NULL;
  server->impl->stats(out);
  return 0;
}

int fv_serve_reset_stats(FvServe* server) {
  if (!server) return FV_ERR_NULL;
  server->impl->reset_stats();
  return 0;
}

}  // extern "C"
