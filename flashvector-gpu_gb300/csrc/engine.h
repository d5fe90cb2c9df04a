// engine.h -- internal interface of the native engine (engine.cpp) used by
// the serving loop (serve.cpp). Nothing here crosses the library boundary.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/fv_bridge.h"
#include "kernels.h"

namespace fv {

class Index;

// One served batch, launched asynchronously on the caller's stream.
//   engine             FV_ENGINE_*
//   top_k              results per query (row stride of every result array);
//                      for IVF with d_topk: the largest k of the batch
//   nprobe, rerank_k   IVF: uniform values, or the batch maxima with
//                      d_nprobe / d_rerank
//   d_queries          [nq][dim] fp32, already prepared (cosine rows
//                      normalised, as prepare_queries does: index.rs:1473-1483)
//   d_topk, d_nprobe, d_rerank   per-query IVF parameters (device) or null;
//                      the flat and tensor-core engines take a uniform k
//   d_filters          per-query filters over logical ids (device) or null
//   d_out              [nq][top_k] answers
//   d_main, d_delta    [nq][top_k] scratch used when the live-insert buffer
//                      is non-empty (main answers, delta answers)
struct BatchLaunch {
  uint32_t engine = 0, nq = 0, top_k = 0, nprobe = 0, rerank_k = 0;
  const float* d_queries = nullptr;
  const uint32_t* d_topk = nullptr;
  const uint32_t* d_nprobe = nullptr;
  const uint32_t* d_rerank = nullptr;
  const QueryFilter* d_filters = nullptr;
  GpuSearchResult* d_out = nullptr;
  GpuSearchResult* d_main = nullptr;
  GpuSearchResult* d_delta = nullptr;
  FvScanOptions scan{0, 1, 0.f, 0};
};

Index* index_of(FvIndex* handle);
uint32_t index_dim(const Index* index);
int index_metric(const Index* index);
bool index_built(const Index* index);
// Normalises query rows in place when the index metric is cosine (the
// engine's prepare_queries, index.rs:1473-1483); otherwise a no-op.
void index_prepare_queries(const Index* index, float* rows, uint32_t n);
uint32_t index_nlist(const Index* index);
// Pins the index state (tables, live-insert buffer, validity words) for
// work in flight: build / add / delete wait until every pin is released.
// A pin may be released from any thread.
void index_pin(Index* index);
void index_unpin(Index* index);
// Enqueues one batch on `stream` (the caller holds a pin until the stream
// has passed the batch). Returns 0 or an error code; nothing is launched
// on an argument error.
int index_launch_batch(Index* index, const BatchLaunch& b, cudaStream_t stream);
// The stream scratch (bytes) index_launch_batch takes for `b` (its device
// pointers are not read; the per-query parameter arrays only count as
// present or absent). The state may change with build / add / delete: a
// caller that relies on the figure holds a pin from estimate to launch.
size_t index_batch_scratch_bytes(const Index* index, const BatchLaunch& b);

}  // namespace fv
