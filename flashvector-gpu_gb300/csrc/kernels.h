// kernels.h -- internal (C++) interface between the C-ABI bridge and the
// kernel translation units. Nothing here crosses the library boundary.
#pragma once

#include <cuda.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include <algorithm>

#include "../../include/fv_types.h"

namespace fv {

inline uint32_t next_pow2(uint32_t v) {
  if (v <= 1) return 1;
  --v;
  v |= v >> 1;
  v |= v >> 2;
  v |= v >> 4;
  v |= v >> 8;
  v |= v >> 16;
  return v + 1;
}

// Per-query filter of a heterogeneous batch: packed LSB-first words over
// logical ids, one row per query (rows may be shared). Ids at or beyond
// nwords * 32 are filtered out, the rule the reference applies to words past
// the end of a user mask (index.rs:1264-1292). words == nullptr: no filter.
// Kernels take a device array of these (nullptr: no per-query filters); it
// is applied on top of the shared slot-validity mask.
struct QueryFilter {
  const uint32_t* words;
  uint32_t nwords;
  uint32_t reserved;
};

// Process-wide tuning knobs (fv_tune_set / fv_tune_get).
bool tune_set(const char* key, int64_t value);
bool tune_get(const char* key, int64_t* value);
int64_t tune_value(const char* key, int64_t dflt);

// Streaming-multiprocessor count of the current device (cached per device).
int device_sm_count();

// Device address of the status word of the current device (see
// fv_read_device_status); allocated on first use.
uint32_t* status_word();

// Host-side launch counter (fv_launch_count).
void note_launch(uint32_t n = 1);

// Optional per-kernel timing (fv_profile_enable): when on, ProfScope
// records a CUDA event pair around the launches in its scope on `stream`.
bool profiling_enabled();
void profile_record(const char* name, cudaEvent_t start, cudaEvent_t stop);
cudaEvent_t profile_event();
struct ProfScope {
  const char* name;
  cudaStream_t stream;
  cudaEvent_t start = nullptr;
  ProfScope(const char* n, cudaStream_t s) : name(n), stream(s) {
    if (profiling_enabled()) {
      start = profile_event();
      cudaEventRecord(start, stream);
    }
  }
  ~ProfScope() {
    if (start) {
      cudaEvent_t stop = profile_event();
      cudaEventRecord(stop, stream);
      profile_record(name, start, stop);
    }
  }
};

// Per-stream scratch arena: returns a device buffer of at least `bytes`
// bytes that stays valid for work enqueued on `stream` until the next call
// for the same stream with a larger size. Grows with stream-ordered
// allocation; returns nullptr on failure. A caller-provided arena installed
// with fv_set_stream_scratch() takes precedence.
void* scratch_get(cudaStream_t stream, size_t bytes);

// Writes `count` {0xFFFFFFFF, 1e30} results (fixtures.cu).
int launch_fill_sentinel(GpuSearchResult* out, size_t count, cudaStream_t stream);

// exact fp32 flat scan (flat_fp32.cu)
struct FlatPlan {
  uint32_t splits = 1, tiles_per_split = 0;
  size_t scratch_bytes = 0;  // per-split heaps (0 when one split)
};
FlatPlan plan_flat_f32(uint32_t n, uint32_t nq, uint32_t k, uint32_t forced_splits);
// fused = true accumulates fmaf(diff, diff, acc) (L2 only): the coarse quantizer
int launch_flat_f32_planned(const FlatPlan& p, const float* vectors, const uint32_t* vec_ids, uint32_t n,
                            uint32_t dim, const float* queries, uint32_t nq, uint32_t k, MetricType metric,
                            const uint32_t* mask, GpuSearchResult* out, bool fused, void* scratch,
                            cudaStream_t stream, const QueryFilter* filters = nullptr);
int launch_flat_f32(const float* vectors, const uint32_t* vec_ids, uint32_t n, uint32_t dim, const float* queries,
                    uint32_t nq, uint32_t k, MetricType metric, const uint32_t* mask, GpuSearchResult* out,
                    uint32_t forced_splits, cudaStream_t stream, const QueryFilter* filters = nullptr);

// tensor-core flat scans (tc_scan.cu)
struct TcTables {
  bool fp8;              // false: fp16 rows, true: e4m3 rows
  const void* base;      // [n][padded_dim] fp16 or e4m3
  const float* norms;    // [n] ||x||^2 (may be null for inner product)
  const float* scales;   // [n] per-row dequantisation scale (fp8 only)
  const float* vectors;  // [n][dim] fp32 rows for the rescore (optional)
  uint32_t n, dim, padded_dim;
  bool fp8_table_scale = true;  // fp8: one power-of-two table scale + norm digits; false: per-row scales
};
struct TcScanArgs;
cudaError_t dispatch_tc_scan_fp16(int kl, int groups, int metric, bool table_scale, const CUtensorMap& ta,
                                  const CUtensorMap& tb, const TcScanArgs& a, uint32_t grid, cudaStream_t stream);
cudaError_t dispatch_tc_scan_fp8(int kl, int groups, int metric, bool table_scale, const CUtensorMap& ta,
                                 const CUtensorMap& tb, const TcScanArgs& a, uint32_t grid, cudaStream_t stream);
int launch_tc_scan(const TcTables& t, const float* queries, uint32_t nq, uint32_t k, MetricType metric,
                   const uint32_t* mask, GpuSearchResult* out, const FvScanOptions& opt, cudaStream_t stream,
                   const QueryFilter* filters = nullptr);
// launch_tc_scan with the scratch given by the caller (ext_scratch: at
// least tc_scan_scratch_bytes, 1 KB aligned; null: the stream's arena) and
// an optional per-query flag array set for a query whose merged shortlist
// may have lost keys to a full range heap (the caller zeroes it).
int launch_tc_scan_ext(const TcTables& t, const float* queries, uint32_t nq, uint32_t k, MetricType metric,
                       const uint32_t* mask, GpuSearchResult* out, const FvScanOptions& opt, cudaStream_t stream,
                       const QueryFilter* filters, void* ext_scratch, uint32_t* incomplete_q);
// The scratch bytes launch_tc_scan takes from the stream's arena for the
// same arguments (same plan, same tuning knobs).
size_t tc_scan_scratch_bytes(const TcTables& t, uint32_t nq, uint32_t k, MetricType metric, const FvScanOptions& opt);

// IVF-PQ / IVF-SQ8 search (ivf.cu)
struct IvfLaunch {
  const float* centroids;
  const float* codebooks;   // PQ
  const float* sq_mins;     // SQ8
  const float* sq_scales;   // SQ8
  const uint8_t* codes;
  const uint32_t* offsets;
  const uint32_t* vec_ids;
  const float* vectors;
  uint32_t num_vectors, dim, nlist, m_pq, sub_dim;
  bool list_major;
  const float* queries;
  uint32_t nq, top_k, nprobe, rerank_k;
  MetricType metric;
  const uint32_t* mask;
  GpuSearchResult* out;
  // heterogeneous batches (all optional): per-query top_k / nprobe / rerank_k
  // (top_k, nprobe and rerank_k above are then their maxima; results are
  // written with a stride of top_k), per-query filters over logical ids
  const uint32_t* q_topk;
  const uint32_t* q_nprobe;
  const uint32_t* q_rerank;
  const QueryFilter* filters;
  // RaBitQ: rotated centroids [nlist][P], sign bits [N][P/32] and meta
  // [N][4] (by id, or by list position when list_major), rotation signs [3P]
  const float* rot_centroids;
  const uint32_t* rq_bits;
  const float* rq_meta;
  const float* rot_signs;
  uint32_t padded_dim;
};
enum { IVF_MODE_PQ = 0, IVF_MODE_SQ8 = 1, IVF_MODE_RABITQ = 2 };
int launch_ivf_search(int mode, const IvfLaunch& L, cudaStream_t stream);
// The scratch bytes launch_ivf_search takes from the stream's arena for the
// same arguments (0 when the call launches nothing or is refused).
size_t ivf_search_scratch_bytes(int mode, const IvfLaunch& L);
// The committed IVF autotuner entry for a shape: out3 = {pipeline, split,
// tc_coarse} (-1: automatic); FV_ERR_ARG when none applies.
int ivf_tune_query(int mode, uint32_t dim, uint64_t n, uint32_t nlist, uint32_t nq, uint32_t nprobe, int32_t* out3);
int launch_relayout_codes(const uint8_t* by_id, const uint32_t* vec_ids, uint32_t n, uint32_t row_bytes,
                          uint8_t* by_list, cudaStream_t stream);

// main + live-insert merge of a served batch (batch.cu): per query the
// stable merge of the two answer rows (stride `stride`), truncated to the
// query's k (q_topk[q], or top_k), padded with {u32::MAX, +inf}
int launch_merge_main_delta(const GpuSearchResult* main_res, const GpuSearchResult* delta_res, uint32_t nq,
                            uint32_t stride, const uint32_t* q_topk, uint32_t top_k, GpuSearchResult* out,
                            cudaStream_t stream);

// IVF index build (index_build.cu)
int launch_kmeans_update(const float* x, uint32_t n, uint32_t dim, const GpuSearchResult* assign, uint32_t k,
                         float* centroids, uint32_t* counts, double* sums, cudaStream_t stream);
int launch_build_lists(const GpuSearchResult* assign, uint32_t n, uint32_t nlist, uint32_t* offsets, uint32_t* vec_ids,
                       uint32_t* work, cudaStream_t stream);
int launch_residuals(const float* x, uint32_t n, uint32_t dim, const float* centroids, const GpuSearchResult* assign,
                     float* out, cudaStream_t stream);
int launch_extract_subspace(const float* x, uint32_t n, uint32_t dim, uint32_t off, uint32_t sub, float* out,
                            cudaStream_t stream);
int launch_pq_encode(const float* x, uint32_t n, uint32_t dim, uint32_t m_pq, const float* codebooks, uint8_t* codes,
                     cudaStream_t stream);
int launch_sq8_fit(const float* r, uint32_t n, uint32_t dim, float* mins, float* scales, uint32_t* work,
                   cudaStream_t stream);
int launch_sq8_encode(const float* r, uint32_t n, uint32_t dim, const float* mins, const float* scales, uint8_t* codes,
                      cudaStream_t stream);
int launch_gather_rows(const float* x, const uint32_t* rows, uint32_t count, uint32_t dim, float* out,
                       cudaStream_t stream);
// RaBitQ encoder: rotated centroids, sign bits and meta of every row's
// rotated residual to its assigned centroid (inv_sqrt_p = 1 / sqrt(P))
uint32_t rabitq_padded_dim(uint32_t dim);
float rabitq_inv_sqrt(uint32_t padded_dim);
void rabitq_rot_signs(uint32_t padded_dim, uint64_t seed, float* out);
int launch_rabitq_encode(const float* x, uint32_t n, uint32_t dim, const float* centroids, uint32_t nlist,
                         const GpuSearchResult* assign, const float* signs, uint32_t padded_dim, float* rot_centroids,
                         uint32_t* bits, float* meta, cudaStream_t stream);
int launch_fill_f32(float* p, size_t n, float v, cudaStream_t stream);
// out row i = in row rows[i] (rows of row_bytes bytes), zeros where rows[i] == zero_row
int launch_gather_row_bytes(const void* in, const uint32_t* rows, uint32_t count, uint32_t row_bytes,
                            uint32_t zero_row, void* out, cudaStream_t stream);

// reduced-precision table encoders (encode.cu)
int launch_encode_fp16(const float* x, uint32_t n, uint32_t dim, uint32_t pd, uint16_t* out, float* norms,
                       cudaStream_t stream);
int launch_encode_fp8(const float* x, uint32_t n, uint32_t dim, uint32_t pd, uint8_t* out, float* scales,
                      float* norms, cudaStream_t stream);
int launch_encode_fp8_per_vector(const float* x, uint32_t n, uint32_t dim, uint32_t pd, uint8_t* out, float* scales,
                                 float* norms, cudaStream_t stream);

// test fixtures (fixtures.cu)
int launch_distance_matrix(const float* queries, const float* base, uint32_t nq, uint32_t n, uint32_t dim,
                           MetricType metric, float* out, cudaStream_t stream);
int launch_bitonic_test(const float* keys_in, const uint32_t* vals_in, float* keys_out, uint32_t* vals_out,
                        uint32_t n, cudaStream_t stream);

}  // namespace fv
