/*
 * fv_bridge.h -- C ABI of libfvgb300 (sm_103a).
 *
 * The `cuda_*` entry points are drop-ins for the functions of the same
 * name in the reference's kernels/include/cuda_bridge.h: same name, same
 * argument order and meaning, same return convention, so the extern block
 * of crates/engine/src/ffi.rs:234-455 binds them unchanged.
 *
 * Return convention (reference: sparse_hybrid.cu:517-524,
 * ivf_pq_lookup.cu:462-472): 0 on success; -1 when a required pointer is
 * null; otherwise the cudaError_t of the failing CUDA call. Empty work
 * (zero queries or top_k == 0) is a successful no-op. All launches are
 * asynchronous on `stream` (a cudaStream_t passed as void*, NULL = legacy
 * default stream); the caller synchronises.
 *
 * `fv_*` entry points are extensions with no reference counterpart.
 */
#ifndef FV_BRIDGE_H
#define FV_BRIDGE_H

#include "fv_types.h"

#ifdef __cplusplus
extern "C" {
#endif

/* Additional return codes of the fv extensions (and of the drop-ins where
 * the reference would have silently failed). */
#define FV_OK 0
#define FV_ERR_NULL (-1)
#define FV_ERR_ARG (-2)        /* argument outside the supported range        */
#define FV_ERR_TIMEOUT (-3)    /* a bounded device wait gave up               */
#define FV_ERR_NOMEM (-4)      /* scratch admission refused                   */
#define FV_ERR_ARCH (-5)       /* device is not sm_103 / sm_100 class         */
#define FV_ERR_SCRATCH_LIMIT (-6) /* work exceeds a fixed scratch area's size  */
#define FV_ERR_QUEUE_FULL (-7)    /* serving loop: admission queue at capacity */

/* ---- device, memory and stream plumbing -------------------------------
 * Replace cuda_bridge.h:11-31 (hnsw_traverse.cu:525-637). */
int cuda_init_device(int device_id);
int cuda_set_device(int device_id);
int cuda_get_device_count(int* count);
int cuda_get_device_memory(size_t* free_bytes, size_t* total_bytes);
int cuda_device_synchronize(void);
int cuda_malloc_device(void** ptr, size_t bytes);
int cuda_free_device(void* ptr);
int cuda_malloc_host(void** ptr, size_t bytes);
int cuda_free_host(void* ptr);
int cuda_memcpy_h2d_async(void* dst, const void* src, size_t bytes, void* stream);
int cuda_memcpy_d2h_async(void* dst, const void* src, size_t bytes, void* stream);
int cuda_memset_device_async(void* dst, int value, size_t bytes, void* stream);
int cuda_host_get_device_pointer(void** dev_ptr, void* host_ptr);
int cuda_create_stream(void** stream);
int cuda_destroy_stream(void* stream);
int cuda_sync_stream(void* stream);

/* ---- exact flat scan ---------------------------------------------------
 * Replaces cuda_bridge.h:150-162 (sparse_hybrid.cu:504-525).
 * Per query: the top_k (clamped to 256) rows of d_vectors by distance,
 * ascending; ties go to the lower slot index. d_vec_ids (optional) maps
 * slot -> reported id; d_valid_mask (optional) is a packed LSB-first bit
 * per slot. num_vectors == 0 fills d_out_results with 0xFF bytes. */
int cuda_flat_scan_batch(const float* d_vectors, const uint32_t* d_vec_ids,
                         uint32_t num_vectors, uint32_t dim,
                         const float* d_queries, uint32_t num_queries,
                         uint32_t top_k, MetricType metric,
                         const uint32_t* d_valid_mask,
                         GpuSearchResult* d_out_results, void* stream);

/* Allocation-free exact flat scan. No counterpart in the reference: it is
 * cuda_flat_scan_batch for callers that may not allocate device memory --
 * threads running while a CUDA graph is captured in global mode (where
 * cudaMalloc is an illegal call), latency-critical serving threads that
 * must not take the allocator's locks or its implicit synchronisation, and
 * hosts that give all device memory to a pool of their own. Same arguments,
 * results (bit-identical) and return codes as cuda_flat_scan_batch; the
 * per-split heaps that cuda_flat_scan_batch keeps in a per-stream arena
 * live instead in one fixed 8 MiB device array that the library holds on
 * every GPU that loads it, until exit. The caller still passes inputs and
 * outputs. A call whose heaps (num_queries x splits x top_k x 8 bytes)
 * would exceed the array is refused with FV_ERR_SCRATCH_LIMIT and
 * launches nothing. The first call on a device looks up the array's device
 * address (cudaGetSymbolAddress) and caches it for the life of the process:
 * make that first call before any stream capture, and do not call this
 * entry point again on a device after cudaDeviceReset (the new context may
 * place the array elsewhere). All calls share the array, which keeps the
 * last call's contents; calls whose GPU work overlaps (other streams, other
 * host threads on the same device) race on it and must be serialised. */
int fv_flat_scan_batch_noalloc(const float* d_vectors, const uint32_t* d_vec_ids,
                               uint32_t num_vectors, uint32_t dim,
                               const float* d_queries, uint32_t num_queries,
                               uint32_t top_k, MetricType metric,
                               const uint32_t* d_valid_mask,
                               GpuSearchResult* d_out_results, void* stream);

/* ---- IVF-PQ / IVF-SQ8 inverted-list scans -------------------------------
 * Replace cuda_bridge.h:96-121 (ivf_pq_lookup.cu:450-473,
 * ivf_quant_lookup.cu:1064-1083). Clamps as launch_ivf_pq_search
 * (ivf_pq_lookup.cu:351-362): top_k <= 256, nprobe in [1, nlist],
 * shortlist = rerank_k ? rerank_k : top_k (>= top_k, <= 10240), exact fp32
 * rerank when rerank_k != 1 and tables->d_vectors is non-null. Coarse
 * probe exact by (L2, list id); nprobe above 256 returns FV_ERR_ARG.
 * Results are vector ids sorted by (distance, id). */
int cuda_ivf_pq_search_batch(const IvfPqGpuTables* tables, const float* d_queries,
                             uint32_t num_queries, uint32_t top_k, uint32_t nprobe,
                             uint32_t rerank_k, MetricType metric,
                             const uint32_t* d_valid_mask, GpuSearchResult* d_out_results,
                             void* stream);
int cuda_ivf_sq_search_batch(const IvfSqGpuTables* tables, const float* d_queries,
                             uint32_t num_queries, uint32_t top_k, uint32_t nprobe,
                             uint32_t rerank_k, MetricType metric,
                             const uint32_t* d_valid_mask, GpuSearchResult* d_out_results,
                             void* stream);
/* Same searches with options (FvIvfOptions, may be NULL): list-major codes
 * stream each posting list as contiguous 16-byte loads. */
int fv_ivf_pq_search_ex(const IvfPqGpuTables* tables, const FvIvfOptions* options,
                        const float* d_queries, uint32_t num_queries, uint32_t top_k,
                        uint32_t nprobe, uint32_t rerank_k, MetricType metric,
                        const uint32_t* d_valid_mask, GpuSearchResult* d_out_results,
                        void* stream);
int fv_ivf_sq_search_ex(const IvfSqGpuTables* tables, const FvIvfOptions* options,
                        const float* d_queries, uint32_t num_queries, uint32_t top_k,
                        uint32_t nprobe, uint32_t rerank_k, MetricType metric,
                        const uint32_t* d_valid_mask, GpuSearchResult* d_out_results,
                        void* stream);
/* IVF-RaBitQ (replaces cuda_bridge.h:123-134, ivf_quant_lookup.cu:333-870,
 * 1085-1104). Clamps and coarse probe as the IVF-PQ scan. The query is
 * rotated (three rounds of d_rot_signs flips, Walsh-Hadamard butterflies
 * and a 1 / sqrt(padded_dim) scale, the scale being the correctly rounded
 * 1.0f / sqrtf(padded_dim) of the reference's host encoder); per probed list
 * its rotated residual is quantised to 4 bits over [min, max] and every
 * posting gets the popcount estimate of its squared L2 distance (for inner
 * product -0.5 (|q|^2 + |x|^2 - est), for cosine 0.5 est); the shortlist of
 * the best rerank_k estimates is re-ranked exactly. tables->words_per_vec
 * must be padded_dim / 32 and padded_dim a power of two >= max(dim, 32),
 * <= 4096, else FV_ERR_ARG. */
int cuda_ivf_rabitq_search_batch(const IvfRabitqGpuTables* tables, const float* d_queries,
                                 uint32_t num_queries, uint32_t top_k, uint32_t nprobe,
                                 uint32_t rerank_k, MetricType metric,
                                 const uint32_t* d_valid_mask, GpuSearchResult* d_out_results,
                                 void* stream);
int fv_ivf_rabitq_search_ex(const IvfRabitqGpuTables* tables, const FvIvfOptions* options,
                            const float* d_queries, uint32_t num_queries, uint32_t top_k,
                            uint32_t nprobe, uint32_t rerank_k, MetricType metric,
                            const uint32_t* d_valid_mask, GpuSearchResult* d_out_results,
                            void* stream);
/* Gathers id-indexed code rows into list order:
 * d_out[i] = d_codes_by_id[d_ivf_vec_ids[i]] (row_bytes each). */
int fv_ivf_relayout_codes(const uint8_t* d_codes_by_id, const uint32_t* d_ivf_vec_ids,
                          uint32_t num_vectors, uint32_t row_bytes, uint8_t* d_out_by_list,
                          void* stream);

/* ---- IVF index build (GPU) ---------------------------------------------
 * Restate the reference's host encoders on the device: PQ nearest-codeword
 * encode of residual rows (cluster.rs:247-287; codebooks [m_pq][256][dim/m_pq]),
 * SQ8 fit + encode of residual rows (quant.rs:14-75), posting lists from a
 * nearest-centroid assignment (index.rs:445-458; ids within a list in no
 * particular order). d_assign is the k = 1 result of a flat scan of the rows
 * against the centroids. */
int fv_build_pq_encode(const float* d_residuals, uint32_t num_vectors, uint32_t dim, uint32_t m_pq,
                       const float* d_codebooks, uint8_t* d_out_codes, void* stream);
int fv_build_sq8(const float* d_residuals, uint32_t num_vectors, uint32_t dim, float* d_out_mins,
                 float* d_out_scales, uint8_t* d_out_codes, void* stream);
int fv_build_ivf_lists(const GpuSearchResult* d_assign, uint32_t num_vectors, uint32_t nlist,
                       uint32_t* d_out_offsets, uint32_t* d_out_vec_ids, void* stream);
/* RaBitQ encoder (RabitqEncoder::encode, quant.rs:156-234) on the device:
 * rot_signs from the reference's seeded generator (host, 3 * padded_dim
 * floats: fv_rabitq_rot_signs), rotated centroids, and per row the sign
 * bits and meta of its rotated residual to centroid d_assign[v].id, with
 * the reference's summation orders (bit-identical to the host encoder).
 * fv_rabitq_padded_dim gives max(dim, 32) rounded up to a power of two. */
uint32_t fv_rabitq_padded_dim(uint32_t dim);
void fv_rabitq_rot_signs(uint32_t padded_dim, uint64_t seed, float* host_out);
int fv_build_rabitq(const float* d_vectors, uint32_t num_vectors, uint32_t dim, const float* d_centroids,
                    uint32_t nlist, const GpuSearchResult* d_assign, const float* d_rot_signs,
                    uint32_t padded_dim, float* d_out_rot_centroids, uint32_t* d_out_bits,
                    float* d_out_meta, void* stream);

/* ---- tensor-core flat scans --------------------------------------------
 * Replaces cuda_bridge.h:138-147 (ivf_quant_lookup.cu:1106-1123). Per
 * query the top_k (<= 256) rows by the fp16 tensor-core distance
 * (IP: -dot, L2: max(0, |q|^2 + |x|^2 - 2 dot), cosine: 1 - dot /
 * (sqrt(|q|^2 |x|^2) + 1e-8)), ties to the lower slot. When
 * tables->d_vectors is non-null (the reference documents it as the fp32
 * copy for exact rerank, types.h:134) a shortlist of 4 * top_k is rescored
 * in fp32 and the band around the k-th distance re-ranked in fp64; the
 * reported distances are then the fp32 (fp64 in the band) values. Ids are
 * slot indices; d_valid_mask filters slots. */
int cuda_fp16_tc_search_batch(const Fp16GpuTables* tables, const float* d_queries,
                              uint32_t num_queries, uint32_t top_k, MetricType metric,
                              const uint32_t* d_valid_mask, GpuSearchResult* d_out_results,
                              void* stream);

/* Same as cuda_fp16_tc_search_batch with explicit options (over-fetch,
 * fp64 boundary band, base-range splits); options may be NULL. */
int fv_fp16_search_batch_ex(const Fp16GpuTables* tables, const float* d_queries,
                            uint32_t num_queries, uint32_t top_k, MetricType metric,
                            const uint32_t* d_valid_mask, const FvScanOptions* options,
                            GpuSearchResult* d_out_results, void* stream);

/* FP8 (E4M3) tensor-core flat scan over a table written by fv_encode_fp8
 * (scale_mode 0, padded_dim >= dim + 3) or fv_encode_fp8_per_vector
 * (scale_mode 1); same contract as the fp16 scan. Queries get a power-of-two
 * scale over a mode-0 table (the smallest 2^a with max|q| <= 448 * 2^a, at
 * least 2^(b-8) for the table scale 2^b), max|q| / 448 over a mode-1 table.
 * No reference counterpart (the reference has no fp8 path). */
int fv_fp8_search_batch(const FvFp8GpuTables* tables, const float* d_queries,
                        uint32_t num_queries, uint32_t top_k, MetricType metric,
                        const uint32_t* d_valid_mask, const FvScanOptions* options,
                        GpuSearchResult* d_out_results, void* stream);

/* Device-side table encoders. fv_encode_fp16_padded restates the
 * reference's host encoder encode_fp16_padded (quant.rs:306-327, rounding
 * of quant.rs:239-274); padded_dim a multiple of 16, >= dim.
 * fv_encode_fp8 has no counterpart: the layout of FvFp8GpuTables
 * (padded_dim a multiple of 16, >= dim + 3; all three outputs required). */
int fv_encode_fp16_padded(const float* d_vectors, uint32_t num_vectors, uint32_t dim,
                          uint32_t padded_dim, uint16_t* d_out_fp16, float* d_out_norms_sq,
                          void* stream);
int fv_encode_fp8(const float* d_vectors, uint32_t num_vectors, uint32_t dim,
                  uint32_t padded_dim, uint8_t* d_out_fp8, float* d_out_scales,
                  float* d_out_norms_sq, void* stream);
/* The per-vector-scale fp8 layout (FvFp8GpuTables scale_mode 1):
 * padded_dim a multiple of 16, >= dim; all three outputs required. */
int fv_encode_fp8_per_vector(const float* d_vectors, uint32_t num_vectors, uint32_t dim,
                             uint32_t padded_dim, uint8_t* d_out_fp8, float* d_out_scales,
                             float* d_out_norms_sq, void* stream);

/* ---- host engine -------------------------------------------------------
 * The reference's GpuVectorIndex (crates/engine/src/index.rs:131-2634) for
 * the scan engines, behind an opaque handle. Host buffers in and out; every
 * call is synchronous like the reference's methods.
 *   fv_index_build    index.rs:328-576 (tables built on the GPU)
 *   fv_index_add      add_vectors, index.rs:647-694 (ids written to out_ids)
 *   fv_index_delete   delete_ids, index.rs:583-643
 *   fv_index_search   batch_search_fp16_tc / batch_search_ivf_mode / the
 *                     exact flat scan (index.rs:1979-2237): params->engine
 *                     selects FV_ENGINE_*; host_mask_words is the optional
 *                     user filter over logical ids (mask_words words);
 *                     host_out receives num_queries * top_k results.
 *   fv_index_search_device  batch_search_ivf_device_ptr (index.rs:2110)
 *   fv_index_stats    MetricsTracker::get_stats (metrics.rs:47-90) */
typedef struct FvIndex FvIndex;
int fv_index_create(const FvIndexConfig* config, FvIndex** out);
int fv_index_destroy(FvIndex* index);
int fv_index_build(FvIndex* index, const float* host_vectors, uint32_t num_vectors);
/* Build from rows already in device memory; d_init_centroids (nlist rows,
 * may be NULL) seeds the coarse k-means, which then runs
 * config.kmeans_iters_given Lloyd iterations (0 = keep them as given). */
int fv_index_build_device(FvIndex* index, const float* d_vectors, uint32_t num_vectors,
                          const float* d_init_centroids);
int fv_index_add(FvIndex* index, const float* host_vectors, uint32_t num_vectors, uint32_t* out_ids);
int fv_index_delete(FvIndex* index, const uint32_t* ids, uint32_t count, uint32_t* out_deleted);
int fv_index_search(FvIndex* index, const FvSearchParams* params, const float* host_queries,
                    uint32_t num_queries, const uint32_t* host_mask_words, uint32_t mask_words,
                    GpuSearchResult* host_out);
int fv_index_search_device(FvIndex* index, const FvSearchParams* params, const float* d_queries,
                           uint32_t num_queries, GpuSearchResult* host_out);
int fv_index_stats(FvIndex* index, FvLatencyStats* out);
int fv_index_info(FvIndex* index, FvIndexInfo* out);
/* Device views of the engine's IVF tables (list-major code rows) and the
 * matching options, for calling fv_ivf_{pq,sq}_search_ex directly (for
 * example inside a captured CUDA graph). Valid until the next build. */
int fv_index_ivf_tables(FvIndex* index, IvfPqGpuTables* pq, IvfSqGpuTables* sq, FvIvfOptions* options);
/* The same for the RaBitQ tables (list-major bits and meta, for
 * fv_ivf_rabitq_search_ex); FV_ERR_ARG when the index has none. */
int fv_index_rabitq_tables(FvIndex* index, IvfRabitqGpuTables* rabitq, FvIvfOptions* options);
/* Copies IVF table `table` to host memory: 0 centroids, 1 codebooks, 2 PQ
 * codes by id, 3 SQ8 mins, 4 SQ8 scales, 5 SQ8 codes by id, 6 list offsets,
 * 7 list ids, 8 RaBitQ rotation signs, 9 rotated centroids, 10 RaBitQ bits
 * by id, 11 RaBitQ meta by id. */
int fv_index_export_ivf(FvIndex* index, uint32_t table, void* host_out, size_t bytes);

/* Snapshots in the reference's FLSHVEC1 format (persistence.rs:1-200,
 * GpuVectorIndex::save_snapshot / load_snapshot, index.rs:845-1260).
 * save: every section the reference's loader requires (the graph
 * sections, whose engines lie outside the scan path, are written empty).
 * load: the file's dim / metric / nlist / m_pq; `config` (optional)
 * supplies build_flags (FV_BUILD_FP8 adds an fp8 table built on the GPU;
 * fp16 rows are taken from the file when padded as this engine pads, else
 * encoded; RaBitQ tables are taken from the file when present, else
 * encoded on the GPU), streams and seed. Sections are copied to the GPU from a
 * read-only mapping of the file; rows whose logical id differs from their
 * slot are placed at their logical id. fv_snapshot_inspect (no GPU
 * needed) writes the manifest as JSON; fv_snapshot_error describes the last
 * failure of these calls on this thread. */
int fv_index_save_snapshot(FvIndex* index, const char* path);
int fv_index_load_snapshot(const char* path, const FvIndexConfig* config, FvIndex** out);
int fv_snapshot_inspect(const char* path, char* manifest_json, size_t len, size_t* needed);
const char* fv_snapshot_error(void);

/* ---- CUDA graphs -------------------------------------------------------
 * Capture the library calls issued on `stream` between fv_graph_begin and
 * fv_graph_end into one replayable graph (the steady-state search of a fixed
 * batch shape). Captured calls keep their device pointers: refill the same
 * query / mask buffers before each fv_graph_launch. Make the same calls once
 * before capturing so that per-stream scratch is already large enough (no
 * allocation happens inside a capture). Not for the legacy NULL stream. */
typedef struct FvGraph FvGraph;
int fv_graph_begin(void* stream);
int fv_graph_end(void* stream, FvGraph** out);
int fv_graph_launch(FvGraph* graph, void* stream);
uint64_t fv_graph_kernel_count(const FvGraph* graph);
int fv_graph_destroy(FvGraph* graph);

/* ---- test fixtures -----------------------------------------------------
 * Replace cuda_bridge.h:195-213 (hnsw_traverse.cu:387-437, 694-735). */
int cuda_compute_distances_warp(const float* d_queries, const float* d_dataset,
                                uint32_t num_queries, uint32_t num_vectors,
                                uint32_t dim, MetricType metric,
                                float* d_out_distances, void* stream);
int cuda_bitonic_sort_test(const float* d_keys_in, const uint32_t* d_vals_in,
                           float* d_keys_out, uint32_t* d_vals_out, uint32_t n,
                           void* stream);

/* ---- extensions --------------------------------------------------------*/
/* Library version string, e.g. "fvgb300 0.1 sm_103a". */
const char* fv_version(void);
/* Reads and clears the device status word that bounded waits and bounds
 * checks of the kernels set (0 = clean). Synchronises the device. */
int fv_read_device_status(uint32_t* status);
/* Number of this library's kernel launches issued since load (all
 * devices, all streams); used to count launches inside timed regions. */
uint64_t fv_launch_count(void);
/* Per-kernel timing: while enabled, each kernel launch of the library is
 * bracketed by a CUDA event pair on its stream. fv_profile_summary waits
 * for the recorded events, writes {"kernel": {"launches": n, "ms": t}, ...}
 * (JSON, NUL-terminated) into buf and clears the record. */
int fv_profile_enable(int on);
int fv_profile_summary(char* buf, size_t len);
/* Process-wide tuning knobs (no reference counterpart). Keys:
 *   "tc.prepass"        -1 automatic (default), 0 off, 1 on where it applies:
 *                       tensor-core scans whose shortlist exceeds the 64-entry
 *                       per-range heap first scan a strided sample of the
 *                       base for a per-query admission bound
 *   "tc.prepass_stride" sample stride in 256-row tiles (0 automatic: the
 *                       tuned value, else 32)
 *   "tc.prepass_margin" 0 (default): the sampled rank r is the smallest
 *                       with P(Poisson(shortlist / stride) >= r) < 1e-7;
 *                       m > 0: r = ceil(m * shortlist / stride)
 *   "tc.pair"           -1 automatic (default), 0 off, 1 on: tensor-core scans
 *                       of long rows (more than two K blocks) run on CTA
 *                       pairs (cta_group::2), each SM streaming half of
 *                       every base tile
 *   "tc.groups"         -1 (default): fp8 scans of a table-scale table (L2,
 *                       inner product) with one K block per tile and a
 *                       shortlist above 48 keys drain each tile with four
 *                       epilogue groups (16 warps, heaps of <= 32 keys),
 *                       other short-row scans with two (heaps of <= 48);
 *                       2 or 4: that many wherever the four-group form
 *                       applies. Same answers
 *   "tc.wait_limit_ns"  0 (default): the tensor-core scan's pipeline waits give
 *                       up after 2 s; n > 0: after n ns. A wait that runs
 *                       out ends the scan early (its answer is not valid)
 *                       and sets the timeout bit that fv_read_device_status
 *                       reports; the context stays usable (a short limit
 *                       exercises that path)
 *   "tc.table"          1 (default): knobs left automatic and a zero
 *                       over-fetch take the committed autotuner results
 *                       for the call's shape (tuning/gb300.json); 0: ignore
 *   "ivf.pipeline"      -1 (default): the committed autotuner's choice for
 *                       the call's shape, else 0; 0: the IVF-PQ list scan
 *                       loads and scores 4 postings per thread per round;
 *                       1: 2 per round with the next round's loads in flight
 *   "ivf.split"         -1 (default): batches of fewer than 4 queries per
 *                       SM cut each query's probed postings into G equal
 *                       ranges scanned by separate CTAs and merged (same
 *                       answer); 0 or 1: never; G > 1: always G ranges
 *   "ivf.compact"       1 (default): with a validity mask, each call compacts
 *                       the mask-admitted list positions once, and a probed
 *                       list whose mask admits under half of it is walked
 *                       over those positions only (same answer); 0: every
 *                       posting is walked and tested against the mask bits
 *   "ivf.tc_coarse"     -1 (default): the committed autotuner's choice for
 *                       the call's shape, else: calls with nlist >= 2048 and >= 256
 *                       queries find the probed lists with an fp16 tensor-
 *                       core scan of the centred queries and centroids, the
 *                       exact distances of each query's best candidates and
 *                       a proof that no other list can enter (else the exact
 *                       scan for that query): the same lists as the exact
 *                       scan; 0: always the exact fp32 scan; 1: the tensor-
 *                       core path whenever nlist >= 256 and dim >= 64;
 *                       2: as 1 with every query sent to the exact fallback
 * "ivf.split" and "ivf.tc_coarse" left at -1 also take the autotuner's
 * choice where an entry covers the call. Unknown keys return FV_ERR_ARG.
 * Values apply to launches issued after the call. */
int fv_tune_set(const char* key, int64_t value);
int fv_tune_get(const char* key, int64_t* value);
/* The committed autotuner entry a tensor-core scan of this shape uses
 * (fp8: 0 fp16 rows, 1 e4m3 rows): out_knobs[4] = {pair, prepass, stride,
 * overfetch}. FV_ERR_ARG when no entry applies (or "tc.table" is 0). */
/* The committed autotuner entry an IVF search of this shape uses (mode: 0
 * PQ, 1 SQ8, 2 RaBitQ): out_knobs[3] = {pipeline, split, tc_coarse}, -1 for
 * automatic. FV_ERR_ARG when no entry applies (or "tc.table" is 0). */
int fv_tune_lookup_ivf(int mode, uint32_t dim, uint64_t num_vectors, uint32_t nlist, uint32_t num_queries,
                       uint32_t nprobe, int32_t* out_knobs);
int fv_tune_lookup(int fp8, MetricType metric, uint32_t dim, uint64_t num_vectors, uint32_t num_queries,
                   uint32_t top_k, int32_t* out_knobs);
/* Installs a caller-owned device buffer as the scratch arena of `stream`
 * (kernels that need scratch then never allocate on that stream; a call
 * needing more than `bytes` fails with cudaErrorMemoryAllocation).
 * d_ptr == NULL removes the caller buffer and returns to library-managed
 * stream-ordered allocation. Replaces the reference's per-call
 * cudaMallocAsync in ivf_pq_lookup.cu:397-401. */
int fv_set_stream_scratch(void* stream, void* d_ptr, size_t bytes);
/* Frees the library-managed scratch arena of `stream`. */
int fv_release_stream_scratch(void* stream);

#ifdef __cplusplus
}
#endif

#endif /* FV_BRIDGE_H */
