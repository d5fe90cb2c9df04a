/*
 * fv_serve.h -- continuous-batching request loop over an FvIndex.
 *
 * Replaces the reference's SearchBatcher (crates/server/src/batcher.rs:82-259):
 * queries submitted one at a time are coalesced into batched launches and
 * each caller gets its own top-k back. Differences, all GB300-first:
 *
 *   - Several batches are in flight at once, each on its own CUDA stream
 *     with its own pinned staging and device buffers (the reference awaits
 *     one spawn_blocking batch at a time, batcher.rs:186).
 *   - Heterogeneous batches: requests with different filters share one
 *     launch (each query carries its own filter row); IVF requests with
 *     different top_k / nprobe / rerank_k share one launch too. Flat and
 *     tensor-core requests batch per (engine, top_k), since their
 *     over-fetch depends on k. With group_by_params = 1 requests batch only
 *     with equal (engine, top_k, nprobe, rerank_k), the reference's BatchKey
 *     rule (batcher.rs:55-61).
 *   - Dispatch is work-conserving: a batch launches as soon as a stream is
 *     free and either the GPU is idle, a class holds max_batch requests, or
 *     its oldest request has waited max_wait_us (the reference always waits
 *     out its window, batcher.rs:139-160).
 *   - Every answer is the answer the engine's blocking search
 *     (fv_index_search) gives that query alone: same clamps, same masks
 *     (tombstones AND the request's filter), same live-insert merge.
 *   - Completion is signalled from the stream (a host function), so no
 *     thread blocks on a stream; latency is measured from arrival (submit,
 *     or the scheduled time of a replayed trace) to completion.
 *   - Admission by scratch memory (the reference gives each stream a fixed
 *     scratch budget, crates/engine/src/streams.rs:43-69): the server owns
 *     one device pool of scratch_budget_kb; a batch is launched only when
 *     its scratch (the exact size its launches take, computed from the same
 *     plan the kernels use) fits in the free part of the pool, else it waits
 *     for batches in flight to finish. A batch whose scratch exceeds the
 *     whole pool is cut into smaller batches; a single request that still
 *     exceeds it fails with FV_ERR_SCRATCH_LIMIT. Device memory therefore
 *     never grows with the load.
 *
 * The index must outlive the server; build / add / delete on the index
 * wait for the batches in flight.
 */
#ifndef FV_SERVE_H
#define FV_SERVE_H

#include "fv_bridge.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct FvServe FvServe;

typedef struct {
    uint32_t max_batch;       /* requests per launch (0: 256; the reference uses 64)        */
    uint32_t max_wait_us;     /* batching window while the GPU is busy (reference: 350)     */
    uint32_t inflight;        /* batches in flight, one stream each (0: 4)                  */
    uint32_t group_by_params; /* 1: batch only equal (engine, top_k, nprobe, rerank_k)       */
    uint32_t queue_capacity;  /* pending requests admitted (0: unbounded); beyond it submit
                                 returns FV_ERR_QUEUE_FULL                                  */
    uint32_t scratch_budget_kb; /* device scratch of all batches in flight together, KiB (0:
                                   512 MiB); one pool of this size is allocated at create  */
    uint32_t graphs;          /* 1: each batch's kernels run as one CUDA graph, captured on
                                 its stream and applied (cudaGraphExecUpdate) to the
                                 stream's executable graph of the same launch shape
                                 (engine, batch size, k, nprobe, rerank_k, filtered or not),
                                 instantiated when the shape is new; a batch whose capture
                                 the driver invalidates runs as plain launches; 0: launched
                                 one by one                                                */
    uint32_t reserved;
} FvServeConfig;

typedef struct {
    uint32_t engine;     /* FV_ENGINE_*                                              */
    uint32_t top_k;      /* 1..256                                                   */
    uint32_t nprobe;     /* IVF engines                                              */
    uint32_t rerank_k;   /* IVF engines (0: top_k; 1: no exact rerank)               */
    int32_t filter_id;   /* fv_serve_add_filter id, or -1 for no filter              */
    uint32_t reserved;
} FvRequest;

typedef struct {
    /* BatcherStats (batcher.rs:63-68) */
    uint64_t total_requests;
    uint64_t total_batches;
    double avg_batch_size;
    /* completions since the last reset */
    uint64_t completed;
    uint64_t failed;
    double qps;          /* completed / (last completion - first arrival)          */
    double p50_us, p90_us, p99_us, p999_us, max_us, mean_us;  /* arrival -> completion */
    double queue_p50_us, queue_p99_us;                         /* arrival -> launch     */
    uint32_t max_inflight;
    uint32_t graph_instantiations; /* executable graphs built since create (graphs = 1)   */
    /* admission by scratch memory */
    uint64_t scratch_waits;       /* times a ready batch waited for scratch to free up      */
    uint64_t scratch_split;       /* batches cut smaller to fit the budget                  */
    uint64_t scratch_peak_bytes;  /* most scratch held by the batches in flight at once     */
    uint64_t scratch_pool_bytes;  /* the budget (pool size)                                 */
    uint64_t graph_fallbacks;     /* graphs = 1: batches whose capture the driver invalidated
                                     (a kernel's first launch in the process loads its module)
                                     and that ran as plain launches, since create           */
} FvServeStats;

/* A batch executor for a server without an index (host-only use and
 * tests, like SearchBatcher::with_executor, batcher.rs:127-131): fills
 * out[i * k_stride + r] for the nq requests of one batch and returns 0 or
 * an error code that every request of the batch then reports. */
typedef int (*FvServeExecutor)(void* user, const FvRequest* requests, const float* queries, uint32_t nq,
                               uint32_t dim, uint32_t k_stride, GpuSearchResult* out);

/* SearchBatcher::for_index (batcher.rs:89-125) over the native engine. */
int fv_serve_create(FvIndex* index, const FvServeConfig* config, FvServe** out);
/* SearchBatcher::with_executor (batcher.rs:127-226); no CUDA call is made. */
int fv_serve_create_with_executor(uint32_t dim, const FvServeConfig* config, FvServeExecutor executor, void* user,
                                  FvServe** out);
/* Processes every submitted request, then stops. */
int fv_serve_destroy(FvServe* server);

/* Registers a filter: packed LSB-first u32 words over logical ids (ids at
 * or beyond 32 * num_words are filtered out). Requests name it by id. A
 * removed filter stays valid for the requests already submitted. */
int fv_serve_add_filter(FvServe* server, const uint32_t* words, uint32_t num_words, int32_t* out_id);
int fv_serve_remove_filter(FvServe* server, int32_t id);

/* SearchBatcher::submit (batcher.rs:228-247), split in two so that a C
 * caller need not block: submit copies the query and returns a ticket;
 * wait blocks (at most timeout_ms; 0 = no limit) until that request is
 * answered, copies min(out_len, top_k) results, frees the ticket and
 * returns the request's status. out_latency_us (optional) receives
 * arrival -> completion. */
int fv_serve_submit(FvServe* server, const FvRequest* request, const float* query, uint64_t* out_ticket);
int fv_serve_wait(FvServe* server, uint64_t ticket, GpuSearchResult* out, uint32_t out_len, uint32_t timeout_ms,
                  double* out_latency_us);

/* Open-loop replay of a request trace: request i (query row i) arrives at
 * start + arrival_ns[i] (non-decreasing offsets); it is submitted then, its
 * latency counted from then, whatever the queue. Blocks until all are
 * answered; out[i * out_stride ...] receives request i's top_k results
 * (out_stride >= every top_k), out_status[i] (optional) its status. */
int fv_serve_replay(FvServe* server, const FvRequest* requests, const float* queries, const uint64_t* arrival_ns,
                    uint32_t num_requests, GpuSearchResult* out, uint32_t out_stride, int32_t* out_status);

/* The scratch bytes one launched batch of `nq` requests like `request`
 * takes (what admission charges against scratch_budget_kb). */
int fv_serve_scratch_estimate(FvServe* server, const FvRequest* request, uint32_t nq, uint64_t* out_bytes);

int fv_serve_stats(FvServe* server, FvServeStats* out);
int fv_serve_reset_stats(FvServe* server);

#ifdef __cplusplus
}
#endif

#endif /* FV_SERVE_H */
