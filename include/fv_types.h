/*
 * fv_types.h -- plain-old-data types that cross the C ABI of libfvgb300.
 *
 * Layout contract: every struct below that has a counterpart in the
 * reference (FlashVector-GPU kernels/include/types.h) keeps that
 * counterpart's field order, field types and alignment, so that a caller
 * built against the reference header (the Rust `#[repr(C)]` mirrors in
 * crates/engine/src/ffi.rs:20-232) can pass its structs unchanged.
 * New structs (FP8 tables, list-major IVF layouts, status words) carry an
 * `Fv` prefix and have no reference counterpart.
 */
#ifndef FV_TYPES_H
#define FV_TYPES_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
#define FV_ALIGN8 alignas(8)
extern "C" {
#else
#define FV_ALIGN8 _Alignas(8)
#endif

/* Distance metric. Values as kernels/include/types.h:15-19 (L2=0, Cosine=1,
 * InnerProduct=2). L2 is the squared Euclidean distance, inner product is
 * reported as -dot so that smaller is always better, cosine as 1-cos. */
typedef enum {
    METRIC_L2 = 0,
    METRIC_COSINE = 1,
    METRIC_INNER_PRODUCT = 2
} MetricType;

/* One (id, distance) hit; 8 bytes, 8-byte aligned (types.h:39-42; the
 * alignment sits on the first member, the form both C11 and C++ accept).
 * Unfilled slots are {0xFFFFFFFF, 1e30f}. */
typedef struct {
    FV_ALIGN8 uint32_t id;
    float distance;
} GpuSearchResult;

/* IVF-PQ tables, field order as types.h:85-97. All pointers are device (or
 * mapped-host for d_vectors) pointers owned by the caller. d_pq_codes is
 * indexed by vector id: row v holds the m_pq one-byte codes of vector v. */
typedef struct {
    const float* d_centroids;      /* [nlist * dim] coarse centroids            */
    const float* d_pq_codebooks;   /* [m_pq * 256 * sub_dim] sub-space codewords */
    const uint8_t* d_pq_codes;     /* [num_vectors * m_pq]                       */
    const uint32_t* d_ivf_offsets; /* [nlist + 1] posting-list prefix offsets    */
    const uint32_t* d_ivf_vec_ids; /* [num_vectors] vector ids in list order     */
    const float* d_vectors;        /* [num_vectors * dim] fp32 rows for rerank   */
    uint32_t num_vectors;
    uint32_t dim;
    uint32_t nlist;
    uint32_t m_pq;
    uint32_t sub_dim;
} IvfPqGpuTables;

/* IVF-SQ8 tables, field order as types.h:100-111. */
typedef struct {
    const float* d_centroids;      /* [nlist * dim]                              */
    const float* d_sq_mins;        /* [dim] per-dimension residual minimum       */
    const float* d_sq_scales;      /* [dim] per-dimension step (range / 255)     */
    const uint8_t* d_sq_codes;     /* [num_vectors * dim] indexed by vector id   */
    const uint32_t* d_ivf_offsets; /* [nlist + 1]                                */
    const uint32_t* d_ivf_vec_ids; /* [num_vectors]                              */
    const float* d_vectors;        /* [num_vectors * dim] fp32 rows for rerank   */
    uint32_t num_vectors;
    uint32_t dim;
    uint32_t nlist;
} IvfSqGpuTables;

/* IVF-RaBitQ tables, field order as types.h:113-128. padded_dim is the
 * power of two >= max(dim, 32) that the rotation works in, words_per_vec =
 * padded_dim / 32. Row v of d_rabitq_bits holds the sign bits of vector v's
 * rotated residual (bit d of word d / 32 set when coordinate d >= 0); row v
 * of d_rabitq_meta holds {|r|^2, |r|^2 / sum_d |rot r|_d, popcount, |x|^2}. */
typedef struct {
    const float* d_centroids;      /* [nlist * dim] coarse centroids            */
    const float* d_rot_centroids;  /* [nlist * padded_dim] rotated centroids    */
    const uint32_t* d_rabitq_bits; /* [num_vectors * words_per_vec]             */
    const float* d_rabitq_meta;    /* [num_vectors * 4]                         */
    const float* d_rot_signs;      /* [3 * padded_dim] +-1 per rotation round   */
    const uint32_t* d_ivf_offsets; /* [nlist + 1]                               */
    const uint32_t* d_ivf_vec_ids; /* [num_vectors]                             */
    const float* d_vectors;        /* [num_vectors * dim] fp32 rows for rerank  */
    uint32_t num_vectors;
    uint32_t dim;
    uint32_t padded_dim;
    uint32_t words_per_vec;
    uint32_t nlist;
} IvfRabitqGpuTables;

/* FP16 flat tables, field order as types.h:131-138. padded_dim is a
 * multiple of 16; columns dim..padded_dim-1 of each fp16 row are zero.
 * When d_vectors (fp32 copy, row stride dim) is non-null the scan is
 * followed by an exact fp32 rescore of an over-fetched shortlist. */
typedef struct {
    const uint16_t* d_vectors_fp16; /* [num_vectors * padded_dim] IEEE binary16 */
    const float* d_vec_norms_sq;    /* [num_vectors] ||x||^2 of the fp32 row     */
    const float* d_vectors;         /* optional [num_vectors * dim] fp32 rows    */
    uint32_t num_vectors;
    uint32_t dim;
    uint32_t padded_dim;
} Fp16GpuTables;

/* FP8 (E4M3) flat tables; no reference counterpart. Two layouts, chosen by
 * scale_mode.
 * scale_mode 0 (fv_encode_fp8; the zero default): one power-of-two
 * scale s = 2^b for the table, the smallest with max_v ||x_v||^2 <= 896 s^2
 * (1 for an all-zero table); every d_scales[v] holds s. Row v of
 * d_vectors_fp8 holds round_e4m3(x_v[d] / s) for d < dim (round to nearest
 * even), then three norm digits n1, n2, n3 at columns dim..dim+2 (n1 the
 * e4m3 value nearest ||x_v||^2 / (2 s^2), n2 and n3 the e4m3 values nearest
 * what the earlier digits leave), then zero padding up to padded_dim (a
 * multiple of 16, >= dim + 3). d_vec_norms_sq holds ||x_v||^2 of the fp32
 * row (compensated sum).
 * scale_mode 1 (fv_encode_fp8_per_vector): per-vector scales d_scales[v] =
 * max|x_v| / 448 (1 for a zero row), codes round_e4m3(x_v[d] / d_scales[v]),
 * zero padding from dim (padded_dim a multiple of 16, >= dim); the scan then
 * applies each row's scale and norm per value. */
typedef struct {
    const uint8_t* d_vectors_fp8;   /* [num_vectors * padded_dim] E4M3 bytes     */
    const float* d_scales;          /* [num_vectors] per-vector dequant scale    */
    const float* d_vec_norms_sq;    /* [num_vectors] ||x||^2 of the fp32 row     */
    const float* d_vectors;         /* optional [num_vectors * dim] fp32 rows    */
    uint32_t num_vectors;
    uint32_t dim;
    uint32_t padded_dim;
    uint32_t scale_mode;            /* 0: table scale + norm digits, 1: per-vector */
} FvFp8GpuTables;

/* Tuning knobs of the reduced-precision flat scans; no reference
 * counterpart. Zero in any field selects the default. */
typedef struct {
    uint32_t overfetch;      /* shortlist = overfetch * top_k (default 4)      */
    uint32_t boundary_fp64;  /* 1 = fp64 re-rank of ties at the k-th boundary  */
    float boundary_eps;      /* relative band around the k-th distance (fp64)  */
    uint32_t splits;         /* base-range splits per query block (0 = auto)   */
} FvScanOptions;

/* Options of the IVF extensions; no reference counterpart. */
typedef struct {
    uint32_t codes_list_major; /* 1: d_pq_codes / d_sq_codes / d_rabitq_bits and
                                  d_rabitq_meta row i belongs to list position i
                                  (fv_ivf_relayout_codes), 0: row v = id v */
    uint32_t reserved[3];
} FvIvfOptions;

/* ---- host engine (the reference's GpuVectorIndex, index.rs:131-2634) ---- */

/* Index configuration; dim / nlist / m_pq / metric as IndexConfig
 * (types.h:74-82). The graph fields of the reference (m, ef_construction)
 * belong to engines outside the scan path and are absent. */
typedef struct {
    uint32_t dim;
    uint32_t metric;        /* MetricType                                     */
    uint32_t nlist;         /* IVF lists (0 = no IVF tables)                  */
    uint32_t m_pq;          /* PQ sub-quantisers (0 = no IVF-PQ)              */
    uint32_t build_flags;   /* FV_BUILD_* bits (0 = FP16 | IVF_PQ | IVF_SQ8 |
                               IVF_RABITQ, the reference's build)            */
    uint32_t kmeans_iters;  /* Lloyd iterations (0 = 10)                      */
    uint32_t pq_iters;      /* per-sub-space k-means iterations (0 = 10)      */
    uint32_t train_rows;    /* rows sampled to train centroids / codebooks
                               (0 = min(n, 256 * nlist))                       */
    uint32_t streams;       /* search stream pool size (0 = 4)               */
    uint32_t kmeans_iters_given; /* Lloyd iterations when initial centroids are
                                    given to fv_index_build_device            */
    uint64_t seed;
} FvIndexConfig;

#define FV_BUILD_FP16 1u
#define FV_BUILD_FP8 2u
#define FV_BUILD_IVF_PQ 4u
#define FV_BUILD_IVF_SQ8 8u
#define FV_BUILD_IVF_RABITQ 16u

/* Search engines of the scan path. */
enum {
    FV_ENGINE_FLAT = 0,    /* exact fp32 scan (cuda_flat_scan_batch)          */
    FV_ENGINE_FP16 = 1,    /* fp16 tensor-core scan + fp32 rescore            */
    FV_ENGINE_FP8 = 2,     /* e4m3 tensor-core scan + fp32 rescore            */
    FV_ENGINE_IVF_PQ = 3,  /* IvfQuantMode::Pq                                */
    FV_ENGINE_IVF_SQ8 = 4, /* IvfQuantMode::Sq8                               */
    FV_ENGINE_IVF_RABITQ = 5 /* IvfQuantMode::Rabitq                          */
};

typedef struct {
    uint32_t engine;       /* FV_ENGINE_*                                     */
    uint32_t top_k;
    uint32_t nprobe;       /* IVF                                             */
    uint32_t rerank_k;     /* IVF                                             */
    FvScanOptions scan;    /* FP16 / FP8                                      */
} FvSearchParams;

/* Latency statistics of MetricsTracker::get_stats (metrics.rs:47-90):
 * per-query amortised batch latency in microseconds, QPS since creation. */
typedef struct {
    uint64_t count;
    double p50_us, p90_us, p99_us, p999_us, min_us, max_us, mean_us, qps;
} FvLatencyStats;

typedef struct {
    uint32_t num_vectors;  /* main slots                                      */
    uint32_t delta_len;    /* live-insert buffer rows                         */
    uint32_t tombstones;
    uint32_t dim, padded_dim, nlist, m_pq, metric;
    uint32_t next_id;
    uint32_t reserved;
    uint64_t device_bytes;
} FvIndexInfo;

#undef FV_ALIGN8

#ifdef __cplusplus
}
#endif

#endif /* FV_TYPES_H */
