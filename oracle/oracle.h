/*
 * oracle.h -- CPU restatement of FlashVector-GPU's distance-scan path.
 *
 * TEST INFRASTRUCTURE ONLY. This library is the checker the parity tests,
 * the smoke check and the CPU-baseline leg of the benchmark compare the
 * CUDA path against. The product (libfvgb300) never links, loads or calls
 * it.
 *
 * Every function cites the reference file:line it restates. Floating-point
 * order matters here: the build recipe compiles with -ffp-contract=off so
 * that `a + b * c` is never fused unless fmaf() is written out, matching
 * the reference's Rust (no contraction) and its CUDA (explicit fmaf).
 */
#ifndef FV_ORACLE_H
#define FV_ORACLE_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct {
    uint32_t id;
    float distance;
} FvoResult; /* same layout as GpuSearchResult */

enum { FVO_L2 = 0, FVO_COSINE = 1, FVO_IP = 2 };

/* Exact fp32 search, the order of RecallEvaluator::exact_knn
 * (crates/engine/src/metrics.rs:103-135): per (query, row) the squared
 * differences are summed in ascending dimension order with separately
 * rounded operations; results sorted by (distance, slot) and truncated to
 * k (Rust's stable sort keeps the lower slot on ties). Extended, in the
 * same summation order, with inner product (-dot) and the cosine formula of
 * distance_metrics.cuh:97-99, an optional slot mask (LSB-first words,
 * distance_metrics.cuh:17-20) and an optional slot->id map (applied to the
 * output ids only). Unfilled outputs are {0xFFFFFFFF, 1e30}. A candidate is
 * admissible when its distance is < 1e30 (sparse_hybrid.cu:64). */
void fvo_exact_knn_f32(const float* base, const uint32_t* vec_ids, uint32_t n, uint32_t dim,
                       const float* queries, uint32_t nq, uint32_t k, int metric,
                       const uint32_t* mask, FvoResult* out, int threads);

/* FP64 brute force: per (query, row) the distance accumulated in double,
 * ties to the lower slot; the numpy FakeBackend of
 * python/tests_adapters/fake_backend.py:74-129 is its model. out_dist may
 * be NULL. Cosine uses 1 - dot / (|q| |x|). */
void fvo_bruteforce_f64(const float* base, uint32_t n, uint32_t dim, const float* queries, uint32_t nq,
                        uint32_t k, int metric, const uint32_t* mask, uint32_t* out_ids, double* out_dist,
                        int threads);

/* The reference's warp-cooperative fp32 distance (distance_metrics.cuh:53-138):
 * 32 lane partials over d = l, l+32, ... with fmaf, then the shuffle-down
 * reduction tree 16, 8, 4, 2, 1. Cosine is evaluated with IEEE sqrt and
 * division (the reference builds with --use_fast_math; see DESIGN). */
float fvo_warp_distance(const float* q, const float* x, uint32_t dim, int metric);
void fvo_distance_matrix(const float* queries, const float* base, uint32_t nq, uint32_t n, uint32_t dim,
                         int metric, float* out);

/* FP16 conversion of crates/engine/src/quant.rs:239-302 (rounds half away
 * from zero on the mantissa, truncates subnormals -- not round-to-nearest-
 * even), and the padded encoder of quant.rs:306-327 (pad to 16, norms as
 * the sequential fp32 sum of the fp32 squares). */
uint16_t fvo_f32_to_f16(float x);
float fvo_f16_to_f32(uint16_t h);
void fvo_encode_fp16_padded(const float* x, uint32_t n, uint32_t dim, uint16_t* out, float* norms_sq);

/* Scalar quantiser of quant.rs:14-75. */
void fvo_sq8_fit(const float* residuals, uint32_t n, uint32_t dim, float* mins, float* scales);
void fvo_sq8_encode(const float* residuals, uint32_t n, uint32_t dim, const float* mins, const float* scales,
                    uint8_t* codes);

/* Seeded k-means of cluster.rs:28-189 (k-means++ on a shuffled seed pool of
 * min(n, 64k) rows, Lloyd iterations, empty-cluster recovery from the row
 * farthest from the global mean among 500 draws, stop when the largest
 * centroid move^2 < 1e-4). The reference draws from thread_rng; this one
 * from a seeded splitmix64 stream, so runs are reproducible. */
void fvo_kmeans(const float* x, uint32_t n, uint32_t dim, uint32_t k, uint32_t iters, uint64_t seed,
                float* centroids, uint32_t* assign, int threads);

/* Product quantiser of cluster.rs:202-287: 256 codewords per sub-space
 * trained by fvo_kmeans (unused codewords set to FLT_MAX), nearest-codeword
 * encode with strict `<`. */
void fvo_pq_train(const float* x, uint32_t n, uint32_t dim, uint32_t m_pq, uint32_t iters, uint64_t seed,
                  float* codebooks, int threads);
void fvo_pq_encode(const float* x, uint32_t n, uint32_t dim, uint32_t m_pq, const float* codebooks,
                   uint8_t* codes, int threads);

/* IVF build of crates/engine/src/index.rs:405-458: nlist clamped to
 * [1, n], k-means (25 iterations), residuals x - centroid(x), posting lists
 * of ascending vector ids. offsets has nlist + 1 entries. */
void fvo_ivf_lists(const uint32_t* assign, uint32_t n, uint32_t nlist, uint32_t* offsets, uint32_t* vec_ids);
void fvo_residuals(const float* x, uint32_t n, uint32_t dim, const float* centroids, const uint32_t* assign,
                   float* out);

/* IVF-PQ search (ivf_pq_lookup.cu:95-221, 226-337, 339-444): clamps of
 * launch_ivf_pq_search (:351-362); coarse top-nprobe by L2 with fmaf in
 * dimension order (ivf_rerank.cuh:78-84; exact here, by (distance, list)
 * -- the reference's per-thread merge is not exact above nprobe 32);
 * residual LUT (:150-162); ADC sum over sub-spaces in order (:176-178);
 * shortlist = top `shortlist` by (ADC, id); exact rerank with the warp-
 * order distance when rerank_k != 1 and vectors != NULL (:39-57); output
 * the first top_k by (distance, id). Returns the clamped top_k. */
uint32_t fvo_ivf_pq_search(const float* centroids, const float* codebooks, const uint8_t* codes,
                           const uint32_t* offsets, const uint32_t* vec_ids, const float* vectors,
                           uint32_t num_vectors, uint32_t dim, uint32_t nlist, uint32_t m_pq, uint32_t sub_dim,
                           const float* queries, uint32_t nq, uint32_t top_k, uint32_t nprobe, uint32_t rerank_k,
                           int metric, const uint32_t* mask, FvoResult* out, int threads);

/* IVF-SQ8 search (ivf_quant_lookup.cu:18-125, 127-230, 232-327): same
 * clamps and structure; the approximate distance is the squared L2 between
 * the query residual and fmaf(code, scale, min), dimension order. */
uint32_t fvo_ivf_sq_search(const float* centroids, const float* mins, const float* scales, const uint8_t* codes,
                           const uint32_t* offsets, const uint32_t* vec_ids, const float* vectors,
                           uint32_t num_vectors, uint32_t dim, uint32_t nlist, const float* queries, uint32_t nq,
                           uint32_t top_k, uint32_t nprobe, uint32_t rerank_k, int metric, const uint32_t* mask,
                           FvoResult* out, int threads);

/* RaBitQ (quant.rs:91-235, ivf_quant_lookup.cu:333-870).
 * padded_dim P = next power of two >= max(dim, 32); rot_signs: 3 P signs
 * from a splitmix64 stream (quant.rs:100-116); the rotation is three rounds
 * of sign flip, Walsh-Hadamard butterflies and a 1/sqrt(P) scale, the
 * scale being the correctly rounded 1.0f / sqrtf(P) of the host encoder
 * (quant.rs:124; the reference's query kernel takes rsqrtf instead).
 * encode: rot_centroids [nlist][P], bits [n][P/32] (bit d = rotated residual
 * coordinate d >= 0), meta [n][4] = {|r|^2, |r|^2 / sum|rot r| (0 when
 * either is <= 1e-12), popcount, |x|^2}, norms summed sequentially. */
uint32_t fvo_rabitq_padded_dim(uint32_t dim);
void fvo_rabitq_rot_signs(uint32_t padded_dim, uint64_t seed, float* out);
float fvo_rabitq_inv_sqrt(uint32_t padded_dim);
void fvo_rabitq_rotate(const float* v, uint32_t len, const float* signs, uint32_t padded_dim, float* out);
void fvo_rabitq_encode(const float* x, uint32_t n, uint32_t dim, const float* centroids, uint32_t nlist,
                       const uint32_t* assign, const float* signs, uint32_t padded_dim, float* rot_centroids,
                       uint32_t* bits, float* meta, int threads);
/* One row's estimated distance from the 4 query bit-planes (planes[j][w]). */
float fvo_rabitq_estimate(const uint32_t* b, const float* m, const uint32_t* planes, uint32_t W, uint32_t P,
                          float q_min, float delta, float sum_u, float q_c, float q_norm_sq, int metric);
/* IVF-RaBitQ search: clamps and coarse probe as IVF-PQ; per probed list the
 * rotated query residual is quantised to 4 bits over [min, max] and every
 * posting gets the popcount estimate (L2, or IP / cosine forms of it);
 * shortlist by (estimate, id); exact rerank; top_k by (distance, id).
 * ||q||^2 (inner product only) is summed in the order of a 256-thread block
 * (ivf_quant_lookup.cu:686-697). Returns the clamped top_k. */
uint32_t fvo_ivf_rabitq_search(const float* centroids, const float* rot_centroids, const uint32_t* bits,
                               const float* meta, const float* signs, const uint32_t* offsets,
                               const uint32_t* vec_ids, const float* vectors, uint32_t num_vectors, uint32_t dim,
                               uint32_t padded_dim, uint32_t nlist, const float* queries, uint32_t nq,
                               uint32_t top_k, uint32_t nprobe, uint32_t rerank_k, int metric, const uint32_t* mask,
                               FvoResult* out, int threads);

/* Coarse probe order only (top-nprobe list ids per query, by (dist, id)). */
void fvo_coarse_probe(const float* centroids, uint32_t nlist, uint32_t dim, const float* queries, uint32_t nq,
                      uint32_t nprobe, uint32_t* out_lists, float* out_dist, int threads);

/* recall = |approx ∩ truth| / |truth| per query, averaged
 * (metrics.rs:138-147); invalid ids (0xFFFFFFFF) never match. */
double fvo_recall(const uint32_t* approx, uint32_t approx_stride, const uint32_t* truth, uint32_t truth_stride,
                  uint32_t nq, uint32_t k);

#ifdef __cplusplus
}
#endif

#endif /* FV_ORACLE_H */
