/*
 * oracle.c -- CPU restatement of FlashVector-GPU's distance-scan path.
 * TEST INFRASTRUCTURE ONLY (see oracle.h). Build: oracle/Makefile
 * (-O2 -ffp-contract=off, no fast-math).
 */
#include "oracle.h"

#include <float.h>
#include <math.h>
#include <stdlib.h>
#include <string.h>

#ifdef _OPENMP
#include <omp.h>
#endif

#define SENT_ID 0xFFFFFFFFu
#define SENT_DIST 1e30f

/* ------------------------------------------------------------ key utils */
/* (distance, slot) ordered as one 64-bit key; -0.0 folded onto +0.0. */
static inline uint64_t key_of(float d, uint32_t slot) {
    d = d + 0.0f;
    uint32_t u;
    memcpy(&u, &d, 4);
    u = (u & 0x80000000u) ? ~u : (u | 0x80000000u);
    return ((uint64_t)u << 32) | slot;
}
static inline float key_dist(uint64_t k) {
    uint32_t o = (uint32_t)(k >> 32);
    uint32_t u = (o & 0x80000000u) ? (o & 0x7FFFFFFFu) : ~o;
    float f;
    memcpy(&f, &u, 4);
    return f;
}
static inline int mask_ok(const uint32_t* mask, uint32_t i) {
    return mask == NULL || ((mask[i >> 5] >> (i & 31u)) & 1u);
}

/* bounded max-heap of keys */
typedef struct {
    uint64_t* h;
    uint32_t cap, size;
} Heap;

static void heap_push(Heap* hp, uint64_t key) {
    uint64_t* h = hp->h;
    if (hp->size < hp->cap) {
        uint32_t i = hp->size++;
        while (i > 0) {
            uint32_t p = (i - 1) / 2;
            if (h[p] >= key) break;
            h[i] = h[p];
            i = p;
        }
        h[i] = key;
        return;
    }
    if (hp->cap == 0 || key >= h[0]) return;
    uint32_t i = 0, n = hp->size;
    for (;;) {
        uint32_t l = 2 * i + 1;
        if (l >= n) break;
        uint32_t c = l;
        if (l + 1 < n && h[l + 1] > h[l]) c = l + 1;
        if (h[c] <= key) break;
        h[i] = h[c];
        i = c;
    }
    h[i] = key;
}

static int cmp_u64(const void* a, const void* b) {
    uint64_t x = *(const uint64_t*)a, y = *(const uint64_t*)b;
    return x < y ? -1 : (x > y);
}

static void heap_sorted(Heap* hp) { qsort(hp->h, hp->size, sizeof(uint64_t), cmp_u64); }

static void set_threads(int threads) {
#ifdef _OPENMP
    if (threads > 0) omp_set_num_threads(threads);
#else
    (void)threads;
#endif
}

/* ------------------------------------------------------ exact fp32 scan */
static float seq_distance(const float* q, const float* x, uint32_t dim, int metric, float qn) {
    if (metric == FVO_L2) {
        float s = 0.0f;
        for (uint32_t d = 0; d < dim; ++d) {
            float t = q[d] - x[d];
            s = s + t * t;
        }
        return s;
    }
    float dot = 0.0f;
    for (uint32_t d = 0; d < dim; ++d) dot = dot + q[d] * x[d];
    if (metric == FVO_IP) return -dot;
    float xn = 0.0f;
    for (uint32_t d = 0; d < dim; ++d) xn = xn + x[d] * x[d];
    float denom = sqrtf(qn) * sqrtf(xn);
    denom = denom + 1e-8f;
    return 1.0f - dot / denom;
}

void fvo_exact_knn_f32(const float* base, const uint32_t* vec_ids, uint32_t n, uint32_t dim,
                       const float* queries, uint32_t nq, uint32_t k, int metric,
                       const uint32_t* mask, FvoResult* out, int threads) {
    set_threads(threads);
#pragma omp parallel for schedule(dynamic, 1)
    for (int64_t qi = 0; qi < (int64_t)nq; ++qi) {
        const float* q = queries + (size_t)qi * dim;
        float qn = 0.0f;
        if (metric == FVO_COSINE)
            for (uint32_t d = 0; d < dim; ++d) qn = qn + q[d] * q[d];
        uint64_t* buf = (uint64_t*)malloc(sizeof(uint64_t) * (k ? k : 1));
        Heap hp = {buf, k, 0};
        for (uint32_t i = 0; i < n; ++i) {
            if (!mask_ok(mask, i)) continue;
            float dd = seq_distance(q, base + (size_t)i * dim, dim, metric, qn);
            if (!(dd < SENT_DIST)) continue;
            heap_push(&hp, key_of(dd, i));
        }
        heap_sorted(&hp);
        for (uint32_t r = 0; r < k; ++r) {
            FvoResult* o = out + (size_t)qi * k + r;
            if (r < hp.size) {
                uint32_t slot = (uint32_t)hp.h[r];
                o->id = vec_ids ? vec_ids[slot] : slot;
                o->distance = key_dist(hp.h[r]);
            } else {
                o->id = SENT_ID;
                o->distance = SENT_DIST;
            }
        }
        free(buf);
    }
}

/* ------------------------------------------------------- fp64 oracle */
typedef struct {
    double d;
    uint32_t id;
} DKey;

static int dkey_less(const DKey* a, const DKey* b) { return a->d < b->d || (a->d == b->d && a->id < b->id); }

void fvo_bruteforce_f64(const float* base, uint32_t n, uint32_t dim, const float* queries, uint32_t nq,
                        uint32_t k, int metric, const uint32_t* mask, uint32_t* out_ids, double* out_dist,
                        int threads) {
    set_threads(threads);
#pragma omp parallel for schedule(dynamic, 1)
    for (int64_t qi = 0; qi < (int64_t)nq; ++qi) {
        const float* q = queries + (size_t)qi * dim;
        double qn = 0.0;
        for (uint32_t d = 0; d < dim; ++d) qn += (double)q[d] * (double)q[d];
        DKey* top = (DKey*)malloc(sizeof(DKey) * (k + 1));
        uint32_t cnt = 0;
        for (uint32_t i = 0; i < n; ++i) {
            if (!mask_ok(mask, i)) continue;
            const float* x = base + (size_t)i * dim;
            double v;
            if (metric == FVO_L2) {
                double s = 0.0;
                for (uint32_t d = 0; d < dim; ++d) {
                    double t = (double)q[d] - (double)x[d];
                    s += t * t;
                }
                v = s;
            } else {
                double dot = 0.0, xn = 0.0;
                for (uint32_t d = 0; d < dim; ++d) {
                    dot += (double)q[d] * (double)x[d];
                    xn += (double)x[d] * (double)x[d];
                }
                if (metric == FVO_IP)
                    v = -dot;
                else
                    v = 1.0 - dot / (sqrt(qn) * sqrt(xn) + 1e-300);
            }
            DKey c = {v, i};
            if (cnt == k && !dkey_less(&c, &top[k - 1])) continue;
            /* insertion into the sorted array */
            uint32_t pos = cnt < k ? cnt : k - 1;
            while (pos > 0 && dkey_less(&c, &top[pos - 1])) {
                top[pos] = top[pos - 1];
                --pos;
            }
            top[pos] = c;
            if (cnt < k) ++cnt;
        }
        for (uint32_t r = 0; r < k; ++r) {
            out_ids[(size_t)qi * k + r] = r < cnt ? top[r].id : SENT_ID;
            if (out_dist) out_dist[(size_t)qi * k + r] = r < cnt ? top[r].d : 1e30;
        }
        free(top);
    }
}

/* ------------------------------------------- reference warp-order distance */
static float warp_tree(float p[32]) {
    /* __shfl_down_sync tree 16, 8, 4, 2, 1: lane l adds lane l+off (lanes
     * past the end add their own value, which never reaches lane 0) */
    float v[32];
    memcpy(v, p, sizeof(v));
    for (int off = 16; off > 0; off >>= 1) {
        float nv[32];
        for (int l = 0; l < 32; ++l) nv[l] = v[l] + (l + off < 32 ? v[l + off] : v[l]);
        memcpy(v, nv, sizeof(v));
    }
    return v[0];
}

float fvo_warp_distance(const float* q, const float* x, uint32_t dim, int metric) {
    float a[32], b[32], c[32];
    for (int l = 0; l < 32; ++l) {
        float dot = 0.0f, nq = 0.0f, nx = 0.0f, acc = 0.0f;
        for (uint32_t d = (uint32_t)l; d < dim; d += 32) {
            if (metric == FVO_L2) {
                float t = q[d] - x[d];
                acc = fmaf(t, t, acc);
            } else {
                dot = fmaf(q[d], x[d], dot);
                if (metric == FVO_COSINE) {
                    nq = fmaf(q[d], q[d], nq);
                    nx = fmaf(x[d], x[d], nx);
                }
            }
        }
        a[l] = metric == FVO_L2 ? acc : dot;
        b[l] = nq;
        c[l] = nx;
    }
    if (metric == FVO_L2) return warp_tree(a);
    if (metric == FVO_IP) return -warp_tree(a);
    float dot = warp_tree(a), nq = warp_tree(b), nx = warp_tree(c);
    float denom = sqrtf(nq) * sqrtf(nx);
    denom = denom + 1e-8f;
    return 1.0f - dot / denom;
}

void fvo_distance_matrix(const float* queries, const float* base, uint32_t nq, uint32_t n, uint32_t dim,
                         int metric, float* out) {
    for (uint32_t q = 0; q < nq; ++q)
        for (uint32_t v = 0; v < n; ++v)
            out[(size_t)q * n + v] = fvo_warp_distance(queries + (size_t)q * dim, base + (size_t)v * dim, dim, metric);
}

/* ------------------------------------------------------------------ fp16 */
uint16_t fvo_f32_to_f16(float x) {
    uint32_t bits;
    memcpy(&bits, &x, 4);
    uint16_t sign = (uint16_t)((bits >> 16) & 0x8000u);
    int32_t exp = (int32_t)((bits >> 23) & 0xffu);
    uint32_t mant = bits & 0x007fffffu;
    if (exp == 255) return mant == 0 ? (uint16_t)(sign | 0x7c00u) : (uint16_t)(sign | 0x7e00u);
    int32_t unb = exp - 127 + 15;
    if (unb >= 31) return (uint16_t)(sign | 0x7c00u);
    if (unb <= 0) {
        if (unb < -10) return sign;
        uint32_t m = (mant | 0x00800000u) >> (14 - unb);
        return (uint16_t)(sign | (uint16_t)m);
    }
    uint32_t rounded = mant + 0x1000u;
    if (rounded & 0x00800000u) {
        int32_t ne = unb + 1;
        if (ne >= 31) return (uint16_t)(sign | 0x7c00u);
        return (uint16_t)(sign | (uint16_t)(ne << 10));
    }
    return (uint16_t)(sign | (uint16_t)(unb << 10) | (uint16_t)(rounded >> 13));
}

float fvo_f16_to_f32(uint16_t h) {
    uint32_t sign = ((uint32_t)h & 0x8000u) << 16;
    uint32_t exp = (h >> 10) & 0x1fu;
    uint32_t mant = h & 0x03ffu;
    uint32_t out;
    if (exp == 0) {
        if (mant == 0) {
            out = sign;
        } else {
            int32_t e = -14;
            uint32_t m = mant;
            while ((m & 0x0400u) == 0) {
                m <<= 1;
                --e;
            }
            m &= 0x03ffu;
            out = sign | ((uint32_t)(e + 127) << 23) | (m << 13);
        }
    } else if (exp == 31) {
        out = sign | (0xffu << 23) | (mant << 13);
    } else {
        out = sign | ((exp + 112) << 23) | (mant << 13);
    }
    float f;
    memcpy(&f, &out, 4);
    return f;
}

void fvo_encode_fp16_padded(const float* x, uint32_t n, uint32_t dim, uint16_t* out, float* norms_sq) {
    uint32_t pd = (dim + 15) / 16 * 16;
    for (uint32_t i = 0; i < n; ++i) {
        const float* s = x + (size_t)i * dim;
        uint16_t* o = out + (size_t)i * pd;
        float nsq = 0.0f;
        for (uint32_t d = 0; d < dim; ++d) {
            nsq = nsq + s[d] * s[d];
            o[d] = fvo_f32_to_f16(s[d]);
        }
        for (uint32_t d = dim; d < pd; ++d) o[d] = 0;
        norms_sq[i] = nsq;
    }
}

/* ------------------------------------------------------------------- SQ8 */
void fvo_sq8_fit(const float* r, uint32_t n, uint32_t dim, float* mins, float* scales) {
    for (uint32_t d = 0; d < dim; ++d) {
        mins[d] = INFINITY;
        scales[d] = -INFINITY; /* holds maxs until the end */
    }
    for (uint32_t i = 0; i < n; ++i)
        for (uint32_t d = 0; d < dim; ++d) {
            float v = r[(size_t)i * dim + d];
            if (v < mins[d]) mins[d] = v;
            if (v > scales[d]) scales[d] = v;
        }
    for (uint32_t d = 0; d < dim; ++d) {
        if (n == 0) {
            mins[d] = 0.0f;
            scales[d] = 0.0f;
        }
        float range = scales[d] - mins[d];
        scales[d] = range > 1e-12f ? range / 255.0f : 0.0f;
    }
}

void fvo_sq8_encode(const float* r, uint32_t n, uint32_t dim, const float* mins, const float* scales,
                    uint8_t* codes) {
    for (uint32_t i = 0; i < n; ++i)
        for (uint32_t d = 0; d < dim; ++d) {
            float s = scales[d];
            uint8_t c = 0;
            if (s > 0.0f) {
                float q = roundf((r[(size_t)i * dim + d] - mins[d]) / s); /* Rust round: half away from zero */
                if (q < 0.0f) q = 0.0f;
                if (q > 255.0f) q = 255.0f;
                c = (uint8_t)q;
            }
            codes[(size_t)i * dim + d] = c;
        }
}

/* --------------------------------------------------------------- k-means */
static uint64_t sm64(uint64_t* s) {
    uint64_t z = (*s += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}
static uint64_t rng_below(uint64_t* s, uint64_t n) { return n ? sm64(s) % n : 0; }
static double rng_unit(uint64_t* s) { return (double)(sm64(s) >> 11) * (1.0 / 9007199254740992.0); }

static float l2_seq(const float* a, const float* b, uint32_t dim) {
    float s = 0.0f;
    for (uint32_t d = 0; d < dim; ++d) {
        float t = a[d] - b[d];
        s = s + t * t;
    }
    return s;
}

void fvo_kmeans(const float* x, uint32_t n, uint32_t dim, uint32_t k, uint32_t iters, uint64_t seed,
                float* cent, uint32_t* assign, int threads) {
    set_threads(threads);
    uint64_t rs = seed ^ 0x5DEECE66Dull;
    float* mean = (float*)calloc(dim, sizeof(float));
    for (uint32_t i = 0; i < n; ++i)
        for (uint32_t d = 0; d < dim; ++d) mean[d] = mean[d] + x[(size_t)i * dim + d];
    float inv = 1.0f / (float)n;
    for (uint32_t d = 0; d < dim; ++d) mean[d] = mean[d] * inv;

    /* k-means++ on a shuffled seed pool (cluster.rs:53-94) */
    uint32_t* idx = (uint32_t*)malloc(sizeof(uint32_t) * n);
    for (uint32_t i = 0; i < n; ++i) idx[i] = i;
    for (uint32_t i = n; i > 1; --i) {
        uint32_t j = (uint32_t)rng_below(&rs, i);
        uint32_t t = idx[i - 1];
        idx[i - 1] = idx[j];
        idx[j] = t;
    }
    uint64_t pool64 = (uint64_t)k * 64u;
    uint32_t pool = (uint32_t)(pool64 < n ? pool64 : n);
    if (pool == 0) pool = 1;
    float* closest = (float*)malloc(sizeof(float) * pool);
    memcpy(cent, x + (size_t)idx[0] * dim, sizeof(float) * dim);
    for (uint32_t i = 0; i < pool; ++i) closest[i] = l2_seq(x + (size_t)idx[i] * dim, cent, dim);
    for (uint32_t c = 1; c < k; ++c) {
        const float* last = cent + (size_t)(c - 1) * dim;
        if (c > 1)
            for (uint32_t i = 0; i < pool; ++i) {
                float cand = l2_seq(x + (size_t)idx[i] * dim, last, dim);
                if (cand < closest[i]) closest[i] = cand;
            }
        double total = 0.0;
        for (uint32_t i = 0; i < pool; ++i) total += (double)closest[i];
        uint32_t chosen = idx[pool - 1];
        if (total > 0.0) {
            double target = rng_unit(&rs) * total;
            for (uint32_t i = 0; i < pool; ++i) {
                target -= (double)closest[i];
                if (target <= 0.0) {
                    chosen = idx[i];
                    break;
                }
            }
        }
        memcpy(cent + (size_t)c * dim, x + (size_t)chosen * dim, sizeof(float) * dim);
    }
    free(closest);
    free(idx);

    float* next = (float*)malloc(sizeof(float) * (size_t)k * dim);
    uint64_t* counts = (uint64_t*)malloc(sizeof(uint64_t) * k);
    for (uint32_t it = 0; it < iters; ++it) {
#pragma omp parallel for schedule(static)
        for (int64_t i = 0; i < (int64_t)n; ++i) {
            const float* v = x + (size_t)i * dim;
            float best = INFINITY;
            uint32_t bc = 0;
            for (uint32_t c = 0; c < k; ++c) {
                float dd = l2_seq(v, cent + (size_t)c * dim, dim);
                if (dd < best) {
                    best = dd;
                    bc = c;
                }
            }
            assign[i] = bc;
        }
        memset(next, 0, sizeof(float) * (size_t)k * dim);
        memset(counts, 0, sizeof(uint64_t) * k);
        for (uint32_t i = 0; i < n; ++i) {
            uint32_t c = assign[i];
            counts[c]++;
            for (uint32_t d = 0; d < dim; ++d) next[(size_t)c * dim + d] = next[(size_t)c * dim + d] + x[(size_t)i * dim + d];
        }
        float max_delta = 0.0f;
        for (uint32_t c = 0; c < k; ++c) {
            float* nc = next + (size_t)c * dim;
            if (counts[c] > 0) {
                float ic = 1.0f / (float)counts[c];
                float delta = 0.0f;
                for (uint32_t d = 0; d < dim; ++d) {
                    nc[d] = nc[d] * ic;
                    float t = nc[d] - cent[(size_t)c * dim + d];
                    delta = delta + t * t;
                }
                if (delta > max_delta) max_delta = delta;
            } else {
                uint32_t far = (uint32_t)rng_below(&rs, n);
                float md = 0.0f;
                uint32_t draws = n < 500 ? n : 500;
                for (uint32_t t = 0; t < draws; ++t) {
                    uint32_t s = (uint32_t)rng_below(&rs, n);
                    float dd = l2_seq(x + (size_t)s * dim, mean, dim);
                    if (dd > md) {
                        md = dd;
                        far = s;
                    }
                }
                memcpy(nc, x + (size_t)far * dim, sizeof(float) * dim);
            }
        }
        memcpy(cent, next, sizeof(float) * (size_t)k * dim);
        if (max_delta < 1e-4f) break;
    }
    /* final assignment against the final centroids (the reference's last
     * assignment is against the previous centroids; index.rs:414-427 then
     * uses it with the final centroids -- the same here) */
    free(next);
    free(counts);
    free(mean);
}

void fvo_pq_train(const float* x, uint32_t n, uint32_t dim, uint32_t m_pq, uint32_t iters, uint64_t seed,
                  float* codebooks, int threads) {
    uint32_t sub = dim / m_pq;
    uint32_t kk = n < 256 ? n : 256;
    float* sv = (float*)malloc(sizeof(float) * (size_t)n * sub);
    uint32_t* asg = (uint32_t*)malloc(sizeof(uint32_t) * (n ? n : 1));
    for (uint32_t m = 0; m < m_pq; ++m) {
        for (uint32_t i = 0; i < n; ++i) memcpy(sv + (size_t)i * sub, x + (size_t)i * dim + m * sub, sizeof(float) * sub);
        float* cb = codebooks + (size_t)m * 256 * sub;
        if (kk > 0) fvo_kmeans(sv, n, sub, kk, iters, seed + 1000003ull * (m + 1), cb, asg, threads);
        for (uint32_t c = kk; c < 256; ++c)
            for (uint32_t d = 0; d < sub; ++d) cb[(size_t)c * sub + d] = FLT_MAX;
    }
    free(sv);
    free(asg);
}

void fvo_pq_encode(const float* x, uint32_t n, uint32_t dim, uint32_t m_pq, const float* codebooks,
                   uint8_t* codes, int threads) {
    set_threads(threads);
    uint32_t sub = dim / m_pq;
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < (int64_t)n; ++i) {
        for (uint32_t m = 0; m < m_pq; ++m) {
            const float* sv = x + (size_t)i * dim + m * sub;
            const float* cb = codebooks + (size_t)m * 256 * sub;
            float best = INFINITY;
            uint32_t bc = 0;
            for (uint32_t c = 0; c < 256; ++c) {
                float dd = l2_seq(sv, cb + (size_t)c * sub, sub);
                if (dd < best) {
                    best = dd;
                    bc = c;
                }
            }
            codes[(size_t)i * m_pq + m] = (uint8_t)bc;
        }
    }
}

void fvo_ivf_lists(const uint32_t* assign, uint32_t n, uint32_t nlist, uint32_t* offsets, uint32_t* vec_ids) {
    memset(offsets, 0, sizeof(uint32_t) * (nlist + 1));
    for (uint32_t i = 0; i < n; ++i) offsets[assign[i] + 1]++;
    for (uint32_t c = 0; c < nlist; ++c) offsets[c + 1] += offsets[c];
    uint32_t* fill = (uint32_t*)malloc(sizeof(uint32_t) * (nlist ? nlist : 1));
    memcpy(fill, offsets, sizeof(uint32_t) * nlist);
    for (uint32_t i = 0; i < n; ++i) vec_ids[fill[assign[i]]++] = i;
    free(fill);
}

void fvo_residuals(const float* x, uint32_t n, uint32_t dim, const float* centroids, const uint32_t* assign,
                   float* out) {
    for (uint32_t i = 0; i < n; ++i)
        for (uint32_t d = 0; d < dim; ++d)
            out[(size_t)i * dim + d] = x[(size_t)i * dim + d] - centroids[(size_t)assign[i] * dim + d];
}

/* ------------------------------------------------------------ IVF search */
static void coarse_topn(const float* q, const float* cent, uint32_t nlist, uint32_t dim, uint32_t nprobe,
                        uint32_t* lists, float* dists) {
    uint64_t* buf = (uint64_t*)malloc(sizeof(uint64_t) * nprobe);
    Heap hp = {buf, nprobe, 0};
    for (uint32_t c = 0; c < nlist; ++c) {
        const float* ce = cent + (size_t)c * dim;
        float s = 0.0f;
        for (uint32_t d = 0; d < dim; ++d) {
            float t = q[d] - ce[d];
            s = fmaf(t, t, s);
        }
        heap_push(&hp, key_of(s, c));
    }
    heap_sorted(&hp);
    for (uint32_t p = 0; p < nprobe; ++p) {
        lists[p] = p < hp.size ? (uint32_t)hp.h[p] : SENT_ID;
        if (dists) dists[p] = p < hp.size ? key_dist(hp.h[p]) : SENT_DIST;
    }
    free(buf);
}

void fvo_coarse_probe(const float* centroids, uint32_t nlist, uint32_t dim, const float* queries, uint32_t nq,
                      uint32_t nprobe, uint32_t* out_lists, float* out_dist, int threads) {
    set_threads(threads);
#pragma omp parallel for schedule(dynamic, 1)
    for (int64_t qi = 0; qi < (int64_t)nq; ++qi)
        coarse_topn(queries + (size_t)qi * dim, centroids, nlist, dim, nprobe, out_lists + (size_t)qi * nprobe,
                    out_dist ? out_dist + (size_t)qi * nprobe : NULL);
}

typedef struct {
    uint32_t top_k, nprobe, shortlist;
    int do_rerank;
} IvfClamp;

static int ivf_clamp(uint32_t nq, uint32_t top_k, uint32_t nprobe, uint32_t rerank_k, uint32_t nlist,
                     const float* vectors, IvfClamp* c) {
    if (nq == 0 || top_k == 0 || nlist == 0) return 0;
    c->top_k = top_k > 256u ? 256u : top_k;
    c->nprobe = nprobe == 0 ? 1u : nprobe;
    if (c->nprobe > nlist) c->nprobe = nlist;
    uint32_t s = rerank_k == 0 ? c->top_k : rerank_k;
    if (s < c->top_k) s = c->top_k;
    if (s > 10240u) s = 10240u;
    c->shortlist = s;
    c->do_rerank = rerank_k != 1u && vectors != NULL;
    return 1;
}

static void ivf_finish(Heap* hp, const float* q, const float* vectors, uint32_t num_vectors, uint32_t dim,
                       int metric, const IvfClamp* c, FvoResult* out) {
    heap_sorted(hp);
    if (c->do_rerank) {
        for (uint32_t i = 0; i < hp->size; ++i) {
            uint32_t id = (uint32_t)hp->h[i];
            if (id >= num_vectors) continue;
            float ex = fvo_warp_distance(q, vectors + (size_t)id * dim, dim, metric);
            hp->h[i] = key_of(ex, id);
        }
        /* rerank results with distance >= 1e30 (or NaN) still occupy a slot in
         * the reference; they sort last with these keys as well */
        heap_sorted(hp);
    }
    for (uint32_t r = 0; r < c->top_k; ++r) {
        if (r < hp->size) {
            out[r].id = (uint32_t)hp->h[r];
            out[r].distance = key_dist(hp->h[r]);
        } else {
            out[r].id = SENT_ID;
            out[r].distance = SENT_DIST;
        }
    }
}

uint32_t fvo_ivf_pq_search(const float* centroids, const float* codebooks, const uint8_t* codes,
                           const uint32_t* offsets, const uint32_t* vec_ids, const float* vectors,
                           uint32_t num_vectors, uint32_t dim, uint32_t nlist, uint32_t m_pq, uint32_t sub_dim,
                           const float* queries, uint32_t nq, uint32_t top_k, uint32_t nprobe, uint32_t rerank_k,
                           int metric, const uint32_t* mask, FvoResult* out, int threads) {
    IvfClamp c;
    if (m_pq == 0 || !ivf_clamp(nq, top_k, nprobe, rerank_k, nlist, vectors, &c)) return 0;
    set_threads(threads);
#pragma omp parallel for schedule(dynamic, 1)
    for (int64_t qi = 0; qi < (int64_t)nq; ++qi) {
        const float* q = queries + (size_t)qi * dim;
        uint32_t* lists = (uint32_t*)malloc(sizeof(uint32_t) * c.nprobe);
        coarse_topn(q, centroids, nlist, dim, c.nprobe, lists, NULL);
        float* lut = (float*)malloc(sizeof(float) * (size_t)m_pq * 256);
        uint64_t* buf = (uint64_t*)malloc(sizeof(uint64_t) * c.shortlist);
        Heap hp = {buf, c.shortlist, 0};
        for (uint32_t p = 0; p < c.nprobe; ++p) {
            uint32_t cl = lists[p];
            if (cl >= nlist) continue;
            const float* ce = centroids + (size_t)cl * dim;
            for (uint32_t m = 0; m < m_pq; ++m)
                for (uint32_t cw = 0; cw < 256; ++cw) {
                    const float* cb = codebooks + ((size_t)m * 256 + cw) * sub_dim;
                    float s = 0.0f;
                    for (uint32_t sd = 0; sd < sub_dim; ++sd) {
                        float t = (q[m * sub_dim + sd] - ce[m * sub_dim + sd]) - cb[sd];
                        s = fmaf(t, t, s);
                    }
                    lut[m * 256 + cw] = s;
                }
            for (uint32_t i = offsets[cl]; i < offsets[cl + 1]; ++i) {
                uint32_t vid = vec_ids[i];
                if (!mask_ok(mask, vid)) continue;
                const uint8_t* cd = codes + (size_t)vid * m_pq;
                float adc = 0.0f;
                for (uint32_t m = 0; m < m_pq; ++m) adc = adc + lut[m * 256 + cd[m]];
                heap_push(&hp, key_of(adc, vid));
            }
        }
        ivf_finish(&hp, q, vectors, num_vectors, dim, metric, &c, out + (size_t)qi * c.top_k);
        free(lists);
        free(lut);
        free(buf);
    }
    return c.top_k;
}

uint32_t fvo_ivf_sq_search(const float* centroids, const float* mins, const float* scales, const uint8_t* codes,
                           const uint32_t* offsets, const uint32_t* vec_ids, const float* vectors,
                           uint32_t num_vectors, uint32_t dim, uint32_t nlist, const float* queries, uint32_t nq,
                           uint32_t top_k, uint32_t nprobe, uint32_t rerank_k, int metric, const uint32_t* mask,
                           FvoResult* out, int threads) {
    IvfClamp c;
    if (dim == 0 || !ivf_clamp(nq, top_k, nprobe, rerank_k, nlist, vectors, &c)) return 0;
    set_threads(threads);
#pragma omp parallel for schedule(dynamic, 1)
    for (int64_t qi = 0; qi < (int64_t)nq; ++qi) {
        const float* q = queries + (size_t)qi * dim;
        uint32_t* lists = (uint32_t*)malloc(sizeof(uint32_t) * c.nprobe);
        coarse_topn(q, centroids, nlist, dim, c.nprobe, lists, NULL);
        float* qres = (float*)malloc(sizeof(float) * dim);
        uint64_t* buf = (uint64_t*)malloc(sizeof(uint64_t) * c.shortlist);
        Heap hp = {buf, c.shortlist, 0};
        for (uint32_t p = 0; p < c.nprobe; ++p) {
            uint32_t cl = lists[p];
            if (cl >= nlist) continue;
            for (uint32_t d = 0; d < dim; ++d) qres[d] = q[d] - centroids[(size_t)cl * dim + d];
            for (uint32_t i = offsets[cl]; i < offsets[cl + 1]; ++i) {
                uint32_t vid = vec_ids[i];
                if (!mask_ok(mask, vid)) continue;
                const uint8_t* cd = codes + (size_t)vid * dim;
                float s = 0.0f;
                for (uint32_t d = 0; d < dim; ++d) {
                    float rec = fmaf((float)cd[d], scales[d], mins[d]);
                    float t = qres[d] - rec;
                    s = fmaf(t, t, s);
                }
                heap_push(&hp, key_of(s, vid));
            }
        }
        ivf_finish(&hp, q, vectors, num_vectors, dim, metric, &c, out + (size_t)qi * c.top_k);
        free(lists);
        free(qres);
        free(buf);
    }
    return c.top_k;
}

double fvo_recall(const uint32_t* approx, uint32_t astride, const uint32_t* truth, uint32_t tstride, uint32_t nq,
                  uint32_t k) {
    if (nq == 0 || k == 0) return 0.0;
    double total = 0.0;
    for (uint32_t q = 0; q < nq; ++q) {
        uint32_t hit = 0, valid = 0;
        for (uint32_t i = 0; i < k; ++i) {
            uint32_t t = truth[(size_t)q * tstride + i];
            if (t == SENT_ID) continue;
            ++valid;
            for (uint32_t j = 0; j < k; ++j)
                if (approx[(size_t)q * astride + j] == t) {
                    ++hit;
                    break;
                }
        }
        total += valid ? (double)hit / (double)valid : 1.0;
    }
    return total / nq;
}

/* ---------------------------------------------------------------- RaBitQ */
uint32_t fvo_rabitq_padded_dim(uint32_t dim) {
    uint32_t p = 32;
    while (p < dim) p <<= 1;
    return p;
}

void fvo_rabitq_rot_signs(uint32_t padded_dim, uint64_t seed, float* out) {
    /* splitmix64 stream started at seed ^ golden-ratio increment; the low bit
     * of each output picks the sign (quant.rs:100-116) */
    const uint64_t inc = 0x9e3779b97f4a7c15ull;
    uint64_t s = seed ^ inc;
    for (uint32_t i = 0; i < 3u * padded_dim; ++i) {
        s += inc;
        uint64_t z = s;
        z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
        z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
        z ^= z >> 31;
        out[i] = (z & 1u) ? -1.0f : 1.0f;
    }
}

float fvo_rabitq_inv_sqrt(uint32_t padded_dim) { return 1.0f / sqrtf((float)padded_dim); }

void fvo_rabitq_rotate(const float* v, uint32_t len, const float* signs, uint32_t padded_dim, float* out) {
    /* three rounds of sign flip, unnormalised Walsh-Hadamard butterflies
     * (half-length 1, 2, 4, ...) and a 1/sqrt(P) scale (quant.rs:119-154) */
    const uint32_t P = padded_dim;
    const float scale = fvo_rabitq_inv_sqrt(P);
    for (uint32_t d = 0; d < P; ++d) out[d] = d < len ? v[d] : 0.0f;
    for (uint32_t st = 0; st < 3; ++st) {
        const float* sg = signs + (size_t)st * P;
        for (uint32_t d = 0; d < P; ++d) out[d] = out[d] * sg[d];
        for (uint32_t h = 1; h < P; h <<= 1)
            for (uint32_t blk = 0; blk < P; blk += 2 * h)
                for (uint32_t o = 0; o < h; ++o) {
                    float x = out[blk + o], y = out[blk + o + h];
                    out[blk + o] = x + y;
                    out[blk + o + h] = x - y;
                }
        for (uint32_t d = 0; d < P; ++d) out[d] = out[d] * scale;
    }
}

void fvo_rabitq_encode(const float* x, uint32_t n, uint32_t dim, const float* centroids, uint32_t nlist,
                       const uint32_t* assign, const float* signs, uint32_t padded_dim, float* rot_centroids,
                       uint32_t* bits, float* meta, int threads) {
    const uint32_t P = padded_dim, W = P / 32;
    for (uint32_t c = 0; c < nlist; ++c)
        fvo_rabitq_rotate(centroids + (size_t)c * dim, dim, signs, P, rot_centroids + (size_t)c * P);
    set_threads(threads);
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < (int64_t)n; ++i) {
        const float* v = x + (size_t)i * dim;
        const float* ce = centroids + (size_t)assign[i] * dim;
        float* r = (float*)malloc(sizeof(float) * dim);
        float* rot = (float*)malloc(sizeof(float) * P);
        float res_sq = 0.0f, vec_sq = 0.0f;
        for (uint32_t d = 0; d < dim; ++d) {
            r[d] = v[d] - ce[d];
            res_sq = res_sq + r[d] * r[d];
            vec_sq = vec_sq + v[d] * v[d];
        }
        fvo_rabitq_rotate(r, dim, signs, P, rot);
        uint32_t* b = bits + (size_t)i * W;
        memset(b, 0, sizeof(uint32_t) * W);
        float abs_sum = 0.0f;
        uint32_t pop = 0;
        for (uint32_t d = 0; d < P; ++d) {
            if (rot[d] >= 0.0f) {
                b[d >> 5] |= 1u << (d & 31u);
                ++pop;
            }
            abs_sum = abs_sum + fabsf(rot[d]);
        }
        const float res_norm = sqrtf(res_sq);
        float* m = meta + (size_t)i * 4;
        m[0] = res_sq;
        m[1] = (res_norm > 1e-12f && abs_sum > 1e-12f) ? (res_norm * res_norm) / abs_sum : 0.0f;
        m[2] = (float)pop;
        m[3] = vec_sq;
        free(r);
        free(rot);
    }
}

/* ||q||^2 in the order of a 256-thread block: thread t accumulates
 * fmaf(q[d], q[d], .) over d = t, t + 256, ...; the 256 partials are then
 * folded pairwise, partial[t] += partial[t + s] for s = 128, 64, ..., 1
 * (ivf_quant_lookup.cu:686-697). */
static float block256_norm_sq(const float* q, uint32_t dim) {
    float part[256];
    for (uint32_t t = 0; t < 256; ++t) {
        float s = 0.0f;
        for (uint32_t d = t; d < dim; d += 256) s = fmaf(q[d], q[d], s);
        part[t] = s;
    }
    for (uint32_t s = 128; s > 0; s >>= 1)
        for (uint32_t t = 0; t < s; ++t) part[t] = part[t] + part[t + s];
    return part[0];
}

float fvo_rabitq_estimate(const uint32_t* b, const float* m, const uint32_t* planes, uint32_t W, uint32_t P,
                          float q_min, float delta, float sum_u, float q_c, float q_norm_sq, int metric) {
    uint32_t acc[4] = {0, 0, 0, 0};
    for (uint32_t w = 0; w < W; ++w)
        for (uint32_t j = 0; j < 4; ++j) acc[j] += (uint32_t)__builtin_popcount(b[w] & planes[j * W + w]);
    const float s_bu = (float)(acc[0] + 2u * acc[1] + 4u * acc[2] + 8u * acc[3]);
    const float A = 2.0f * m[2] - (float)P;
    const float B = 2.0f * s_bu - sum_u;
    /* the estimator of ivf_quant_lookup.cu:467-481 with its roundings fixed:
     * q_min * A rounded, delta * B fused into it, times rescale rounded */
    const float t = fmaf(delta, B, q_min * A);
    const float inner = m[1] * t;
    const float est_l2 = (q_c + m[0]) - 2.0f * inner;
    if (metric == FVO_IP) return -0.5f * ((q_norm_sq + m[3]) - est_l2);
    if (metric == FVO_COSINE) return 0.5f * est_l2;
    return est_l2;
}

/* The 4-bit query code of one probed list (ivf_quant_lookup.cu:389-460):
 * diff = rot_q - rot_centroid over all P coordinates, u = clamp(rint((diff -
 * min) * 15 / range), 0, 15) (0 everywhere when range <= 1e-12), bit-planes
 * planes[j][w] bit l = bit j of u[32 w + l]. Returns sum u. */
static uint32_t rabitq_query_code(const float* rot_q, const float* rot_c, uint32_t P, uint32_t* planes,
                                  float* q_min_out, float* delta_out) {
    const uint32_t W = P / 32;
    float lo = 1e30f, hi = -1e30f;
    for (uint32_t d = 0; d < P; ++d) {
        float v = rot_q[d] - rot_c[d];
        if (v < lo) lo = v;
        if (v > hi) hi = v;
    }
    const float range = hi - lo;
    const float delta = range > 1e-12f ? range / 15.0f : 0.0f;
    const float inv_delta = range > 1e-12f ? 15.0f / range : 0.0f;
    memset(planes, 0, sizeof(uint32_t) * 4 * W);
    uint32_t sum_u = 0;
    for (uint32_t d = 0; d < P; ++d) {
        uint32_t u = 0;
        if (delta > 0.0f) {
            float v = rot_q[d] - rot_c[d];
            long qi = lrintf((v - lo) * inv_delta);
            u = qi < 0 ? 0u : qi > 15 ? 15u : (uint32_t)qi;
        }
        sum_u += u;
        for (uint32_t j = 0; j < 4; ++j)
            if (u & (1u << j)) planes[j * W + (d >> 5)] |= 1u << (d & 31u);
    }
    *q_min_out = lo;
    *delta_out = delta;
    return sum_u;
}

uint32_t fvo_ivf_rabitq_search(const float* centroids, const float* rot_centroids, const uint32_t* bits,
                               const float* meta, const float* signs, const uint32_t* offsets,
                               const uint32_t* vec_ids, const float* vectors, uint32_t num_vectors, uint32_t dim,
                               uint32_t padded_dim, uint32_t nlist, const float* queries, uint32_t nq,
                               uint32_t top_k, uint32_t nprobe, uint32_t rerank_k, int metric, const uint32_t* mask,
                               FvoResult* out, int threads) {
    IvfClamp c;
    const uint32_t P = padded_dim, W = P / 32;
    if (dim == 0 || P < 32 || (P & (P - 1)) || P < dim) return 0;
    if (!ivf_clamp(nq, top_k, nprobe, rerank_k, nlist, vectors, &c)) return 0;
    set_threads(threads);
#pragma omp parallel for schedule(dynamic, 1)
    for (int64_t qi = 0; qi < (int64_t)nq; ++qi) {
        const float* q = queries + (size_t)qi * dim;
        uint32_t* lists = (uint32_t*)malloc(sizeof(uint32_t) * c.nprobe);
        float* cdist = (float*)malloc(sizeof(float) * c.nprobe);
        coarse_topn(q, centroids, nlist, dim, c.nprobe, lists, cdist);
        const float qn = block256_norm_sq(q, dim);
        float* rot_q = (float*)malloc(sizeof(float) * P);
        uint32_t* planes = (uint32_t*)malloc(sizeof(uint32_t) * 4 * W);
        fvo_rabitq_rotate(q, dim, signs, P, rot_q);
        uint64_t* buf = (uint64_t*)malloc(sizeof(uint64_t) * c.shortlist);
        Heap hp = {buf, c.shortlist, 0};
        for (uint32_t p = 0; p < c.nprobe; ++p) {
            uint32_t cl = lists[p];
            if (cl >= nlist) continue;
            float q_min, delta;
            const uint32_t sum_u = rabitq_query_code(rot_q, rot_centroids + (size_t)cl * P, P, planes, &q_min, &delta);
            for (uint32_t i = offsets[cl]; i < offsets[cl + 1]; ++i) {
                uint32_t vid = vec_ids[i];
                if (!mask_ok(mask, vid)) continue;
                float est = fvo_rabitq_estimate(bits + (size_t)vid * W, meta + (size_t)vid * 4, planes, W, P, q_min,
                                                delta, (float)sum_u, cdist[p], qn, metric);
                if (est < SENT_DIST) heap_push(&hp, key_of(est, vid));
            }
        }
        ivf_finish(&hp, q, vectors, num_vectors, dim, metric, &c, out + (size_t)qi * c.top_k);
        free(lists);
        free(cdist);
        free(rot_q);
        free(planes);
        free(buf);
    }
    return c.top_k;
}
