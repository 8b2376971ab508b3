/*
 * pgeof_oracle.c -- CPU restatement of pgeof's neighbour-search and local-PCA
 * feature path. TEST INFRASTRUCTURE ONLY: the parity checker and the timed CPU
 * baseline. Nothing in the shipped library links or calls this file.
 *
 * Reference: drprojects/point_geometric_features (pgeof 0.3.3)
 *   include/pca.hpp:72-98    pca_from_pointcloud   (mean, centred C^T C / k,
 *                            SelfAdjointEigenSolver, clamp >= 0, v2.z >= 0 flip;
 *                            NO sort -> eigenvalues in Eigen's ascending order)
 *   include/pca.hpp:113-129  pca_from_neighborhood (CSR gather)
 *   include/pca.hpp:140-150  compute_eigentropy
 *   include/pca.hpp:160-200  compute_features      (11 features)
 *   include/pca.hpp:212-295  compute_selected_features
 *   include/pgeof.hpp:75-117, 123-211, 243-310, 325-375  drivers
 *   include/nn_search.hpp:31-67, 85-132  kNN / radius search (nanoflann)
 *
 * Parity status. The reference cannot be built here (its Eigen, nanoflann and
 * Taskflow submodules are empty), so no reference output exists to compare
 * with. Neighbour search is pinned by the reference's own tests
 * (tests/test_pgeof.py:8-27 compare against scipy's KDTree, which the oracle
 * tests repeat). Feature VALUES are "parity unpinned" against the reference
 * binary: they are pinned by hand-derived known answers of the formulas above
 * and by an independent FP64 numpy restatement.
 *
 * Arithmetic follows the reference literally and is compiled with
 * -ffp-contract=off (no FMA), as the reference's x86-64 Release build runs:
 *   - mean:       sequential float sum over the neighbours, then / k
 *                 (Eigen colwise().mean() = sum / rows);
 *   - covariance: centred float products summed sequentially, then / k;
 *   - eigen:      the float covariance is diagonalised EXACTLY (cyclic Jacobi
 *                 in double to convergence) and rounded to float, then sorted
 *                 ascending with Eigen's selection rule (first minimum wins);
 *   - features:   float formulas in the reference's operation order.
 * Third-party arithmetic restated from published behaviour:
 *   - nanoflann metric_L2_Simple: d = sum over x,y,z of (q - p)^2 in float,
 *     accumulated in that order; a point enters a result set only if
 *     d < worstDist (strict). KNNResultSet/RKNNResultSet keep ascending order.
 *     RKNNResultSet::init writes radius^2 into the LAST distance slot, so a
 *     radius row with fewer than max_knn hits reports radius^2 there.
 *   - Ties at equal distance: nanoflann keeps traversal order; this oracle
 *     (and the GPU library) orders by (distance, index).
 */
#include <math.h>
#include <pthread.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#include <unistd.h>

#define ORACLE_EIG_ASCENDING 0
#define ORACLE_EIG_DESCENDING 1

/* ------------------------------------------------------------------------- */
/* parallel for                                                              */
/* ------------------------------------------------------------------------- */
typedef void (*range_fn)(void* ctx, size_t lo, size_t hi);
typedef struct {
    range_fn fn;
    void* ctx;
    size_t n, chunk;
    size_t next;
    pthread_mutex_t mu;
} pfor_t;

static void* pfor_worker(void* arg) {
    pfor_t* p = (pfor_t*)arg;
    for (;;) {
        pthread_mutex_lock(&p->mu);
        size_t lo = p->next;
        p->next = lo + p->chunk;
        pthread_mutex_unlock(&p->mu);
        if (lo >= p->n) break;
        size_t hi = lo + p->chunk < p->n ? lo + p->chunk : p->n;
        p->fn(p->ctx, lo, hi);
    }
    return NULL;
}

static int oracle_threads(int requested) {
    if (requested > 0) return requested;
    long c = sysconf(_SC_NPROCESSORS_ONLN);
    return c > 0 ? (int)c : 1;
}

static void parallel_for(size_t n, int nthreads, range_fn fn, void* ctx) {
    nthreads = oracle_threads(nthreads);
    if (n == 0) return;
    pfor_t p;
    p.fn = fn;
    p.ctx = ctx;
    p.n = n;
    p.chunk = n / ((size_t)nthreads * 16) + 1;
    p.next = 0;
    pthread_mutex_init(&p.mu, NULL);
    if (nthreads == 1) {
        pfor_worker(&p);
    } else {
        pthread_t* th = (pthread_t*)malloc(sizeof(pthread_t) * (size_t)nthreads);
        int started = 0;
        for (int t = 0; t < nthreads; ++t)
            if (pthread_create(&th[t], NULL, pfor_worker, &p) == 0) ++started;
        if (started == 0) pfor_worker(&p);
        for (int t = 0; t < started; ++t) pthread_join(th[t], NULL);
        free(th);
    }
    pthread_mutex_destroy(&p.mu);
}

/* ------------------------------------------------------------------------- */
/* exact symmetric 3x3 eigen-decomposition (cyclic Jacobi, double)            */
/* ------------------------------------------------------------------------- */
/* Diagonalises the symmetric matrix a (only a[i][j], i<=j are meaningful on
 * entry; both triangles are kept in sync). On return a is diagonal (the
 * eigenvalues) and the columns of v are the eigenvectors. Classical cyclic
 * Jacobi (Golub & Van Loan, "Matrix Computations", sec. 8.5), rotating every
 * non-zero off-diagonal entry until all vanish or are negligible. */
static void jacobi3(double a[3][3], double v[3][3]) {
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) v[i][j] = (i == j) ? 1.0 : 0.0;
    static const int P[3] = {0, 0, 1}, Q[3] = {1, 2, 2};
    for (int sweep = 0; sweep < 64; ++sweep) {
        if (a[0][1] == 0.0 && a[0][2] == 0.0 && a[1][2] == 0.0) break;
        for (int r = 0; r < 3; ++r) {
            const int p = P[r], q = Q[r];
            const double apq = a[p][q];
            if (apq == 0.0) continue;
            const double g = 100.0 * fabs(apq);
            if (sweep > 4 && fabs(a[p][p]) + g == fabs(a[p][p]) && fabs(a[q][q]) + g == fabs(a[q][q])) {
                a[p][q] = a[q][p] = 0.0;
                continue;
            }
            const double h = a[q][q] - a[p][p];
            double t;
            if (fabs(h) + g == fabs(h)) {
                t = apq / h;
            } else {
                const double theta = 0.5 * h / apq;
                t = 1.0 / (fabs(theta) + sqrt(1.0 + theta * theta));
                if (theta < 0.0) t = -t;
            }
            const double c = 1.0 / sqrt(1.0 + t * t);
            const double s = t * c;
            const double tau = s / (1.0 + c);
            a[p][p] -= t * apq;
            a[q][q] += t * apq;
            a[p][q] = a[q][p] = 0.0;
            const int o = 3 - p - q; /* the remaining index */
            const double aop = a[o][p], aoq = a[o][q];
            a[o][p] = a[p][o] = aop - s * (aoq + tau * aop);
            a[o][q] = a[q][o] = aoq + s * (aop - tau * aoq);
            for (int k = 0; k < 3; ++k) {
                const double vkp = v[k][p], vkq = v[k][q];
                v[k][p] = vkp - s * (vkq + tau * vkp);
                v[k][q] = vkq + s * (vkp - tau * vkq);
            }
        }
    }
}

/* Sort eigenpairs ascending the way Eigen's SelfAdjointEigenSolver does:
 * for each position, take the FIRST minimum of the remaining values. */
static void sort_ascending(double w[3], double v[3][3]) {
    for (int i = 0; i < 2; ++i) {
        int k = i;
        for (int j = i + 1; j < 3; ++j)
            if (w[j] < w[k]) k = j;
        if (k != i) {
            double t = w[i];
            w[i] = w[k];
            w[k] = t;
            for (int r = 0; r < 3; ++r) {
                t = v[r][i];
                v[r][i] = v[r][k];
                v[r][k] = t;
            }
        }
    }
}

/* ------------------------------------------------------------------------- */
/* PCA + features, generated for float and double                            */
/* ------------------------------------------------------------------------- */
#define REAL float
#define SFX(name) name##_f32
#define RSQRT sqrtf
#define RPOW powf
#define RLOG logf
#define RABS fabsf
#include "pca_body.h"
#undef REAL
#undef SFX
#undef RSQRT
#undef RPOW
#undef RLOG
#undef RABS

#define REAL double
#define SFX(name) name##_f64
#define RSQRT sqrt
#define RPOW pow
#define RLOG log
#define RABS fabs
#include "pca_body.h"
#undef REAL
#undef SFX
#undef RSQRT
#undef RPOW
#undef RLOG
#undef RABS

/* ------------------------------------------------------------------------- */
/* CSR feature drivers (include/pgeof.hpp)                                   */
/* ------------------------------------------------------------------------- */
typedef struct {
    const float* xyz;
    const uint32_t* nn;
    const uint32_t* ptr;
    size_t k_min;
    int order;
    float* out;
    /* multiscale */
    const uint32_t* scales;
    size_t n_scales;
    /* optimal */
    uint32_t k_step, k_min_search;
    /* scratch per thread is allocated on the fly */
} csr_ctx;

static float* gather_f32(const float* xyz, const uint32_t* nn, size_t base, size_t k) {
    float* pts = (float*)malloc(sizeof(float) * 3 * (k ? k : 1));
    for (size_t j = 0; j < k; ++j) {
        const size_t id = nn[base + j];
        pts[3 * j + 0] = xyz[3 * id + 0];
        pts[3 * j + 1] = xyz[3 * id + 1];
        pts[3 * j + 2] = xyz[3 * id + 2];
    }
    return pts;
}

/* include/pgeof.hpp:93-109 */
static void features_range(void* vctx, size_t lo, size_t hi) {
    csr_ctx* c = (csr_ctx*)vctx;
    for (size_t i = lo; i < hi; ++i) {
        const size_t k_nn = (size_t)(uint32_t)(c->ptr[i + 1] - c->ptr[i]);
        if (k_nn >= c->k_min) {
            float* pts = gather_f32(c->xyz, c->nn, c->ptr[i], k_nn);
            pca_f32 p;
            pca_from_pointcloud_f32(pts, k_nn, c->order, &p);
            compute_features_f32(&p, &c->out[i * 11]);
            free(pts);
        }
    }
}

/* include/pgeof.hpp:183-199 */
static void multiscale_range(void* vctx, size_t lo, size_t hi) {
    csr_ctx* c = (csr_ctx*)vctx;
    for (size_t i = lo; i < hi; ++i) {
        const size_t k_nn = (size_t)(uint32_t)(c->ptr[i + 1] - c->ptr[i]);
        for (size_t s = 0; s < c->n_scales; ++s) {
            const size_t ks = c->scales[s];
            if (k_nn < ks) break;
            float* pts = gather_f32(c->xyz, c->nn, c->ptr[i], ks);
            pca_f32 p;
            pca_from_pointcloud_f32(pts, ks, c->order, &p);
            compute_features_f32(&p, &c->out[(i * c->n_scales + s) * 11]);
            free(pts);
        }
    }
}

/* include/pgeof.hpp:264-299 */
static void optimal_range(void* vctx, size_t lo, size_t hi) {
    csr_ctx* c = (csr_ctx*)vctx;
    const size_t kmin = c->k_min, kms = c->k_min_search;
    for (size_t i = lo; i < hi; ++i) {
        const size_t k_nn = (size_t)(uint32_t)(c->ptr[i + 1] - c->ptr[i]);
        if (!(k_nn >= kmin && k_nn >= kms)) continue;
        size_t k0 = kmin > kms ? kmin : kms;
        if (k0 > k_nn) k0 = k_nn;
        float* pts = gather_f32(c->xyz, c->nn, c->ptr[i], k_nn);
        pca_f32 best;
        float best_e = 1.0f;
        size_t k_opt = k_nn;
        for (size_t k = k0; k <= k_nn; ++k) {
            if (k > k0 && (k % c->k_step) != 0 && k != k_nn) continue;
            pca_f32 p;
            pca_from_pointcloud_f32(pts, k, c->order, &p);
            const float e = compute_eigentropy_f32(&p);
            if (k == k0 || e < best_e) {
                best_e = e;
                k_opt = k;
                best = p;
            }
        }
        compute_features_f32(&best, &c->out[i * 12]);
        c->out[i * 12 + 11] = (float)k_opt;
        free(pts);
    }
}

int oracle_compute_features(const float* xyz, const uint32_t* nn, const uint32_t* ptr, size_t n,
                            size_t k_min, int order, int nthreads, float* out) {
    if (k_min < 1) return 1;
    memset(out, 0, sizeof(float) * n * 11);
    csr_ctx c = {xyz, nn, ptr, k_min, order, out, NULL, 0, 0, 0};
    parallel_for(n, nthreads, features_range, &c);
    return 0;
}

int oracle_compute_features_multiscale(const float* xyz, const uint32_t* nn, const uint32_t* ptr, size_t n,
                                       const uint32_t* scales, size_t n_scales, int order, int nthreads,
                                       float* out) {
    uint32_t prev = 1;
    for (size_t s = 0; s < n_scales; ++s) {
        if (scales[s] < prev) return 1;
        prev = scales[s];
    }
    memset(out, 0, sizeof(float) * n * n_scales * 11);
    csr_ctx c = {xyz, nn, ptr, 1, order, out, scales, n_scales, 0, 0};
    parallel_for(n, nthreads, multiscale_range, &c);
    return 0;
}

int oracle_compute_features_optimal(const float* xyz, const uint32_t* nn, const uint32_t* ptr, size_t n,
                                    uint32_t k_min, uint32_t k_step, uint32_t k_min_search, int order,
                                    int nthreads, float* out) {
    if (k_min < 1 && k_min_search < 1) return 1;
    if (k_step < 1) return 1;
    memset(out, 0, sizeof(float) * n * 12);
    csr_ctx c = {xyz, nn, ptr, k_min, order, out, NULL, 0, k_step, k_min_search};
    parallel_for(n, nthreads, optimal_range, &c);
    return 0;
}

/* ------------------------------------------------------------------------- */
/* the same three drivers with real_t = double (the templates of              */
/* include/pgeof.hpp instantiated for double; pgeof binds them for float only) */
/* ------------------------------------------------------------------------- */
typedef struct {
    const double* xyz;
    const uint32_t* nn;
    const uint32_t* ptr;
    size_t k_min;
    int order;
    double* out;
    const uint32_t* scales;
    size_t n_scales;
    uint32_t k_step, k_min_search;
    int kind;
} csr64_ctx;

static double* gather_f64(const double* xyz, const uint32_t* nn, size_t base, size_t k) {
    double* pts = (double*)malloc(sizeof(double) * 3 * (k ? k : 1));
    for (size_t j = 0; j < k; ++j) {
        const size_t id = nn[base + j];
        pts[3 * j + 0] = xyz[3 * id + 0];
        pts[3 * j + 1] = xyz[3 * id + 1];
        pts[3 * j + 2] = xyz[3 * id + 2];
    }
    return pts;
}

/* include/pgeof.hpp:93-109, 183-199, 264-299 for double */
static void range_f64(void* vctx, size_t lo, size_t hi) {
    csr64_ctx* c = (csr64_ctx*)vctx;
    for (size_t i = lo; i < hi; ++i) {
        const size_t k_nn = (size_t)(uint32_t)(c->ptr[i + 1] - c->ptr[i]);
        if (c->kind == 0) {
            if (k_nn < c->k_min) continue;
            double* pts = gather_f64(c->xyz, c->nn, c->ptr[i], k_nn);
            pca_f64 p;
            pca_from_pointcloud_f64(pts, k_nn, c->order, &p);
            compute_features_f64(&p, &c->out[i * 11]);
            free(pts);
        } else if (c->kind == 1) {
            for (size_t s = 0; s < c->n_scales; ++s) {
                const size_t ks = c->scales[s];
                if (k_nn < ks) break;
                double* pts = gather_f64(c->xyz, c->nn, c->ptr[i], ks);
                pca_f64 p;
                pca_from_pointcloud_f64(pts, ks, c->order, &p);
                compute_features_f64(&p, &c->out[(i * c->n_scales + s) * 11]);
                free(pts);
            }
        } else {
            const size_t kmin = c->k_min, kms = c->k_min_search;
            if (!(k_nn >= kmin && k_nn >= kms)) continue;
            size_t k0 = kmin > kms ? kmin : kms;
            if (k0 > k_nn) k0 = k_nn;
            double* pts = gather_f64(c->xyz, c->nn, c->ptr[i], k_nn);
            pca_f64 best;
            double best_e = 1.0;
            size_t k_opt = k_nn;
            for (size_t k = k0; k <= k_nn; ++k) {
                if (k > k0 && (k % c->k_step) != 0 && k != k_nn) continue;
                pca_f64 p;
                pca_from_pointcloud_f64(pts, k, c->order, &p);
                const double e = compute_eigentropy_f64(&p);
                if (k == k0 || e < best_e) {
                    best_e = e;
                    k_opt = k;
                    best = p;
                }
            }
            compute_features_f64(&best, &c->out[i * 12]);
            c->out[i * 12 + 11] = (double)k_opt;
            free(pts);
        }
    }
}

/* kind 0: compute_features (out n x 11), 1: multiscale (n x n_scales x 11),
 * 2: optimal (n x 12). Returns 1 on the reference's argument errors. */
int oracle_compute_features_f64(int kind, const double* xyz, const uint32_t* nn, const uint32_t* ptr, size_t n,
                                size_t k_min, const uint32_t* scales, size_t n_scales, uint32_t k_step,
                                uint32_t k_min_search, int order, int nthreads, double* out) {
    size_t width = 11;
    if (kind == 0 && k_min < 1) return 1;
    if (kind == 1) {
        uint32_t prev = 1;
        for (size_t s = 0; s < n_scales; ++s) {
            if (scales[s] < prev) return 1;
            prev = scales[s];
        }
        width = n_scales * 11;
    }
    if (kind == 2) {
        if (k_min < 1 && k_min_search < 1) return 1;
        if (k_step < 1) return 1;
        width = 12;
    }
    memset(out, 0, sizeof(double) * n * width);
    csr64_ctx c = {xyz, nn, ptr, k_min, order, out, scales, n_scales, k_step, k_min_search, kind};
    parallel_for(n, nthreads, range_f64, &c);
    return 0;
}

/* ------------------------------------------------------------------------- */
/* neighbour search (include/nn_search.hpp with nanoflann semantics)          */
/* ------------------------------------------------------------------------- */
/* metric_L2_Simple: result = 0; result += (a_i - b_i)^2 for i = x, y, z. */
static inline float l2_f32(const float* a, const float* b) {
    const float tx = a[0] - b[0];
    const float ty = a[1] - b[1];
    const float tz = a[2] - b[2];
    float r = tx * tx;
    r = r + ty * ty;
    r = r + tz * tz;
    return r;
}
static inline double l2_f64(const double* a, const double* b) {
    const double tx = a[0] - b[0];
    const double ty = a[1] - b[1];
    const double tz = a[2] - b[2];
    double r = tx * tx;
    r = r + ty * ty;
    r = r + tz * tz;
    return r;
}

/* Insert (d, id) into the sorted prefix [0, *count) of capacity cap, ordered by
 * (distance, index). Returns nothing; drops the element if it does not fit. */
#define DEFINE_INSERT(NAME, DT)                                                          \
    static inline void NAME(DT* ds, int64_t* ids, size_t* count, size_t cap, DT d, int64_t id) { \
        size_t n = *count;                                                               \
        if (n == cap) {                                                                  \
            if (!(d < ds[n - 1] || (d == ds[n - 1] && id < ids[n - 1]))) return;         \
            n = cap - 1;                                                                 \
        }                                                                                \
        size_t pos = n;                                                                  \
        while (pos > 0 && (ds[pos - 1] > d || (ds[pos - 1] == d && ids[pos - 1] > id))) { \
            ds[pos] = ds[pos - 1];                                                       \
            ids[pos] = ids[pos - 1];                                                     \
            --pos;                                                                       \
        }                                                                                \
        ds[pos] = d;                                                                     \
        ids[pos] = id;                                                                   \
        if (*count < cap) ++*count;                                                      \
    }
DEFINE_INSERT(insert_f32, float)
DEFINE_INSERT(insert_f64, double)

typedef struct {
    const float* data;
    size_t n;
    const float* q;
    uint32_t k;
    float r2; /* radius mode when has_radius */
    int has_radius;
    void* idx; /* uint32_t* (knn) or int32_t* (radius) */
    float* d2;
} nn_ctx;

static void nn_range(void* vctx, size_t lo, size_t hi) {
    nn_ctx* c = (nn_ctx*)vctx;
    const size_t cap = c->k;
    float* ds = (float*)malloc(sizeof(float) * (cap ? cap : 1));
    int64_t* ids = (int64_t*)malloc(sizeof(int64_t) * (cap ? cap : 1));
    for (size_t i = lo; i < hi; ++i) {
        size_t count = 0;
        const float* qi = &c->q[3 * i];
        if (cap) {
            for (size_t j = 0; j < c->n; ++j) {
                const float d = l2_f32(qi, &c->data[3 * j]);
                if (c->has_radius && !(d < c->r2)) continue;
                insert_f32(ds, ids, &count, cap, d, (int64_t)j);
            }
        }
        if (c->has_radius) {
            int32_t* out = (int32_t*)c->idx + i * cap;
            for (size_t j = 0; j < cap; ++j) {
                out[j] = j < count ? (int32_t)ids[j] : -1;
                c->d2[i * cap + j] = j < count ? ds[j] : 0.0f;
            }
            if (cap && count < cap) c->d2[i * cap + cap - 1] = c->r2;
        } else {
            uint32_t* out = (uint32_t*)c->idx + i * cap;
            for (size_t j = 0; j < cap; ++j) {
                out[j] = (uint32_t)ids[j];
                c->d2[i * cap + j] = ds[j];
            }
        }
    }
    free(ds);
    free(ids);
}

/* include/nn_search.hpp:31-67 */
int oracle_knn_search(const float* data, size_t n, const float* query, size_t m, uint32_t k, int nthreads,
                      uint32_t* idx, float* d2) {
    if ((size_t)k > n) return 1;
    nn_ctx c = {data, n, query, k, 0.0f, 0, idx, d2};
    parallel_for(m, nthreads, nn_range, &c);
    return 0;
}

/* include/nn_search.hpp:85-132 */
int oracle_radius_search(const float* data, size_t n, const float* query, size_t m, float radius,
                         uint32_t max_knn, int nthreads, int32_t* idx, float* d2) {
    if ((size_t)max_knn > n) return 1;
    nn_ctx c = {data, n, query, max_knn, radius * radius, 1, idx, d2};
    parallel_for(m, nthreads, nn_range, &c);
    return 0;
}

/* ------------------------------------------------------------------------- */
/* fused radius + selected features (include/pgeof.hpp:325-375)              */
/* ------------------------------------------------------------------------- */
typedef struct {
    const void* xyz;
    size_t n;
    double r2d;
    float r2f;
    uint32_t max_knn;
    const int32_t* ids;
    size_t n_ids;
    int order;
    int is_f64;
    void* out;
} sel_ctx;

static void selected_range(void* vctx, size_t lo, size_t hi) {
    sel_ctx* c = (sel_ctx*)vctx;
    const size_t cap = c->max_knn;
    for (size_t i = lo; i < hi; ++i) {
        /* collect every point strictly inside the radius, nearest first */
        size_t count = 0, num_found = 0;
        if (c->is_f64) {
            const double* x = (const double*)c->xyz;
            double* ds = (double*)malloc(sizeof(double) * (cap ? cap : 1));
            int64_t* ids = (int64_t*)malloc(sizeof(int64_t) * (cap ? cap : 1));
            for (size_t j = 0; j < c->n; ++j) {
                const double d = l2_f64(&x[3 * i], &x[3 * j]);
                if (!(d < c->r2d)) continue;
                ++num_found;
                if (cap) insert_f64(ds, ids, &count, cap, d, (int64_t)j);
            }
            if (num_found >= 2) {
                double* pts = (double*)malloc(sizeof(double) * 3 * (count ? count : 1));
                for (size_t j = 0; j < count; ++j)
                    for (int a = 0; a < 3; ++a) pts[3 * j + a] = x[3 * ids[j] + a];
                pca_f64 p;
                pca_from_pointcloud_f64(pts, count, c->order, &p);
                compute_selected_features_f64(&p, c->ids, c->n_ids, (double*)c->out + i * c->n_ids);
                free(pts);
            }
            free(ds);
            free(ids);
        } else {
            const float* x = (const float*)c->xyz;
            float* ds = (float*)malloc(sizeof(float) * (cap ? cap : 1));
            int64_t* ids = (int64_t*)malloc(sizeof(int64_t) * (cap ? cap : 1));
            for (size_t j = 0; j < c->n; ++j) {
                const float d = l2_f32(&x[3 * i], &x[3 * j]);
                if (!(d < c->r2f)) continue;
                ++num_found;
                if (cap) insert_f32(ds, ids, &count, cap, d, (int64_t)j);
            }
            if (num_found >= 2) {
                float* pts = (float*)malloc(sizeof(float) * 3 * (count ? count : 1));
                for (size_t j = 0; j < count; ++j)
                    for (int a = 0; a < 3; ++a) pts[3 * j + a] = x[3 * ids[j] + a];
                pca_f32 p;
                pca_from_pointcloud_f32(pts, count, c->order, &p);
                compute_selected_features_f32(&p, c->ids, c->n_ids, (float*)c->out + i * c->n_ids);
                free(pts);
            }
            free(ds);
            free(ids);
        }
    }
}

int oracle_selected_f32(const float* xyz, size_t n, float radius, uint32_t max_knn, const int32_t* ids,
                        size_t n_ids, int order, int nthreads, float* out) {
    memset(out, 0, sizeof(float) * n * n_ids);
    sel_ctx c = {xyz, n, 0.0, radius * radius, max_knn, ids, n_ids, order, 0, out};
    parallel_for(n, nthreads, selected_range, &c);
    return 0;
}

int oracle_selected_f64(const double* xyz, size_t n, double radius, uint32_t max_knn, const int32_t* ids,
                        size_t n_ids, int order, int nthreads, double* out) {
    memset(out, 0, sizeof(double) * n * n_ids);
    sel_ctx c = {xyz, n, radius * radius, 0.0f, max_knn, ids, n_ids, order, 1, out};
    parallel_for(n, nthreads, selected_range, &c);
    return 0;
}

/* ------------------------------------------------------------------------- */
/* single-neighbourhood entry points for known-answer tests                  */
/* ------------------------------------------------------------------------- */
/* pts: k x 3 float. out: val[3], v0[3], v1[3], v2[3] (12 floats) then the 11
 * features then the eigentropy (24 floats total). */
void oracle_pca_features_f32(const float* pts, size_t k, int order, float* out) {
    pca_f32 p;
    pca_from_pointcloud_f32(pts, k, order, &p);
    for (int a = 0; a < 3; ++a) {
        out[a] = p.val[a];
        out[3 + a] = p.v0[a];
        out[6 + a] = p.v1[a];
        out[9 + a] = p.v2[a];
    }
    for (int f = 0; f < 11; ++f) out[12 + f] = 0.0f;
    compute_features_f32(&p, out + 12);
    out[23] = compute_eigentropy_f32(&p);
}

/* The float covariance exactly as the reference forms it (6 entries:
 * xx, xy, xz, yy, yz, zz) -- used to pin the GPU covariance bit-exactly. */
void oracle_covariance_f32(const float* pts, size_t k, float* cov6) {
    float c[3][3];
    covariance_f32(pts, k, c);
    cov6[0] = c[0][0];
    cov6[1] = c[0][1];
    cov6[2] = c[0][2];
    cov6[3] = c[1][1];
    cov6[4] = c[1][2];
    cov6[5] = c[2][2];
}

int oracle_num_threads(void) { return oracle_threads(0); }
