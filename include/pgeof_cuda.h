/*
 * pgeof_cuda.h -- C ABI of libpgeof_cuda.so, the GB300 (sm_103a) implementation
 * of pgeof's neighbour-search and local-PCA geometric-feature path.
 *
 * Plain pointers, sizes and status codes only. Every entry point replaces one
 * function of pgeof 0.3.3 (drprojects/point_geometric_features); the citation
 * above each declaration names the reference function it stands in for, with
 * the same argument meaning, output layout and error conditions.
 *
 * Two families:
 *   pgeof_*       device pointers (inputs and outputs already in GPU memory),
 *                 enqueued on `stream`, asynchronous. Host-side argument errors
 *                 are returned immediately; errors that only the data reveals
 *                 (an `nn` index >= n_xyz, a decreasing `nn_ptr`) are recorded
 *                 on the device and reported by pgeof_take_device_errors().
 *   pgeof_host_*  host pointers, synchronous: the reference's own contract
 *                 (host arrays in, host arrays out). Copies run inside the call
 *                 and data errors come back as the return code.
 *
 * Conventions shared with the reference:
 *   xyz / data / query : float32 (n, 3) row-major (RefCloud<float>, pca.hpp:18)
 *   nn, nn_ptr         : uint32 CSR; neighbours of point i are
 *                        nn[nn_ptr[i] : nn_ptr[i+1]]; n_points = len(nn_ptr) - 1
 *   features           : float32 row-major, EFeatureID order (pca.hpp:47-63)
 *   eigenvalues        : in Eigen's ascending order, exactly as pca.hpp:79-97
 *                        uses them (val[0] = smallest); see pgeof_set_eig_order.
 *   normal sign        : v2 flipped so that v2.z >= 0 (pca.hpp:96)
 */
#ifndef PGEOF_CUDA_H
#define PGEOF_CUDA_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define PGEOF_ABI_VERSION 1

/* Return codes. INVALID_ARGUMENT and DATA_ERROR are the reference's
 * std::invalid_argument (nanobind maps it to ValueError). */
typedef enum pgeof_status {
    PGEOF_OK = 0,
    PGEOF_ERR_INVALID_ARGUMENT = 1, /* bad size / parameter (reference throws)          */
    PGEOF_ERR_DATA = 2,             /* nn index >= n_xyz, nn_ptr decreasing or > len(nn) */
    PGEOF_ERR_OUT_OF_MEMORY = 3,
    PGEOF_ERR_CUDA = 4,             /* CUDA runtime failure (message has the detail)      */
    PGEOF_ERR_NO_DEVICE = 5,        /* no usable GB300 / CUDA device                       */
    PGEOF_ERR_INTERNAL = 6          /* an internal bound was exceeded                      */
} pgeof_status;

/* EFeatureID, include/pca.hpp:47-63 (same integer values). */
typedef enum pgeof_feature_id {
    PGEOF_LINEARITY = 0,
    PGEOF_PLANARITY = 1,
    PGEOF_SCATTERING = 2,
    PGEOF_VERTICALITY_PGEOF = 3,
    PGEOF_NORMAL_X = 4,
    PGEOF_NORMAL_Y = 5,
    PGEOF_NORMAL_Z = 6,
    PGEOF_LENGTH = 7,
    PGEOF_SURFACE = 8,
    PGEOF_VOLUME = 9,
    PGEOF_CURVATURE = 10,
    PGEOF_K_OPTIMAL = 11,
    PGEOF_VERTICALITY = 12,
    PGEOF_EIGENTROPY = 13
} pgeof_feature_id;

/* A cudaStream_t. NULL is the legacy default stream. */
typedef void* pgeof_stream_t;

/* ---------------------------------------------------------------- library */
int pgeof_abi_version(void);
const char* pgeof_status_string(int status);
/* Detail of the last failure on the calling host thread (never NULL). */
const char* pgeof_last_error_message(void);
/* Number of kernels this library has launched in this process. */
uint64_t pgeof_kernel_launch_count(void);
/* Number of device memory allocations (memory-pool and cudaMalloc) this
 * library has made in this process. */
uint64_t pgeof_device_alloc_count(void);
/* Eigenpair order fed to the feature formulas: 0 = ascending (Eigen's order,
 * what pca.hpp:79-97 does, the default), 1 = descending (val[0] = largest, so
 * v2 is the surface normal). Process-wide. */
int pgeof_set_eig_order(int order);
int pgeof_get_eig_order(void);
/* Kernel timing for measurement harnesses (no reference counterpart). While
 * enabled, every kernel launch is bracketed by CUDA events recorded on the
 * stream it is launched on. pgeof_profile_report() waits for those events,
 * writes one line "<kernel> <launches> <total_ms>\n" per kernel name into buf
 * (NUL-terminated, truncated to buf_len) and clears the record. */
int pgeof_profile_enable(int on);
int pgeof_profile_report(char* buf, size_t buf_len);
/* Synchronises `stream` and returns (then clears) the device-side data-error
 * bits recorded since the last call (bit 0: nn index out of range, bit 1:
 * nn_ptr not monotone or beyond len(nn), bit 2: internal bound exceeded). */
int pgeof_take_device_errors(pgeof_stream_t stream, uint32_t* bits);
/* Pinned host buffers for result arrays (no reference counterpart: the
 * reference returns freshly allocated arrays). Writing a result into freshly
 * mapped pageable memory costs a page fault per page, several times the copy
 * itself; these blocks are page-locked once and cached, so a binding that
 * backs its result arrays with them receives results at DMA speed.
 * pgeof_host_alloc returns a block of at least `bytes` (2 MiB granules) from the
 * cache or a new cudaHostAlloc; pgeof_host_free returns it to the cache, which
 * keeps at most PGEOF_HOST_POOL_BYTES (environment, default 8 GiB; 0 disables
 * caching) and releases blocks beyond that. pgeof_host_pool_trim releases every
 * cached block. Thread-safe. */
int pgeof_host_alloc(size_t bytes, void** ptr);
int pgeof_host_free(void* ptr);
int pgeof_host_pool_trim(void);

/* ------------------------------------------------ device-pointer API (async) */

/* nanoflann_knn_search<float>, include/nn_search.hpp:31-67.
 * For each query row: the `knn` nearest data rows (self included when the query
 * is in the data), ascending squared distance; ties ordered by lower index.
 * indices / sqr_dist: (n_query, knn). Errors: knn > n_data. */
int pgeof_knn_search_f32(const float* data, int64_t n_data, const float* query, int64_t n_query, uint32_t knn,
                         uint32_t* indices, float* sqr_dist, pgeof_stream_t stream);

/* nanoflann_radius_search<float>, include/nn_search.hpp:85-132.
 * Up to max_knn nearest data rows with squared distance < search_radius^2
 * (computed in float), ascending. Missing entries: index -1, distance 0, except
 * that a row with fewer than max_knn hits reports search_radius^2 in its last
 * distance slot (nanoflann's RKNNResultSet::init). Errors: max_knn > n_data. */
int pgeof_radius_search_f32(const float* data, int64_t n_data, const float* query, int64_t n_query,
                            float search_radius, uint32_t max_knn, int32_t* indices, float* sqr_dist,
                            pgeof_stream_t stream);

/* Radius search straight to CSR neighbourhoods (no reference counterpart: pgeof
 * builds this pair on the host from radius_search's padded table, README.md:
 * 157-163). nn_ptr (n_query + 1 entries) and nn (capacity n_query * max_knn)
 * receive, for every query, the indices radius_search would return in its row
 * (nearest first, at most max_knn, the -1 padding dropped); nn_ptr[n_query] is
 * the number of entries written. Requires n_query * max_knn < 2^32. Device
 * pointers, asynchronous on `stream`. */
int pgeof_radius_search_csr_f32(const float* data, int64_t n_data, const float* query, int64_t n_query,
                                float search_radius, uint32_t max_knn, uint32_t* nn, uint32_t* nn_ptr,
                                pgeof_stream_t stream);

/* compute_geometric_features<float, 11>, include/pgeof.hpp:75-117.
 * features: (n_points, 11); rows with fewer than k_min neighbours are 0.
 * Errors: k_min < 1. */
int pgeof_compute_features_f32(const float* xyz, int64_t n_xyz, const uint32_t* nn, int64_t nnz,
                               const uint32_t* nn_ptr, int64_t n_points, uint64_t k_min, float* features,
                               pgeof_stream_t stream);

/* compute_geometric_features_multiscale<float, 11>, include/pgeof.hpp:123-211.
 * k_scales is a HOST array; features: (n_points, n_scales, 11). A point stops
 * at the first scale larger than its neighbour count (later scales are 0).
 * Errors: a scale < 1 or scales not non-decreasing (check_scales, :123-132). */
int pgeof_compute_features_multiscale_f32(const float* xyz, int64_t n_xyz, const uint32_t* nn, int64_t nnz,
                                          const uint32_t* nn_ptr, int64_t n_points, const uint32_t* k_scales,
                                          int64_t n_scales, float* features, pgeof_stream_t stream);

/* kNN + features in one device pipeline for feature-only callers (no
 * reference counterpart: the reference composes knn_search and
 * compute_features* through host arrays). Writes what
 * compute_features(xyz, knn_search(xyz, xyz, knn)) writes when n_scales == 0
 * (n x 11), or compute_features_multiscale(..., k_scales) (n x n_scales x 11)
 * with k_scales ascending and <= knn. The neighbour lists stay in device
 * scratch in cell order and no distances are written. Device pointers;
 * k_scales is a host array. */
int pgeof_knn_features_f32(const float* xyz, int64_t n, uint32_t knn, const uint32_t* k_scales, int64_t n_scales,
                           float* features, pgeof_stream_t stream);

/* compute_geometric_features_optimal<float, 12>, include/pgeof.hpp:243-310.
 * features: (n_points, 12); column 11 holds the optimal k as a float.
 * Errors: k_min < 1 and k_min_search < 1; k_step == 0 (the reference divides
 * by it). */
int pgeof_compute_features_optimal_f32(const float* xyz, int64_t n_xyz, const uint32_t* nn, int64_t nnz,
                                       const uint32_t* nn_ptr, int64_t n_points, uint32_t k_min, uint32_t k_step,
                                       uint32_t k_min_search, float* features, pgeof_stream_t stream);

/* The three CSR feature passes above for a float64 cloud: the reference's
 * drivers and PCA are templates on real_t (include/pgeof.hpp:75-117, 123-211,
 * 243-310; include/pca.hpp:72-200) that its binding instantiates for float
 * only; these are the real_t = double instantiations (two-pass covariance,
 * eigen solve and feature formulas in double). Same arguments, checks, zero
 * rules and output layouts, with double xyz and double features. */
int pgeof_compute_features_f64(const double* xyz, int64_t n_xyz, const uint32_t* nn, int64_t nnz,
                               const uint32_t* nn_ptr, int64_t n_points, uint64_t k_min, double* features,
                               pgeof_stream_t stream);
int pgeof_compute_features_multiscale_f64(const double* xyz, int64_t n_xyz, const uint32_t* nn, int64_t nnz,
                                          const uint32_t* nn_ptr, int64_t n_points, const uint32_t* k_scales,
                                          int64_t n_scales, double* features, pgeof_stream_t stream);
int pgeof_compute_features_optimal_f64(const double* xyz, int64_t n_xyz, const uint32_t* nn, int64_t nnz,
                                       const uint32_t* nn_ptr, int64_t n_points, uint32_t k_min, uint32_t k_step,
                                       uint32_t k_min_search, double* features, pgeof_stream_t stream);

/* compute_geometric_features_selected<float>, include/pgeof.hpp:325-375.
 * Radius search (< search_radius^2) around every point, the nearest max_knn
 * kept, PCA, then the selected EFeatureIDs in list order. `selected` is a HOST
 * array of EFeatureID values. Points with fewer than 2 points inside the radius
 * are 0; K_optimal and unknown ids stay 0. features: (n, n_selected). */
int pgeof_compute_features_selected_f32(const float* xyz, int64_t n, float search_radius, uint32_t max_knn,
                                        const int32_t* selected, int64_t n_selected, float* features,
                                        pgeof_stream_t stream);

/* compute_geometric_features_selected<double>, include/pgeof.hpp:325-375
 * (bound first in src/pgeof_ext.cpp:148). Same as above in double precision. */
int pgeof_compute_features_selected_f64(const double* xyz, int64_t n, double search_radius, uint32_t max_knn,
                                        const int32_t* selected, int64_t n_selected, double* features,
                                        pgeof_stream_t stream);

/* compute_features for callers that cannot allocate GPU memory. No
 * counterpart in the reference: pgeof allocates freely on the CPU.
 * Same arguments, checks and output as pgeof_compute_features_f32, plus
 * `error_bits`: an optional caller-owned device word (zero it first) into
 * which the kernels OR the data-error bits of pgeof_take_device_errors; with
 * NULL they accumulate in a fixed library word for the device, which
 * pgeof_take_device_errors reads and clears (that call is not itself
 * allocation-free on its first use on a device).
 * This call makes no cudaMalloc, cudaFree or pool allocation: its scratch (a
 * float4 copy of xyz) is a fixed 16 MiB device array that every GPU loading
 * the library holds until exit, so xyz is limited to 1,048,576 points (more
 * returns PGEOF_ERR_INVALID_ARGUMENT). All calls share that array: calls that
 * overlap on the GPU race and must be serialised by the caller. The first call
 * on each device looks the array's address up (cudaGetSymbolAddress) with that
 * device current; make it before any stream capture (a failed lookup is
 * retried by the next call). */
int pgeof_compute_features_f32_noalloc(const float* xyz, int64_t n_xyz, const uint32_t* nn, int64_t nnz,
                                       const uint32_t* nn_ptr, int64_t n_points, uint64_t k_min, float* features,
                                       uint32_t* error_bits, pgeof_stream_t stream);

/* ------------------------------------------------ multi-cloud batches */
/* knn_search(cloud, cloud, knn) followed by compute_features(k_min=1) on the
 * kNN CSR, for many clouds at once (include/nn_search.hpp:31-67 and
 * include/pgeof.hpp:75-117 per cloud). xyz holds the clouds back to back;
 * `offsets` is a HOST array of n_clouds + 1 row offsets (offsets[0] = 0).
 * indices: (N, knn) uint32, local to each cloud; sqr_dist: (N, knn);
 * features: (N, 11) or NULL. Results equal the per-cloud calls exactly.
 * Errors: knn larger than some cloud. */
int pgeof_batch_knn_features_f32(const float* xyz, const int64_t* offsets, int64_t n_clouds, uint32_t knn,
                                 uint32_t* indices, float* sqr_dist, float* features, pgeof_stream_t stream);

/* The same pipeline captured once into a CUDA graph for a fixed batch shape
 * and fixed device buffers: create (tunes the speed parameters on the given
 * data -- the grid cell occupancy factor and the queries per search work
 * item -- or reuses those of an earlier plan of the same shape class: device,
 * knn and the log2 buckets of the point count, mean cloud size and cloud
 * count; synchronises `stream`), then launch any number of times after
 * refilling xyz in place. No reference counterpart (the reference has no
 * batch API). */
typedef struct pgeof_batch_plan_s* pgeof_batch_plan;
int pgeof_batch_plan_create(const float* xyz, const int64_t* offsets, int64_t n_clouds, uint32_t knn,
                            uint32_t* indices, float* sqr_dist, float* features, pgeof_stream_t stream,
                            pgeof_batch_plan* out);
int pgeof_batch_plan_launch(pgeof_batch_plan plan, pgeof_stream_t stream);
/* The parameters a plan runs with: cell occupancy factor (times the default
 * knn / 3.5 points per cell), queries per search work item (0: guided items,
 * long while many queries remain, short at the end), the pipeline time
 * with them and with the defaults (1.0, 16) at tuning, and whether they came
 * from the shape-class cache. Any output pointer may be NULL. */
int pgeof_batch_plan_info(pgeof_batch_plan plan, float* cell_factor, uint32_t* queries_per_item, float* tuned_ms,
                          float* default_ms, int* from_cache);
int pgeof_batch_plan_destroy(pgeof_batch_plan plan);

/* ------------------------------------------------ request server */
/* compute_features_selected (include/pgeof.hpp:325-375) served to a stream of
 * independent requests (no reference counterpart: pgeof has no serving layer).
 * `slots` worker threads, each with its own CUDA stream, admit requests in
 * arrival order as soon as a slot is free and the request's device-memory
 * footprint fits in `budget_bytes` next to the requests in flight (a request
 * larger than the budget runs alone), so requests overlap on the GPU. Each
 * request runs pgeof_host_compute_features_selected_f32/_f64 with its own
 * HOST buffers, which must stay valid until pgeof_server_wait returns for it;
 * its result equals that call made alone.
 * create: on the current device. submit: enqueues and returns at once.
 * wait: blocks until the request is done, returns ITS status (argument and
 * data errors of the call) and forgets it; latency_ms = submit to done,
 * queue_ms = submit to admission, slot = the worker that ran it (each may be
 * NULL). destroy: finishes queued and in-flight requests, joins the workers;
 * no other call on the same server may run during or after it. submit, wait
 * and stats are thread-safe. */
typedef struct pgeof_server_s* pgeof_server;
int pgeof_server_create(int slots, uint64_t budget_bytes, pgeof_server* out);
int pgeof_server_submit_selected_f32(pgeof_server server, const float* xyz, int64_t n, float search_radius,
                                     uint32_t max_knn, const int32_t* selected, int64_t n_selected, float* features,
                                     uint64_t* request_id);
int pgeof_server_submit_selected_f64(pgeof_server server, const double* xyz, int64_t n, double search_radius,
                                     uint32_t max_knn, const int32_t* selected, int64_t n_selected, double* features,
                                     uint64_t* request_id);
/* Resident clouds: add_cloud uploads a float32 cloud and builds its grid once
 * (synchronous; radius_hint / k_hint choose the cell size as the per-call
 * radius path does, results never depend on them) and reserves its device
 * bytes from the budget; requests submitted with its id skip the upload and
 * the grid build and return exactly what the call on the same xyz returns.
 * remove_cloud refuses new requests on it, waits for the queued ones and
 * releases its bytes. The caller's xyz is not referenced after add_cloud. */
int pgeof_server_add_cloud_f32(pgeof_server server, const float* xyz, int64_t n, float radius_hint,
                               uint32_t k_hint, uint64_t* cloud_id);
int pgeof_server_remove_cloud(pgeof_server server, uint64_t cloud_id);
int pgeof_server_submit_selected_resident_f32(pgeof_server server, uint64_t cloud_id, float search_radius,
                                              uint32_t max_knn, const int32_t* selected, int64_t n_selected,
                                              float* features, uint64_t* request_id);
int pgeof_server_wait(pgeof_server server, uint64_t request_id, double* latency_ms, double* queue_ms, int* slot);
int pgeof_server_stats(pgeof_server server, uint64_t* peak_bytes, int* peak_in_flight, uint64_t* completed);
int pgeof_server_destroy(pgeof_server server);

/* ------------------------------------------------ resident cloud index */
/* The reference rebuilds its KD-tree inside every search call
 * (include/nn_search.hpp:35,39,90,97; include/pgeof.hpp:330,333); a resident
 * index builds one cloud's grid once and serves any number of searches with
 * any k or radius, each returning exactly what pgeof_knn_search_f32 /
 * pgeof_radius_search_f32 return for the same data (the search is exact for
 * any cell size; the hints only steer its speed).
 *
 * create: `data` (device, (n_data, 3)) is read during the call only (the index
 * keeps its own cell-ordered copy); k_hint = the neighbour count searches will
 * mostly ask for (0: 16), radius_hint = their radius (0: none). Synchronises
 * `stream`; afterwards any stream of the same device may search the index,
 * concurrently, and calls from several host threads are safe. destroy waits
 * for the searches enqueued so far; no call on the index may run during or
 * after it.
 * query == NULL searches the indexed points themselves (n_query ignored,
 * n_data rows in the cloud's original order): the self-search of
 * knn_search(xyz, xyz, k).
 * index_knn_features: the kNN -> compute_features(k_min = 1) or
 * compute_features_multiscale(k_scales) pipeline of pgeof_knn_features_f32
 * on the indexed cloud; features (n_data, max(1, n_scales), 11). */
typedef struct pgeof_index_s* pgeof_index;
int pgeof_index_create_f32(const float* data, int64_t n_data, uint32_t k_hint, float radius_hint,
                           pgeof_stream_t stream, pgeof_index* out);
int pgeof_index_destroy(pgeof_index index);
int pgeof_index_size(pgeof_index index, int64_t* n_points);
/* nanoflann_knn_search<float>, include/nn_search.hpp:31-67, on the index. */
int pgeof_index_knn_search_f32(pgeof_index index, const float* query, int64_t n_query, uint32_t knn,
                               uint32_t* indices, float* sqr_dist, pgeof_stream_t stream);
/* nanoflann_radius_search<float>, include/nn_search.hpp:85-132, on the index. */
int pgeof_index_radius_search_f32(pgeof_index index, const float* query, int64_t n_query, float search_radius,
                                  uint32_t max_knn, int32_t* indices, float* sqr_dist, pgeof_stream_t stream);
int pgeof_index_knn_features_f32(pgeof_index index, uint32_t knn, const uint32_t* k_scales, int64_t n_scales,
                                 float* features, pgeof_stream_t stream);

/* ------------------------------------------------ host-pointer API (sync) */
/* Same semantics as the device entry points above; every pointer is host
 * memory. These are what the Python drop-in binding calls for numpy inputs. */

/* include/nn_search.hpp:31-67 */
int pgeof_host_knn_search_f32(const float* data, int64_t n_data, const float* query, int64_t n_query,
                              uint32_t knn, uint32_t* indices, float* sqr_dist);
/* include/nn_search.hpp:85-132 */
int pgeof_host_radius_search_f32(const float* data, int64_t n_data, const float* query, int64_t n_query,
                                 float search_radius, uint32_t max_knn, int32_t* indices, float* sqr_dist);
/* include/pgeof.hpp:75-117 */
int pgeof_host_compute_features_f32(const float* xyz, int64_t n_xyz, const uint32_t* nn, int64_t nnz,
                                    const uint32_t* nn_ptr, int64_t n_points, uint64_t k_min, float* features);
/* include/pgeof.hpp:123-211 */
int pgeof_host_compute_features_multiscale_f32(const float* xyz, int64_t n_xyz, const uint32_t* nn, int64_t nnz,
                                               const uint32_t* nn_ptr, int64_t n_points, const uint32_t* k_scales,
                                               int64_t n_scales, float* features);
/* include/pgeof.hpp:243-310 */
int pgeof_host_compute_features_optimal_f32(const float* xyz, int64_t n_xyz, const uint32_t* nn, int64_t nnz,
                                            const uint32_t* nn_ptr, int64_t n_points, uint32_t k_min,
                                            uint32_t k_step, uint32_t k_min_search, float* features);
/* float64 instantiations of the three passes above */
int pgeof_host_compute_features_f64(const double* xyz, int64_t n_xyz, const uint32_t* nn, int64_t nnz,
                                    const uint32_t* nn_ptr, int64_t n_points, uint64_t k_min, double* features);
int pgeof_host_compute_features_multiscale_f64(const double* xyz, int64_t n_xyz, const uint32_t* nn, int64_t nnz,
                                               const uint32_t* nn_ptr, int64_t n_points, const uint32_t* k_scales,
                                               int64_t n_scales, double* features);
int pgeof_host_compute_features_optimal_f64(const double* xyz, int64_t n_xyz, const uint32_t* nn, int64_t nnz,
                                            const uint32_t* nn_ptr, int64_t n_points, uint32_t k_min,
                                            uint32_t k_step, uint32_t k_min_search, double* features);
/* include/pgeof.hpp:325-375 (float) */
int pgeof_host_compute_features_selected_f32(const float* xyz, int64_t n, float search_radius, uint32_t max_knn,
                                             const int32_t* selected, int64_t n_selected, float* features);
/* include/pgeof.hpp:325-375 (double) */
int pgeof_host_compute_features_selected_f64(const double* xyz, int64_t n, double search_radius,
                                             uint32_t max_knn, const int32_t* selected, int64_t n_selected,
                                             double* features);

#ifdef __cplusplus
}
#endif

#endif /* PGEOF_CUDA_H */
