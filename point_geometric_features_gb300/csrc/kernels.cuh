// kernels.cuh -- host-side launchers shared between the translation units of
// libpgeof_cuda (feature kernels, grid index, neighbour search).
#pragma once

#include "common.cuh"

namespace pgeof {

// ----------------------------------------------------------- feature passes
int pad_xyz(const float* xyz, uint64_t n, float4* out, cudaStream_t s);
// cloud_off (device, n_clouds + 1): rows of a multi-cloud batch, neighbour
// indices local to each cloud's slice of xyz4 (null: one cloud).
// ptr == nullptr: every row has uniform_k neighbours (row i at nn[i * uniform_k]).
// row_map (n_points entries): row i's features go to output row row_map[i].idx.
// row_base: the launch covers rows [row_base, row_base + n_points) of ptr / out.
// row_map_input: row i also reads CSR row row_map[i].idx (rows processed in the
// order of row_map, each written to its own output row).
template <typename T>
struct SPoint;
int launch_features(const float4* xyz4, uint64_t n_xyz, const uint32_t* nn, uint64_t nnz, const uint32_t* ptr,
                    uint64_t n_points, bool full, uint64_t k_min, const uint32_t* scales, int n_scales,
                    float* out, unsigned long long* resolved, cudaStream_t s, const uint64_t* cloud_off = nullptr,
                    int n_clouds = 0, const SPoint<float>* row_map = nullptr, uint32_t uniform_k = 0,
                    uint64_t row_base = 0, bool row_map_input = false, unsigned long long* defer = nullptr);
// The three CSR feature passes for a float64 cloud (kind 0 compute_features,
// 1 multiscale over the HOST array `scales`, 2 optimal); out is float64 with
// rows of 11, n_scales * 11 or 12 values.
int launch_features_f64(const double* xyz, uint64_t n_xyz, const uint32_t* nn, uint64_t nnz, const uint32_t* ptr,
                        uint64_t n_points, int kind, uint64_t k_min, const uint32_t* scales, int n_scales,
                        uint32_t k_step, uint32_t k_min_search, double* out, cudaStream_t s);
// out[3 i .. 3 i + 2]: coordinates of CSR row i's first neighbour (point 0's for
// an empty or invalid row).
int first_neighbour_xyz(const float* xyz, uint64_t n_xyz, const uint32_t* nn, uint64_t nnz, const uint32_t* ptr,
                        uint64_t n_rows, float* out, cudaStream_t s);
int launch_optimal(const float4* xyz4, uint64_t n_xyz, const uint32_t* nn, uint64_t nnz, const uint32_t* ptr,
                   uint64_t n_points, uint32_t k_min, uint32_t k_step, uint32_t k_min_search, float* out,
                   unsigned long long* stats, cudaStream_t s);

// ----------------------------------------------------------- grid index
// Uniform grid over the bounding box. Cells are numbered x-fastest
// (id = (cz * gy + cy) * gx + cx); points are counting-sorted by cell so every
// cell, and every run of cells along x, is one contiguous range. Cells may be
// split `xsub` times along x: a search still reads one contiguous run per row
// of cells (fixed y, z), so the finer x edge only trims the ends of each run
// closer to the query's sphere, at no cost in rows.
struct GridParams {
    float ox, oy, oz;    // origin (bounding-box minimum)
    float h, inv_h;      // cell edge along y and z, and its inverse
    float hx, inv_hx;    // cell edge along x (h / xsub), and its inverse
    int xsub;            // x cells per y/z edge
    int gx, gy, gz;      // cells per axis
    uint32_t n_cells;    // gx * gy * gz
    float margin;        // slack added to every cell-distance bound
};

// Min / max of three coordinates over the block (blockDim.x a multiple of 32,
// every thread calls it); thread 0 holds the result. One atomic per value and
// block then replaces one per warp, which serialised on six addresses.
__device__ __forceinline__ void block_box_reduce(float (&mn)[3], float (&mx)[3]) {
    __shared__ float part[6][32];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
#pragma unroll
    for (int a = 0; a < 3; ++a)
        for (int o = 16; o > 0; o >>= 1) {
            mn[a] = fminf(mn[a], __shfl_xor_sync(0xffffffffu, mn[a], o));
            mx[a] = fmaxf(mx[a], __shfl_xor_sync(0xffffffffu, mx[a], o));
        }
    if (lane == 0) {
#pragma unroll
        for (int a = 0; a < 3; ++a) {
            part[a][w] = mn[a];
            part[3 + a][w] = mx[a];
        }
    }
    __syncthreads();
    if (w == 0) {
#pragma unroll
        for (int a = 0; a < 3; ++a) {
            mn[a] = lane < nw ? part[a][lane] : INFINITY;
            mx[a] = lane < nw ? part[3 + a][lane] : -INFINITY;
            for (int o = 16; o > 0; o >>= 1) {
                mn[a] = fminf(mn[a], __shfl_xor_sync(0xffffffffu, mn[a], o));
                mx[a] = fmaxf(mx[a], __shfl_xor_sync(0xffffffffu, mx[a], o));
            }
        }
    }
}

// A point in cell order: coordinates plus its original row index.
template <typename T>
struct SPoint;
template <>
struct __align__(16) SPoint<float> {
    float x, y, z;
    uint32_t idx;
};
template <>
struct __align__(32) SPoint<double> {
    double x, y, z;
    uint32_t idx, pad;
};

template <typename T>
struct GridIndex {
    GridParams g{};
    uint64_t n = 0;
    uint32_t* cell_start = nullptr;  // n_cells + 1 (device)
    SPoint<T>* pts = nullptr;        // n (device), cell order
    Scratch cell_mem, pts_mem;
};

// Build the index of `xyz` (device, row-major (n, 3)). `k_target` steers the
// cell size towards ~k_target/3.5 points per cell around an average point;
// `h_min`/`h_max` (> 0) clamp the edge (radius searches).
template <typename T>
int build_grid(const T* xyz, uint64_t n, uint32_t k_target, float h_min, float h_max, GridIndex<T>& out,
               cudaStream_t s);

// Counting-sort arbitrary query points into `grid`'s cell order; `start`
// receives the per-cell offsets of the sorted queries (n_cells + 1).
template <typename T>
int sort_queries(const T* q, uint64_t m, const GridParams& g, Scratch& out_mem, SPoint<T>** out, Scratch& start,
                 cudaStream_t s);

// Multi-cloud batches: cloud c owns points [off[c], off[c + 1]) of the
// concatenated input and of the cell-sorted point array, and cells
// [cell_base[c], cell_base[c] + g[c].n_cells) of the shared cell table, whose
// entries are positions in the shared sorted array. n == 0: a single cloud.
struct CloudTable {
    const GridParams* g = nullptr;
    const uint32_t* cell_base = nullptr;
    const uint64_t* off = nullptr;
    int n = 0;
};

// The cloud owning position `pos` (last c with off[c] <= pos).
__device__ __forceinline__ int cloud_of(const CloudTable& ct, uint64_t pos) {
    int lo = 0, hi = ct.n - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (ct.off[mid] <= pos) lo = mid;
        else hi = mid - 1;
    }
    return lo;
}

// ----------------------------------------------------------- neighbour search
enum SearchMode { MODE_KNN = 0, MODE_RADIUS = 1 };

// compute_features_selected fused into the radius search
// (include/pgeof.hpp:325-375): each query's nearest min(found, max_knn)
// neighbours go from the search's selection straight to PCA and the selected
// features; no neighbour table is written.
constexpr int kSelMaxIds = 32;  // feature ids per launch
template <typename T>
struct SelSpec {
    const float4* xyz4 = nullptr;  // float: the cloud padded to 16-byte rows, original order
    const T* xyz = nullptr;        // double: the cloud, (n, 3), original order
    T* out = nullptr;              // (n, out_stride)
    uint32_t max_knn = 0;
    uint32_t out_stride = 0;       // values per output row
    uint32_t id_offset = 0;        // first output column of this launch
    int n_ids = 0;
    int ids[kSelMaxIds] = {};
    int order = 0;
    int ring = 1;                  // queries a warp gathers before its lanes solve them together
};
// Queries a warp parks before solving them one per lane: up to 32 while the
// parked neighbour lists fit ~4 KB of shared memory per warp.
__host__ __device__ inline int sel_ring_slots(uint32_t max_knn) {
    const uint32_t r = 1024u / (max_knn > 0 ? max_knn : 1u);
    return (int)(r < 1 ? 1 : (r > 32 ? 32 : r));
}
__host__ __device__ inline size_t sel_ring_bytes(uint32_t max_knn, int ring) {
    const size_t words = (size_t)(max_knn > 0 ? max_knn : 1) * (ring + 1) + 2 * (size_t)ring;
    return (words * sizeof(uint32_t) + 15) / 16 * 16;
}

template <typename T>
struct SearchOut {
    void* indices = nullptr;          // uint32 (knn) or int32 (radius), (m, k)
    T* sqr_dist = nullptr;            // (m, k), may be null
    uint32_t* found = nullptr;        // optional: uncapped count inside the radius
    bool radius_fill_last = true;     // nanoflann RKNN: radius^2 in the last slot of short rows
    bool rows_in_query_order = false; // row q holds queries[q] (cell order), not queries[q].idx
    const SelSpec<T>* sel = nullptr;  // radius mode: selected features instead of the table
};

// `queries` are in `grid`'s cell order; `qstart` (n_cells + 1) gives each
// cell's range of them (grid.cell_start when the queries are the points).
template <typename T>
int launch_search(const GridIndex<T>& grid, const SPoint<T>* queries, const uint32_t* qstart, uint64_t m, int mode,
                  uint32_t k, T radius, const SearchOut<T>& out, cudaStream_t s);

// Self-kNN over a multi-cloud batch: `pts` are all clouds' points in (cloud,
// cell) order with cloud-local indices, `cell_start` the shared cell table;
// output rows are global (off[c] + local index), neighbour indices local.
// `work` points to 8 zeroed words and `ovf` to n_points words of device scratch.
// `chunk`: consecutive queries per work item of the search (speed only).
int launch_search_batch(const CloudTable& ct, const uint32_t* cell_start, const SPoint<float>* pts, uint64_t n_points,
                        uint32_t k, uint32_t* indices, float* sqr_dist, uint32_t* work, uint32_t* ovf,
                        cudaStream_t s, uint32_t chunk = 16);

// Exclusive scan of G counts into out[0..G] (out[G] = total) with caller-owned
// partials (ceil(G / 1024) words).
int exclusive_scan_into(const uint32_t* in, uint32_t G, uint32_t* out, uint32_t* partials, cudaStream_t s);

// Radius-search table (m, max_knn) + uncapped counts -> CSR: nn_ptr[0..m] and
// the first min(found, max_knn) entries of each row packed into nn. `counts`
// (m words) and `partials` (ceil(m / 1024) words) are scratch.
int launch_csr_from_table(const int32_t* table, const uint32_t* found, uint64_t m, uint32_t max_knn,
                          uint32_t* counts, uint32_t* partials, uint32_t* nn_ptr, uint32_t* nn, cudaStream_t s);

// A float32 cloud kept on the device with its grid, for repeated
// compute_features_selected requests (request server).
struct ResidentCloud {
    uint64_t n = 0;
    Scratch xyz;  // (n, 3) float32, original order
    GridIndex<float> grid;
};
// Upload + grid build on the calling thread's host stream; synchronous.
int resident_cloud_build(const float* xyz, uint64_t n, float radius_hint, uint32_t k_hint, ResidentCloud& out);
// compute_features_selected on a resident cloud; `features` is host memory,
// synchronous on the calling thread's host stream.
int host_selected_resident(const ResidentCloud& c, float radius, uint32_t max_knn, const int32_t* ids,
                           int64_t n_ids, float* features);


}  // namespace pgeof
