// batch.cu -- many clouds of uneven size through one device-resident pipeline:
// per-cloud bounding boxes and grid parameters computed on the device, one
// counting sort of every point by (cloud, cell), one kNN launch and one feature
// launch over all points. No host round trip happens between the kernels, so
// the whole pipeline can be captured once into a CUDA graph and replayed
// (pgeof_batch_plan_*); the per-cloud alternative is one knn_search and one
// compute_features call per cloud (include/nn_search.hpp:31-67,
// include/pgeof.hpp:75-117), each with its own grid build and launches.
//
// Results equal the per-cloud calls exactly: neighbour indices are local to
// each cloud, rows keep the input order, and selection is exact whatever the
// cell size.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <map>
#include <mutex>
#include <tuple>
#include <vector>

#include "kernels.cuh"

namespace pgeof {

namespace {

__device__ __forceinline__ uint32_t ord_key(float f) {
    const uint32_t u = __float_as_uint(f);
    return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}
__device__ __forceinline__ float ord_val(uint32_t k) {
    const uint32_t u = (k & 0x80000000u) ? (k & 0x7fffffffu) : ~k;
    return __uint_as_float(u);
}

__device__ __forceinline__ int cloud_of_off(const uint64_t* off, int n, uint64_t pos) {
    int lo = 0, hi = n - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (off[mid] <= pos) lo = mid;
        else hi = mid - 1;
    }
    return lo;
}

// grid: x splits a cloud's points, y = cloud
__global__ void batch_bbox_kernel(const float* __restrict__ xyz, const uint64_t* __restrict__ off,
                                  uint32_t* __restrict__ box) {
    const int c = blockIdx.y;
    const uint64_t b = off[c], e = off[c + 1];
    float mn[3] = {INFINITY, INFINITY, INFINITY}, mx[3] = {-INFINITY, -INFINITY, -INFINITY};
    for (uint64_t i = b + blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < e;
         i += (uint64_t)gridDim.x * blockDim.x) {
#pragma unroll
        for (int a = 0; a < 3; ++a) {
            const float v = xyz[3 * i + a];
            mn[a] = fminf(mn[a], v);
            mx[a] = fmaxf(mx[a], v);
        }
    }
    block_box_reduce(mn, mx);
    if (threadIdx.x == 0 && e > b) {
#pragma unroll
        for (int a = 0; a < 3; ++a) {
            atomicMin(box + 6 * c + a, ord_key(mn[a]));
            atomicMax(box + 6 * c + 3 + a, ord_key(mx[a]));
        }
    }
}

__global__ void box_init_kernel(uint32_t* box, int n_clouds) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < 6 * n_clouds; i += gridDim.x * blockDim.x)
        box[i] = (i % 6) < 3 ? 0xffffffffu : 0u;
}

// Grid parameters of one cloud for edge h, growing h until the cloud's cell cap
// holds (same rules as the single-cloud build).
__device__ void cloud_params(const float* mn, const float* mx, double h, uint64_t cap, GridParams& g) {
    for (int it = 0; it < 200; ++it) {
        uint64_t G = 1;
        int d[3];
        bool ok = true;
        for (int a = 0; a < 3; ++a) {
            const double cells = floor(((double)mx[a] - (double)mn[a]) / h) + 1.0;
            if (cells > 2.0e9) {
                ok = false;
                break;
            }
            d[a] = (int)cells;
            G *= (uint64_t)d[a];
            if (G > cap) {
                ok = false;
                break;
            }
        }
        if (ok) {
            g.ox = mn[0];
            g.oy = mn[1];
            g.oz = mn[2];
            g.h = (float)h;
            g.inv_h = (float)(1.0 / h);
            g.hx = g.h;
            g.inv_hx = g.inv_h;
            g.xsub = 1;
            g.gx = d[0];
            g.gy = d[1];
            g.gz = d[2];
            g.n_cells = (uint32_t)G;
            double maxc = 0.0;
            for (int a = 0; a < 3; ++a) maxc = fmax(maxc, fmax(fabs((double)mn[a]), fabs((double)mx[a])));
            int ex = 0;
            frexp(fmax(maxc, 1e-30), &ex);
            g.margin = (float)(16.0 * ldexp(1.0, ex - 24) + 1e-5 * h);
            return;
        }
        h *= 1.25;
    }
}

// One thread per cloud. pass 0: trial edge (volume estimate); pass 1: the edge
// corrected by the measured point-weighted occupancy (surface exponent). The
// single block also lays out the cells of all clouds (exclusive scan).
__global__ void batch_params_kernel(const uint32_t* __restrict__ box, const uint64_t* __restrict__ off, int n_clouds,
                                    float target, int pass, const unsigned long long* __restrict__ occ,
                                    GridParams* __restrict__ g, uint32_t* __restrict__ cell_base) {
    for (int c = threadIdx.x; c < n_clouds; c += blockDim.x) {
        const uint64_t n = off[c + 1] - off[c];
        float mn[3], mx[3];
        for (int a = 0; a < 3; ++a) {
            mn[a] = n ? ord_val(box[6 * c + a]) : 0.0f;
            mx[a] = n ? ord_val(box[6 * c + 3 + a]) : 0.0f;
        }
        double ext_max = 1e-30, vol = 1.0;
        for (int a = 0; a < 3; ++a) ext_max = fmax(ext_max, (double)mx[a] - (double)mn[a]);
        for (int a = 0; a < 3; ++a) vol *= fmax((double)mx[a] - (double)mn[a], ext_max * 1e-3);
        const uint64_t cap = 4 * n + 64;
        const double floor_h = ext_max * 1e-7 + 1e-30;
        double h = fmax(cbrt(vol * target / (double)(n ? n : 1)), floor_h);
        if (pass == 1 && n > 64) {
            const double m_w = (double)occ[c] / (double)n;
            if (m_w > 0.0) h = fmax(h * fmin(16.0, fmax(1.0 / 16.0, sqrt(target / m_w))), floor_h);
        }
        GridParams gp;
        cloud_params(mn, mx, h, cap, gp);
        g[c] = gp;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        uint32_t acc = 0;
        for (int c = 0; c < n_clouds; ++c) {
            cell_base[c] = acc;
            acc += g[c].n_cells;
        }
        cell_base[n_clouds] = acc;
    }
}

__device__ __forceinline__ uint32_t local_cell(const GridParams& g, float x, float y, float z) {
    const float fx = (x - g.ox) * g.inv_hx, fy = (y - g.oy) * g.inv_h, fz = (z - g.oz) * g.inv_h;
    const int cx = (int)floorf(fminf(fmaxf(fx, 0.0f), (float)(g.gx - 1)));
    const int cy = (int)floorf(fminf(fmaxf(fy, 0.0f), (float)(g.gy - 1)));
    const int cz = (int)floorf(fminf(fmaxf(fz, 0.0f), (float)(g.gz - 1)));
    return ((uint32_t)cz * (uint32_t)g.gy + (uint32_t)cy) * (uint32_t)g.gx + (uint32_t)cx;
}

__global__ void batch_hist_kernel(const float* __restrict__ xyz, uint64_t n, const uint64_t* __restrict__ off,
                                  int n_clouds, const GridParams* __restrict__ g, const uint32_t* __restrict__ cell_base,
                                  uint32_t* __restrict__ counts, uint32_t* __restrict__ cell_out,
                                  uint32_t* __restrict__ rank_out) {
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
        const int c = cloud_of_off(off, n_clouds, i);
        const uint32_t cell = cell_base[c] + local_cell(g[c], xyz[3 * i], xyz[3 * i + 1], xyz[3 * i + 2]);
        const uint32_t r = atomicAdd(counts + cell, 1u);
        if (cell_out) {
            cell_out[i] = cell;
            rank_out[i] = r;
        }
    }
}

// point-weighted occupancy per cloud: sum over its cells of count^2
__global__ void batch_occ_kernel(const uint32_t* __restrict__ counts, const uint32_t* __restrict__ cell_base,
                                 int n_clouds, unsigned long long* __restrict__ occ) {
    const uint32_t total = cell_base[n_clouds];
    for (uint32_t cell = blockIdx.x * blockDim.x + threadIdx.x; cell < total; cell += gridDim.x * blockDim.x) {
        const uint32_t v = counts[cell];
        if (v) {
            int lo = 0, hi = n_clouds - 1;
            while (lo < hi) {
                const int mid = (lo + hi + 1) >> 1;
                if (cell_base[mid] <= cell) lo = mid;
                else hi = mid - 1;
            }
            atomicAdd(occ + lo, (unsigned long long)v * v);
        }
    }
}

__global__ void batch_scatter_kernel(const float* __restrict__ xyz, uint64_t n, const uint64_t* __restrict__ off,
                                     int n_clouds, const uint32_t* __restrict__ start, const uint32_t* __restrict__ cell,
                                     const uint32_t* __restrict__ rank, SPoint<float>* __restrict__ out) {
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
        const int c = cloud_of_off(off, n_clouds, i);
        SPoint<float> p;
        p.x = xyz[3 * i];
        p.y = xyz[3 * i + 1];
        p.z = xyz[3 * i + 2];
        p.idx = (uint32_t)(i - off[c]);
        out[start[cell[i]] + rank[i]] = p;
    }
}

__global__ void uniform_ptr_kernel(uint32_t* ptr, uint64_t n, uint32_t k) {
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i <= n; i += (uint64_t)gridDim.x * blockDim.x)
        ptr[i] = (uint32_t)(i * k);
}

unsigned blocks_for(uint64_t n, int threads, int sm_count) {
    return (unsigned)std::max<uint64_t>(1, std::min<uint64_t>(ceil_div_u(n, threads), (uint64_t)sm_count * 8));
}

}  // namespace

// Device buffers of one batch shape (sizes fixed by the cloud offsets).
struct BatchWorkspace {
    uint64_t n = 0;
    int n_clouds = 0;
    uint64_t max_cells = 0;
    uint32_t k = 0;
    void* base = nullptr;  // one allocation holding everything below
    uint64_t* off = nullptr;
    uint32_t* box = nullptr;
    GridParams* g = nullptr;
    uint32_t* cell_base = nullptr;
    unsigned long long* occ = nullptr;
    uint32_t* counts = nullptr;
    uint32_t* cell_start = nullptr;
    uint32_t* cell = nullptr;
    uint32_t* rank = nullptr;
    SPoint<float>* pts = nullptr;
    float4* xyz4 = nullptr;
    uint32_t* nn_ptr = nullptr;
    uint32_t* words = nullptr;
    uint32_t* scan_part = nullptr;
    unsigned long long* defer = nullptr;  // the feature pass's exact-solve queue
};

namespace {

size_t align_up(size_t x) { return (x + 255) & ~size_t(255); }

// Carve the workspace out of one block of device memory.
size_t layout(BatchWorkspace& w, char* base) {
    size_t o = 0;
    auto take = [&](size_t bytes) {
        char* p = base ? base + o : nullptr;
        o += align_up(bytes);
        return p;
    };
    const uint64_t n = w.n, nc = (uint64_t)w.n_clouds, cells = w.max_cells;
    w.off = (uint64_t*)take((nc + 1) * 8);
    w.box = (uint32_t*)take(nc * 6 * 4);
    w.g = (GridParams*)take(nc * sizeof(GridParams));
    w.cell_base = (uint32_t*)take((nc + 1) * 4);
    w.occ = (unsigned long long*)take(nc * 8);
    w.counts = (uint32_t*)take(cells * 4);
    w.cell_start = (uint32_t*)take((cells + 1) * 4);
    w.cell = (uint32_t*)take(n * 4);
    w.rank = (uint32_t*)take(n * 4);
    w.pts = (SPoint<float>*)take(n * sizeof(SPoint<float>));
    w.xyz4 = (float4*)take(n * sizeof(float4));
    w.nn_ptr = (uint32_t*)take((n + 1) * 4);
    w.words = (uint32_t*)take((n + 8) * 4);
    w.scan_part = (uint32_t*)take((cells / 1024 + 2) * 4);
    w.defer = (unsigned long long*)take((n + 1) * 8);
    return o;
}

int workspace_init(BatchWorkspace& w, const int64_t* offsets, int64_t n_clouds, uint32_t k, bool from_pool,
                   cudaStream_t s) {
    w.n_clouds = (int)n_clouds;
    w.n = (uint64_t)offsets[n_clouds];
    w.k = k;
    w.max_cells = 0;
    for (int64_t c = 0; c < n_clouds; ++c) w.max_cells += 4 * (uint64_t)(offsets[c + 1] - offsets[c]) + 64;
    if (w.max_cells >= 0xffffffffull) return fail(PGEOF_ERR_INVALID_ARGUMENT, "batch too large for 32-bit cell ids");
    const size_t bytes = layout(w, nullptr);
    if (from_pool) {
        PGEOF_TRY(scratch_alloc(&w.base, bytes, s));
    } else {
        PGEOF_CUDA_TRY(cudaMalloc(&w.base, bytes));
        count_device_alloc();
    }
    layout(w, (char*)w.base);
    std::vector<uint64_t> off(n_clouds + 1);
    for (int64_t c = 0; c <= n_clouds; ++c) off[c] = (uint64_t)offsets[c];
    PGEOF_CUDA_TRY(cudaMemcpyAsync(w.off, off.data(), off.size() * 8, cudaMemcpyHostToDevice, s));
    // the staging vector dies here: make the copy complete first
    PGEOF_CUDA_TRY(cudaStreamSynchronize(s));
    return PGEOF_OK;
}

// exclusive scan of w.counts[0..max_cells) into w.cell_start (three passes)
int batch_scan(BatchWorkspace& w, cudaStream_t s);

// Speed parameters of the pipeline (results never depend on them): the grid
// cell occupancy target as a factor of the default k / 3.5 points per cell
// (each cloud's edge is still fitted to its own density), and the consecutive
// queries of one search work item (0: guided items, long while many queries
// remain and short at the end).
struct BatchTune {
    float cell = 1.0f;
    uint32_t chunk = 16;
};

// The whole pipeline: enqueue only (no host synchronisation, no allocation).
int run_pipeline(BatchWorkspace& w, const float* xyz, uint32_t* idx, float* d2, float* features,
                 const BatchTune& tune, cudaStream_t s) {
    const DeviceInfo* di;
    PGEOF_TRY(current_device_info(&di));
    const int nc = w.n_clouds;
    const uint64_t n = w.n;
    const float target = std::min(48.0f, std::max(2.0f, (float)w.k / 3.5f * tune.cell));
    // 1. bounding boxes
    box_init_kernel<<<blocks_for(6 * (uint64_t)nc, 256, di->sm_count), 256, 0, s>>>(w.box, nc);
    {
        KernelTimer kt("batch_bbox_kernel", s);
        dim3 grid(std::max(1u, std::min(64u, (unsigned)ceil_div_u(n / std::max(nc, 1) + 1, 2048))), (unsigned)nc);
        batch_bbox_kernel<<<grid, 256, 0, s>>>(xyz, w.off, w.box);
    }
    // 2. trial edge, occupancy, corrected edge
    {
        KernelTimer kt("batch_grid_params_kernels", s);
        batch_params_kernel<<<1, 256, 0, s>>>(w.box, w.off, nc, target, 0, w.occ, w.g, w.cell_base);
        PGEOF_CUDA_TRY(cudaMemsetAsync(w.counts, 0, w.max_cells * 4, s));
        PGEOF_CUDA_TRY(cudaMemsetAsync(w.occ, 0, (size_t)nc * 8, s));
        batch_hist_kernel<<<blocks_for(n, 256, di->sm_count), 256, 0, s>>>(xyz, n, w.off, nc, w.g, w.cell_base,
                                                                             w.counts, nullptr, nullptr);
        batch_occ_kernel<<<blocks_for(w.max_cells, 256, di->sm_count), 256, 0, s>>>(w.counts, w.cell_base, nc, w.occ);
        batch_params_kernel<<<1, 256, 0, s>>>(w.box, w.off, nc, target, 1, w.occ, w.g, w.cell_base);
    }
    // 3. counting sort by (cloud, cell)
    PGEOF_CUDA_TRY(cudaMemsetAsync(w.counts, 0, w.max_cells * 4, s));
    {
        KernelTimer kt("batch_sort_kernels", s);
        batch_hist_kernel<<<blocks_for(n, 256, di->sm_count), 256, 0, s>>>(xyz, n, w.off, nc, w.g, w.cell_base,
                                                                             w.counts, w.cell, w.rank);
        PGEOF_TRY(batch_scan(w, s));
        batch_scatter_kernel<<<blocks_for(n, 256, di->sm_count), 256, 0, s>>>(xyz, n, w.off, nc, w.cell_start, w.cell,
                                                                                w.rank, w.pts);
    }
    count_launch(8);
    PGEOF_TRY(check_launch("batch grid build"));
    // 4. kNN over all clouds
    CloudTable ct;
    ct.g = w.g;
    ct.cell_base = w.cell_base;
    ct.off = w.off;
    ct.n = nc;
    PGEOF_TRY(launch_search_batch(ct, w.cell_start, w.pts, n, w.k, idx, d2, w.words, w.words + 8, s, tune.chunk));
    // 5. features from the kNN rows (CSR with nn_ptr = k * row)
    if (features) {
        PGEOF_TRY(pad_xyz(xyz, n, w.xyz4, s));
        uniform_ptr_kernel<<<blocks_for(n + 1, 256, di->sm_count), 256, 0, s>>>(w.nn_ptr, n, w.k);
        count_launch();
        PGEOF_TRY(launch_features(w.xyz4, n, idx, n * w.k, w.nn_ptr, n, true, 1, nullptr, 0, features, nullptr, s,
                                  w.off, nc, nullptr, 0, 0, false, w.defer));
    }
    return PGEOF_OK;
}

}  // namespace

int exclusive_scan_into(const uint32_t* in, uint32_t G, uint32_t* out, uint32_t* partials, cudaStream_t s);

namespace {
int batch_scan(BatchWorkspace& w, cudaStream_t s) {
    return exclusive_scan_into(w.counts, (uint32_t)w.max_cells, w.cell_start, w.scan_part, s);
}
}  // namespace

struct BatchPlan {
    BatchWorkspace w;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    BatchTune tune;
    float tuned_ms = 0.0f;    // pipeline time with `tune` at creation
    float default_ms = 0.0f;  // ... and with the default parameters
    int from_cache = 0;       // `tune` came from an earlier plan of the same shape class
};

// Tuned parameters by batch shape class: (device, k, log2 of the point count,
// log2 of the mean cloud size, log2 of the cloud count). A plan of a class
// seen before reuses its parameters without re-tuning.
using TuneKey = std::tuple<int, uint32_t, int, int, int>;
struct TuneEntry {
    BatchTune tune;
    float tuned_ms, default_ms;
};
std::mutex g_tune_mu;
std::map<TuneKey, TuneEntry> g_tune_cache;

int log2_bucket(double v) { return v >= 1.0 ? (int)std::floor(std::log2(v)) : 0; }

// Times every candidate (cell factor x work-item size) twice on the plan's
// own data and keeps the fastest second run.
int autotune(BatchPlan* plan, const float* xyz, uint32_t* indices, float* sqr_dist, float* features, cudaStream_t s) {
    static const float kCells[3] = {0.6f, 1.0f, 1.6f};
    static const uint32_t kChunks[4] = {0, 8, 16, 32};  // 0: guided items (64 shrinking to 4)
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    PGEOF_CUDA_TRY(cudaEventCreate(&e0));
    if (cudaEventCreate(&e1) != cudaSuccess) {
        cudaEventDestroy(e0);
        return fail(PGEOF_ERR_CUDA, "batch autotune: event");
    }
    int st = PGEOF_OK;
    float best = 1e30f;
    for (int rep = 0; rep < 2 && st == PGEOF_OK; ++rep) {
        for (float c : kCells) {
            for (uint32_t q : kChunks) {
                BatchTune t;
                t.cell = c;
                t.chunk = q;
                cudaEventRecord(e0, s);
                st = run_pipeline(plan->w, xyz, indices, sqr_dist, features, t, s);
                cudaEventRecord(e1, s);
                if (st != PGEOF_OK) break;
                if (cudaEventSynchronize(e1) != cudaSuccess) {
                    st = fail(PGEOF_ERR_CUDA, "batch autotune");
                    break;
                }
                float ms = 0.0f;
                cudaEventElapsedTime(&ms, e0, e1);
                if (rep == 1) {
                    if (ms < best) {
                        best = ms;
                        plan->tune = t;
                        plan->tuned_ms = ms;
                    }
                    if (c == 1.0f && q == 16) plan->default_ms = ms;
                }
            }
            if (st != PGEOF_OK) break;
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    return st;
}

}  // namespace pgeof

using namespace pgeof;

namespace {

int check_batch_args(const float* xyz, const int64_t* offsets, int64_t n_clouds, uint32_t knn) {
    if (n_clouds < 1 || !offsets) return fail(PGEOF_ERR_INVALID_ARGUMENT, "a batch needs at least one cloud");
    if (offsets[0] != 0) return fail(PGEOF_ERR_INVALID_ARGUMENT, "offsets[0] must be 0");
    for (int64_t c = 0; c < n_clouds; ++c) {
        if (offsets[c + 1] < offsets[c]) return fail(PGEOF_ERR_INVALID_ARGUMENT, "offsets must be non-decreasing");
        if ((int64_t)knn > offsets[c + 1] - offsets[c])
            return fail(PGEOF_ERR_INVALID_ARGUMENT, "knn size is greater than the data point cloud size (cloud " +
                                                        std::to_string(c) + ")");
    }
    if ((uint64_t)offsets[n_clouds] > 0xfffffffeull) return fail(PGEOF_ERR_INVALID_ARGUMENT, "batch too large");
    if (offsets[n_clouds] > 0 && !xyz) return fail(PGEOF_ERR_INVALID_ARGUMENT, "xyz is null");
    return PGEOF_OK;
}

}  // namespace

extern "C" {

int pgeof_batch_knn_features_f32(const float* xyz, const int64_t* offsets, int64_t n_clouds, uint32_t knn,
                                 uint32_t* indices, float* sqr_dist, float* features, pgeof_stream_t stream) {
    PGEOF_TRY(check_batch_args(xyz, offsets, n_clouds, knn));
    if (offsets[n_clouds] == 0 || knn == 0) return PGEOF_OK;
    const cudaStream_t s = (cudaStream_t)stream;
    BatchWorkspace w;
    PGEOF_TRY(workspace_init(w, offsets, n_clouds, knn, true, s));
    const int st = run_pipeline(w, xyz, indices, sqr_dist, features, BatchTune{}, s);
    scratch_free(w.base, s);
    return st;
}

int pgeof_batch_plan_create(const float* xyz, const int64_t* offsets, int64_t n_clouds, uint32_t knn,
                            uint32_t* indices, float* sqr_dist, float* features, pgeof_stream_t stream,
                            pgeof_batch_plan* out) {
    if (!out) return fail(PGEOF_ERR_INVALID_ARGUMENT, "out is null");
    *out = nullptr;
    PGEOF_TRY(check_batch_args(xyz, offsets, n_clouds, knn));
    if (offsets[n_clouds] == 0 || knn == 0) return fail(PGEOF_ERR_INVALID_ARGUMENT, "empty batch");
    const cudaStream_t s = (cudaStream_t)stream;
    BatchPlan* plan = new BatchPlan();
    int st = workspace_init(plan->w, offsets, n_clouds, knn, false, s);
    // tune the speed parameters on this batch, or reuse those of its shape class
    if (st == PGEOF_OK) {
        int dev = 0;
        cudaGetDevice(&dev);
        const double total = (double)offsets[n_clouds];
        const TuneKey key{dev, knn, log2_bucket(total), log2_bucket(total / (double)n_clouds),
                          log2_bucket((double)n_clouds)};
        bool cached = false;
        {
            std::lock_guard<std::mutex> lk(g_tune_mu);
            const auto it = g_tune_cache.find(key);
            if (it != g_tune_cache.end()) {
                plan->tune = it->second.tune;
                plan->tuned_ms = it->second.tuned_ms;
                plan->default_ms = it->second.default_ms;
                plan->from_cache = 1;
                cached = true;
            }
        }
        if (!cached) {
            st = autotune(plan, xyz, indices, sqr_dist, features, s);
            if (st == PGEOF_OK) {
                std::lock_guard<std::mutex> lk(g_tune_mu);
                g_tune_cache[key] = TuneEntry{plan->tune, plan->tuned_ms, plan->default_ms};
            }
        }
    }
    // capture the tuned pipeline once
    if (st == PGEOF_OK) {
        cudaStream_t cs = nullptr;
        cudaError_t e = cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking);
        if (e == cudaSuccess) e = cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal);
        if (e == cudaSuccess) {
            st = run_pipeline(plan->w, xyz, indices, sqr_dist, features, plan->tune, cs);
            const cudaError_t e2 = cudaStreamEndCapture(cs, &plan->graph);
            if (st == PGEOF_OK && e2 != cudaSuccess)
                st = fail(PGEOF_ERR_CUDA, std::string("graph capture: ") + cudaGetErrorString(e2));
        } else {
            st = fail(PGEOF_ERR_CUDA, std::string("graph capture: ") + cudaGetErrorString(e));
        }
        if (st == PGEOF_OK) {
            e = cudaGraphInstantiate(&plan->exec, plan->graph, 0);
            if (e != cudaSuccess) st = fail(PGEOF_ERR_CUDA, std::string("graph instantiate: ") + cudaGetErrorString(e));
        }
        if (cs) cudaStreamDestroy(cs);
        (void)cudaGetLastError();
    }
    if (st != PGEOF_OK) {
        pgeof_batch_plan_destroy(reinterpret_cast<pgeof_batch_plan>(plan));
        return st;
    }
    *out = reinterpret_cast<pgeof_batch_plan>(plan);
    return PGEOF_OK;
}

int pgeof_batch_plan_launch(pgeof_batch_plan handle, pgeof_stream_t stream) {
    BatchPlan* plan = reinterpret_cast<BatchPlan*>(handle);
    if (!plan || !plan->exec) return fail(PGEOF_ERR_INVALID_ARGUMENT, "invalid plan");
    PGEOF_CUDA_TRY(cudaGraphLaunch(plan->exec, (cudaStream_t)stream));
    count_launch(1);
    return PGEOF_OK;
}

int pgeof_batch_plan_info(pgeof_batch_plan handle, float* cell_factor, uint32_t* queries_per_item, float* tuned_ms,
                          float* default_ms, int* from_cache) {
    const BatchPlan* plan = reinterpret_cast<const BatchPlan*>(handle);
    if (!plan) return fail(PGEOF_ERR_INVALID_ARGUMENT, "invalid plan");
    if (cell_factor) *cell_factor = plan->tune.cell;
    if (queries_per_item) *queries_per_item = plan->tune.chunk;
    if (tuned_ms) *tuned_ms = plan->tuned_ms;
    if (default_ms) *default_ms = plan->default_ms;
    if (from_cache) *from_cache = plan->from_cache;
    return PGEOF_OK;
}

int pgeof_batch_plan_destroy(pgeof_batch_plan handle) {
    BatchPlan* plan = reinterpret_cast<BatchPlan*>(handle);
    if (!plan) return PGEOF_OK;
    if (plan->exec) cudaGraphExecDestroy(plan->exec);
    if (plan->graph) cudaGraphDestroy(plan->graph);
    if (plan->w.base) cudaFree(plan->w.base);
    delete plan;
    return PGEOF_OK;
}

}  // extern "C"
