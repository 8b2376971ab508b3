// grid.cu -- uniform-grid spatial index: bounding box, cell-size selection,
// counting sort of points into cells, and the cell-offset table.
//
// Replaces the nanoflann KD-tree that pgeof rebuilds on every call
// (include/nn_search.hpp:39, :97; include/pgeof.hpp:333). A grid is the GPU
// shape of the problem: the cell table is a prefix sum, points sort into
// cell order with one atomic histogram and one scatter (no comparison sort),
// and a query's candidates are a handful of contiguous runs of that order.
//
// Cell size. The cost of a query is (cells visited) + (candidates examined).
// The target is a point-weighted occupancy sum_c count_c^2 / n (the number of
// points sharing a cell with an average point) of about k/3.5, which puts the
// k-th neighbour roughly one cell away. Occupancy is measured, not assumed:
// LiDAR-like clouds are surfaces (occupancy ~ h^2), volumes give h^3, so the
// edge is found by two trial histograms and a power-law fit of their exponent.
#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <mutex>

#include "kernels.cuh"

namespace pgeof {

namespace {

__device__ __forceinline__ uint32_t ord_key(float f) {
    const uint32_t u = __float_as_uint(f);
    return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}
static inline float ord_decode(uint32_t k) {
    const uint32_t u = (k & 0x80000000u) ? (k & 0x7fffffffu) : ~k;
    float f;
    memcpy(&f, &u, 4);
    return f;
}

template <typename T>
__global__ void bbox_kernel(const T* __restrict__ xyz, uint64_t n, uint32_t* out6) {
    float mn[3] = {INFINITY, INFINITY, INFINITY}, mx[3] = {-INFINITY, -INFINITY, -INFINITY};
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
#pragma unroll
        for (int a = 0; a < 3; ++a) {
            const float v = (float)xyz[3 * i + a];
            mn[a] = fminf(mn[a], v);
            mx[a] = fmaxf(mx[a], v);
        }
    }
    block_box_reduce(mn, mx);
    if (threadIdx.x == 0) {
#pragma unroll
        for (int a = 0; a < 3; ++a) {
            atomicMin(out6 + a, ord_key(mn[a]));
            atomicMax(out6 + 3 + a, ord_key(mx[a]));
        }
    }
}

template <typename T>
__device__ __forceinline__ uint32_t cell_of(const GridParams& g, T x, T y, T z) {
    const float fx = ((float)x - g.ox) * g.inv_hx;
    const float fy = ((float)y - g.oy) * g.inv_h;
    const float fz = ((float)z - g.oz) * g.inv_h;
    const int cx = (int)floorf(fminf(fmaxf(fx, 0.0f), (float)(g.gx - 1)));
    const int cy = (int)floorf(fminf(fmaxf(fy, 0.0f), (float)(g.gy - 1)));
    const int cz = (int)floorf(fminf(fmaxf(fz, 0.0f), (float)(g.gz - 1)));
    return ((uint32_t)cz * (uint32_t)g.gy + (uint32_t)cy) * (uint32_t)g.gx + (uint32_t)cx;
}

template <typename T>
__global__ void hist_kernel(const T* __restrict__ xyz, uint64_t n, GridParams g, uint32_t* __restrict__ counts,
                            uint32_t* __restrict__ cell_out, uint32_t* __restrict__ rank_out) {
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
        const uint32_t c = cell_of<T>(g, xyz[3 * i], xyz[3 * i + 1], xyz[3 * i + 2]);
        const uint32_t r = atomicAdd(counts + c, 1u);
        if (cell_out) {
            cell_out[i] = c;
            rank_out[i] = r;
        }
    }
}

__global__ void sumsq_kernel(const uint32_t* __restrict__ counts, uint32_t G, unsigned long long* out) {
    unsigned long long s = 0;
    for (uint32_t c = blockIdx.x * blockDim.x + threadIdx.x; c < G; c += gridDim.x * blockDim.x) {
        const unsigned long long v = counts[c];
        s += v * v;
    }
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if ((threadIdx.x & 31) == 0 && s) atomicAdd(out, s);
}

// ---- exclusive scan of uint32 counts (three passes over 1024-element tiles)
constexpr int kScanThreads = 256;
constexpr int kScanTile = 1024;

__global__ void scan_partials_kernel(const uint32_t* __restrict__ in, uint32_t G, uint32_t* __restrict__ partial) {
    __shared__ uint32_t warp_sums[kScanThreads / 32];
    const uint32_t base = blockIdx.x * kScanTile;
    uint32_t s = 0;
    for (int t = threadIdx.x; t < kScanTile; t += kScanThreads) {
        const uint32_t i = base + t;
        if (i < G) s += in[i];
    }
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if ((threadIdx.x & 31) == 0) warp_sums[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
        uint32_t t = 0;
        for (int w = 0; w < kScanThreads / 32; ++w) t += warp_sums[w];
        partial[blockIdx.x] = t;
    }
}

// Single block: exclusive scan of the tile partials in place, four
// consecutive partials per thread (1024 per block step).
__global__ void scan_top_kernel(uint32_t* partial, uint32_t nb) {
    __shared__ uint32_t carry;
    __shared__ uint32_t warp_sums[kScanThreads / 32];
    if (threadIdx.x == 0) carry = 0;
    __syncthreads();
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    for (uint32_t base = 0; base < nb; base += 4 * kScanThreads) {
        uint32_t v[4], s = 0;
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            const uint32_t i = base + threadIdx.x * 4 + q;
            v[q] = i < nb ? partial[i] : 0u;
            s += v[q];
        }
        uint32_t x = s;
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
            if (lane >= o) x += y;
        }
        if (lane == 31) warp_sums[w] = x;
        __syncthreads();
        uint32_t wo = 0;
        for (int q = 0; q < w; ++q) wo += warp_sums[q];
        uint32_t run = carry + wo + x - s;
        const uint32_t block_end = carry + wo + x;  // thread kScanThreads - 1: the step's total
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            const uint32_t i = base + threadIdx.x * 4 + q;
            if (i < nb) partial[i] = run;
            run += v[q];
        }
        __syncthreads();
        if (threadIdx.x == kScanThreads - 1) carry = block_end;
        __syncthreads();
    }
}

__global__ void scan_final_kernel(const uint32_t* __restrict__ in, uint32_t G, const uint32_t* __restrict__ partial,
                                  uint32_t* __restrict__ out) {
    __shared__ uint32_t warp_sums[kScanThreads / 32];
    const uint32_t base = blockIdx.x * kScanTile;
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    // each thread owns 4 consecutive elements
    uint32_t v[4], s = 0;
#pragma unroll
    for (int q = 0; q < 4; ++q) {
        const uint32_t i = base + threadIdx.x * 4 + q;
        v[q] = i < G ? in[i] : 0u;
        s += v[q];
    }
    uint32_t x = s;
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) warp_sums[w] = x;
    __syncthreads();
    uint32_t wo = 0;
    for (int q = 0; q < w; ++q) wo += warp_sums[q];
    uint32_t run = partial[blockIdx.x] + wo + x - s;
#pragma unroll
    for (int q = 0; q < 4; ++q) {
        const uint32_t i = base + threadIdx.x * 4 + q;
        if (i < G) out[i] = run;
        run += v[q];
        if (i == G - 1) out[G] = run;
    }
}

template <typename T>
__global__ void scatter_kernel(const T* __restrict__ xyz, uint64_t n, const uint32_t* __restrict__ start,
                               const uint32_t* __restrict__ cell, const uint32_t* __restrict__ rank,
                               SPoint<T>* __restrict__ out) {
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
        SPoint<T> p;
        p.x = xyz[3 * i];
        p.y = xyz[3 * i + 1];
        p.z = xyz[3 * i + 2];
        p.idx = (uint32_t)i;
        out[start[cell[i]] + rank[i]] = p;
    }
}

}  // namespace
int exclusive_scan_into(const uint32_t* in, uint32_t G, uint32_t* out, uint32_t* partials, cudaStream_t s);
namespace {

unsigned grid_blocks(uint64_t n, int threads) {
    const DeviceInfo* di = nullptr;
    current_device_info(&di);
    const uint64_t cap = di ? (uint64_t)di->sm_count * 8 : 1024;
    return (unsigned)std::max<uint64_t>(1, std::min<uint64_t>(ceil_div_u(n, threads), cap));
}

int exclusive_scan(const uint32_t* in, uint32_t G, uint32_t* out, cudaStream_t s) {
    const uint32_t nb = ceil_div_u(G, kScanTile);
    Scratch part;
    PGEOF_TRY(part.alloc((size_t)nb * sizeof(uint32_t), s));
    return exclusive_scan_into(in, G, out, part.as<uint32_t>(), s);
}

struct HostBox {
    float mn[3], mx[3];
};

// Cell edges chosen for recent clouds, keyed by size, bounding box and target:
// repeated searches over the same cloud (feature passes at several k, serving
// resident clouds) skip the trial histograms and their host round trips. The
// edge only steers speed; results do not depend on it.
struct EdgeKey {
    uint64_t n;
    uint32_t k;
    float h_min, h_max;
    float box[6];
    bool operator==(const EdgeKey& o) const {
        return n == o.n && k == o.k && h_min == o.h_min && h_max == o.h_max && memcmp(box, o.box, sizeof(box)) == 0;
    }
};
std::mutex g_edge_mu;
// 256 entries: a request server cycles through many clouds (the serving
// stream draws from ~100), and a miss costs two trial histograms with their
// host round trips.
constexpr int kEdgeCache = 256;
EdgeKey g_edge_keys[kEdgeCache];
double g_edge_vals[kEdgeCache];
int g_edge_n = 0, g_edge_next = 0;

bool edge_cache_get(const EdgeKey& k, double& h) {
    std::lock_guard<std::mutex> lk(g_edge_mu);
    for (int i = 0; i < g_edge_n; ++i)
        if (g_edge_keys[i] == k) {
            h = g_edge_vals[i];
            return true;
        }
    return false;
}

void edge_cache_put(const EdgeKey& k, double h) {
    std::lock_guard<std::mutex> lk(g_edge_mu);
    for (int i = 0; i < g_edge_n; ++i)
        if (g_edge_keys[i] == k) {
            g_edge_vals[i] = h;
            return;
        }
    g_edge_keys[g_edge_next] = k;
    g_edge_vals[g_edge_next] = h;
    g_edge_next = (g_edge_next + 1) % kEdgeCache;
    g_edge_n = std::min(g_edge_n + 1, kEdgeCache);
}

// Grid dimensions for edge h (x edge h / xsub), or false when it would
// exceed `cap` cells.
static bool make_params(const HostBox& b, double h, uint64_t cap, GridParams& g, int xsub = 1) {
    uint64_t G = 1;
    int d[3];
    const double hx = h / xsub;
    for (int a = 0; a < 3; ++a) {
        const double ext = (double)b.mx[a] - (double)b.mn[a];
        const double cells = std::floor(ext / (a == 0 ? hx : h)) + 1.0;
        if (cells > 2.0e9) return false;
        d[a] = (int)cells;
        G *= (uint64_t)d[a];
        if (G > cap) return false;
    }
    g.ox = b.mn[0];
    g.oy = b.mn[1];
    g.oz = b.mn[2];
    g.h = (float)h;
    g.inv_h = (float)(1.0 / h);
    g.hx = (float)hx;
    g.inv_hx = (float)(1.0 / hx);
    g.xsub = xsub;
    g.gx = d[0];
    g.gy = d[1];
    g.gz = d[2];
    g.n_cells = (uint32_t)G;
    double maxc = 0.0;
    for (int a = 0; a < 3; ++a) maxc = std::max({maxc, std::fabs((double)b.mn[a]), std::fabs((double)b.mx[a])});
    int ex = 0;
    std::frexp(std::max(maxc, 1e-30), &ex);
    const double ulp = std::ldexp(1.0, ex - 24);
    g.margin = (float)(16.0 * ulp + 1e-5 * h);
    return true;
}

template <typename T>
static int occupancy(const T* xyz, uint64_t n, const GridParams& g, uint32_t* counts, unsigned long long* dsum,
                     double& m_w, cudaStream_t s) {
    PGEOF_CUDA_TRY(cudaMemsetAsync(counts, 0, (size_t)g.n_cells * sizeof(uint32_t), s));
    PGEOF_CUDA_TRY(cudaMemsetAsync(dsum, 0, sizeof(unsigned long long), s));
    KernelTimer kt("grid_occupancy_kernels", s);
    hist_kernel<T><<<grid_blocks(n, 256), 256, 0, s>>>(xyz, n, g, counts, nullptr, nullptr);
    sumsq_kernel<<<grid_blocks(g.n_cells, 256), 256, 0, s>>>(counts, g.n_cells, dsum);
    count_launch(2);
    PGEOF_TRY(check_launch("occupancy"));
    unsigned long long h = 0;
    PGEOF_CUDA_TRY(cudaMemcpyAsync(&h, dsum, sizeof(h), cudaMemcpyDeviceToHost, s));
    PGEOF_CUDA_TRY(cudaStreamSynchronize(s));
    m_w = (double)h / (double)n;
    return PGEOF_OK;
}

}  // namespace

// Exclusive scan of G counts into out[0..G] with caller-owned partials
// (ceil(G / 1024) words): no allocation, so it can be captured in a graph.
int exclusive_scan_into(const uint32_t* in, uint32_t G, uint32_t* out, uint32_t* partials, cudaStream_t s) {
    const uint32_t nb = ceil_div_u(G, kScanTile);
    KernelTimer kt("scan_kernels", s);
    scan_partials_kernel<<<nb, kScanThreads, 0, s>>>(in, G, partials);
    scan_top_kernel<<<1, kScanThreads, 0, s>>>(partials, nb);
    scan_final_kernel<<<nb, kScanThreads, 0, s>>>(in, G, partials, out);
    count_launch(3);
    return check_launch("exclusive_scan");
}

template <typename T>
int build_grid(const T* xyz, uint64_t n, uint32_t k_target, float h_min, float h_max, GridIndex<T>& out,
               cudaStream_t s) {
    out.n = n;
    if (n == 0) return PGEOF_OK;
    if (n >= 0xffffffffull) return fail(PGEOF_ERR_INVALID_ARGUMENT, "point clouds are limited to 2^32-1 points");
    // 1. bounding box
    Scratch misc;
    PGEOF_TRY(misc.alloc(64, s));
    uint32_t* box = misc.as<uint32_t>();
    PGEOF_CUDA_TRY(cudaMemsetAsync(box, 0xff, 3 * sizeof(uint32_t), s));
    PGEOF_CUDA_TRY(cudaMemsetAsync(box + 3, 0, 3 * sizeof(uint32_t), s));
    {
        KernelTimer kt("bbox_kernel", s);
        bbox_kernel<T><<<grid_blocks(n, 256), 256, 0, s>>>(xyz, n, box);
    }
    count_launch();
    PGEOF_TRY(check_launch("bbox_kernel"));
    uint32_t hb[6];
    PGEOF_CUDA_TRY(cudaMemcpyAsync(hb, box, sizeof(hb), cudaMemcpyDeviceToHost, s));
    PGEOF_CUDA_TRY(cudaStreamSynchronize(s));
    HostBox b;
    for (int a = 0; a < 3; ++a) {
        b.mn[a] = ord_decode(hb[a]);
        b.mx[a] = ord_decode(hb[3 + a]);
        if (!(b.mn[a] <= b.mx[a]) || !std::isfinite(b.mn[a]) || !std::isfinite(b.mx[a]))
            return fail(PGEOF_ERR_INVALID_ARGUMENT, "point coordinates must be finite");
    }
    // 2. cell edge
    double ext_max = 1e-30;
    for (int a = 0; a < 3; ++a) ext_max = std::max(ext_max, (double)b.mx[a] - (double)b.mn[a]);
    double vol = 1.0;
    for (int a = 0; a < 3; ++a) vol *= std::max((double)b.mx[a] - (double)b.mn[a], ext_max * 1e-3);
    // Occupancy target (points per cell, point-weighted): k / 3.5 for clouds of
    // surfaces, finer cells for volume-filling clouds -- on a uniform cube
    // k / 12 is 19% faster at k = 50 than k / 3.5, on an outdoor scene of
    // walls and ground k / 3.5 is best. The dimension comes from two trial
    // histograms: (occupancy - 1) scales as h^dim (the 1 is the point itself).
    const double target2 = std::min(48.0, std::max(2.0, (double)k_target / 3.5));
    const uint64_t cap = std::max<uint64_t>(4 * n, 1u << 16);
    const double hmin = h_min > 0 ? (double)h_min : 0.0;
    const double hmax = h_max > 0 ? (double)h_max : 1e300;
    auto clamp_h = [&](double h) {
        h = std::min(std::max(h, hmin), hmax);
        h = std::max(h, ext_max * 1e-7 + 1e-30);
        // respect the cell cap
        GridParams g;
        while (!make_params(b, h, cap, g)) h *= 1.25;
        return h;
    };
    double h0 = clamp_h(std::cbrt(vol * target2 / (double)n));
    double h = h0;
    EdgeKey key{n, k_target, h_min, h_max, {b.mn[0], b.mn[1], b.mn[2], b.mx[0], b.mx[1], b.mx[2]}};
    double cached = 0.0;
    if (edge_cache_get(key, cached)) {
        h = cached;
    } else if (n > 64) {
        GridParams g;
        make_params(b, h0, cap, g);
        Scratch cnt;
        PGEOF_TRY(cnt.alloc((size_t)cap * sizeof(uint32_t), s));
        unsigned long long* acc = reinterpret_cast<unsigned long long*>(box + 8);
        double m0 = 0.0;
        PGEOF_TRY(occupancy<T>(xyz, n, g, cnt.as<uint32_t>(), acc, m0, s));
        // surfaces: move towards target2 until a trial lands within 60% of it
        double h1 = h0, m1 = 0.0;
        if (!(m0 > target2 / 1.6 && m0 < target2 * 1.6) && m0 > 0.0) {
            h1 = clamp_h(h0 * std::min(16.0, std::max(1.0 / 16.0, std::sqrt(target2 / m0))));
            if (h1 != h0) {
                make_params(b, h1, cap, g);
                PGEOF_TRY(occupancy<T>(xyz, n, g, cnt.as<uint32_t>(), acc, m1, s));
                h = h1;
                if (!(m1 > target2 / 1.6 && m1 < target2 * 1.6) && m1 > 0.0 && m0 != m1) {
                    double dim = std::log(m0 / m1) / std::log(h0 / h1);
                    if (!std::isfinite(dim)) dim = 2.0;
                    dim = std::min(3.0, std::max(1.0, dim));
                    h = clamp_h(h1 * std::pow(target2 / m1, 1.0 / dim));
                }
            }
        } else if (m0 > 0.0) {
            // on target at the first trial: a half-edge trial for the dimension
            h1 = clamp_h(h0 * 0.5);
            if (h1 != h0) {
                make_params(b, h1, cap, g);
                PGEOF_TRY(occupancy<T>(xyz, n, g, cnt.as<uint32_t>(), acc, m1, s));
            }
        }
        // volume-filling clouds: finer cells, placed by (m - 1) ~ h^dim
        if (m0 > 1.05 && m1 > 1.05 && h1 != h0) {
            double dim = std::log((m0 - 1.0) / (m1 - 1.0)) / std::log(h0 / h1);
            if (!std::isfinite(dim)) dim = 2.0;
            dim = std::min(3.0, std::max(1.0, dim));
            const double w = std::min(1.0, std::max(0.0, (dim - 2.3) / 0.6));
            if (w > 0.0) {
                const double target = std::min(48.0, std::max(2.0, (double)k_target / (3.5 + 8.5 * w)));
                const bool use1 = std::fabs(std::log(m1 / target)) < std::fabs(std::log(m0 / target));
                const double hr = use1 ? h1 : h0, mr = use1 ? m1 : m0;
                h = clamp_h(hr * std::pow((target - 1.0) / (mr - 1.0), 1.0 / dim));
            }
        }
    }
    edge_cache_put(key, h);
    // the final grid splits cells along x (see GridParams) while the cell
    // table stays within 8 entries per point
    GridParams g;
    make_params(b, h, cap, g);
    static const int xsub_max = [] {
        const char* e = getenv("PGEOF_GRID_XSUB");
        const int v = e ? atoi(e) : 4;
        return v < 1 ? 1 : (v > 16 ? 16 : v);
    }();
    const uint64_t cap_fine = std::max<uint64_t>(8 * n, 1u << 16);
    for (int xs = xsub_max; xs > 1; xs /= 2) {
        GridParams gf;
        if (make_params(b, h, cap_fine, gf, xs)) {
            g = gf;
            break;
        }
    }
    out.g = g;
    // 3. counting sort into cells
    PGEOF_TRY(out.cell_mem.alloc(((size_t)g.n_cells + 1) * sizeof(uint32_t), s));
    PGEOF_TRY(out.pts_mem.alloc((size_t)n * sizeof(SPoint<T>), s));
    out.cell_start = out.cell_mem.template as<uint32_t>();
    out.pts = out.pts_mem.template as<SPoint<T>>();
    Scratch counts, cell, rank;
    PGEOF_TRY(counts.alloc((size_t)g.n_cells * sizeof(uint32_t), s));
    PGEOF_TRY(cell.alloc((size_t)n * sizeof(uint32_t), s));
    PGEOF_TRY(rank.alloc((size_t)n * sizeof(uint32_t), s));
    PGEOF_CUDA_TRY(cudaMemsetAsync(counts.p, 0, (size_t)g.n_cells * sizeof(uint32_t), s));
    {
        KernelTimer kt("hist_kernel", s);
        hist_kernel<T><<<grid_blocks(n, 256), 256, 0, s>>>(xyz, n, g, counts.as<uint32_t>(), cell.as<uint32_t>(),
                                                            rank.as<uint32_t>());
    }
    count_launch();
    PGEOF_TRY(check_launch("hist_kernel"));
    PGEOF_TRY(exclusive_scan(counts.as<uint32_t>(), g.n_cells, out.cell_start, s));
    KernelTimer kt("scatter_kernel", s);
    scatter_kernel<T><<<grid_blocks(n, 256), 256, 0, s>>>(xyz, n, out.cell_start, cell.as<uint32_t>(),
                                                           rank.as<uint32_t>(), out.pts);
    count_launch();
    return check_launch("scatter_kernel");
}

template <typename T>
int sort_queries(const T* q, uint64_t m, const GridParams& g, Scratch& out_mem, SPoint<T>** out, Scratch& start,
                 cudaStream_t s) {
    *out = nullptr;
    if (m == 0) return PGEOF_OK;
    PGEOF_TRY(out_mem.alloc((size_t)m * sizeof(SPoint<T>), s));
    Scratch counts, cell, rank;
    PGEOF_TRY(counts.alloc((size_t)g.n_cells * sizeof(uint32_t), s));
    PGEOF_TRY(start.alloc(((size_t)g.n_cells + 1) * sizeof(uint32_t), s));
    PGEOF_TRY(cell.alloc((size_t)m * sizeof(uint32_t), s));
    PGEOF_TRY(rank.alloc((size_t)m * sizeof(uint32_t), s));
    PGEOF_CUDA_TRY(cudaMemsetAsync(counts.p, 0, (size_t)g.n_cells * sizeof(uint32_t), s));
    {
        KernelTimer kt("query_hist_kernel", s);
        hist_kernel<T><<<grid_blocks(m, 256), 256, 0, s>>>(q, m, g, counts.as<uint32_t>(), cell.as<uint32_t>(),
                                                            rank.as<uint32_t>());
    }
    count_launch();
    PGEOF_TRY(check_launch("hist_kernel(queries)"));
    PGEOF_TRY(exclusive_scan(counts.as<uint32_t>(), g.n_cells, start.as<uint32_t>(), s));
    KernelTimer kt("query_scatter_kernel", s);
    scatter_kernel<T><<<grid_blocks(m, 256), 256, 0, s>>>(q, m, start.as<uint32_t>(), cell.as<uint32_t>(),
                                                           rank.as<uint32_t>(), out_mem.as<SPoint<T>>());
    count_launch();
    *out = out_mem.as<SPoint<T>>();
    return check_launch("scatter_kernel(queries)");
}

template int build_grid<float>(const float*, uint64_t, uint32_t, float, float, GridIndex<float>&, cudaStream_t);
template int build_grid<double>(const double*, uint64_t, uint32_t, float, float, GridIndex<double>&, cudaStream_t);
template int sort_queries<float>(const float*, uint64_t, const GridParams&, Scratch&, SPoint<float>**, Scratch&,
                                 cudaStream_t);
template int sort_queries<double>(const double*, uint64_t, const GridParams&, Scratch&, SPoint<double>**, Scratch&,
                                  cudaStream_t);

}  // namespace pgeof
