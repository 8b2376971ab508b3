// search.cu -- exact k-nearest / radius neighbour search over the grid index
// (include/nn_search.hpp:31-132) and the radius-search + PCA path of
// compute_features_selected (include/pgeof.hpp:325-375).
//
// Candidates of a query are streamed as contiguous runs of the cell-ordered
// point array: every row of cells (fixed y, z; a range of x) is one run, and
// runs are packed across the 32 lanes so no lane idles at row ends. Distances
// use nanoflann's metric_L2_Simple arithmetic -- (q - p)^2 per axis, summed x,
// y, z, each operation rounded (no FMA) -- so values are bit-identical to the
// reference's. Results are the exact smallest (d^2, index) pairs: ties at equal
// distance order by index (nanoflann keeps its tree-traversal order there).
//
// Two kernels:
//  * fast_search_kernel (float, k <= 128): a warp takes chunks of 16
//    consecutive queries in cell order. One pass over the cells within a bound
//    tau of the query appends every point with d^2 <= tau^2 to a shared-memory
//    buffer; selection then runs in shared memory (64-bin distance histogram,
//    counting-sort scatter of the bins up to the k-th, insertion sort inside the
//    few-entry bins). For kNN, tau comes from the queries the warp solved last
//    (one per lane): d_k(p) + |q - p| / 2 minimised over the lanes, an
//    optimistic form of the triangle inequality d_k(q) <= d_k(p) + |q - p| that
//    is exact whenever it holds >= k points; only the first query of a chunk
//    needs a pilot pass; radius search uses tau = r. Queries whose buffer
//    overflows or whose radius fell short go to a list: a second fast pass with
//    pilot bounds, then the general kernel.
//  * search_kernel (float and double, any k): the general path. A pilot pass
//    histograms a block of cells holding >= k points to bound the k-th distance,
//    then passes over the cells within that bound refine a window of bins (first
//    on d^2, then on the index when distances tie exactly) until the survivors
//    fit the buffer.
//
// compute_features_selected runs inside the radius search (SEL instantiations):
// instead of writing a query's row, a warp parks its sorted neighbour indices
// in shared memory; once `ring` queries are parked, each lane takes one of
// them through the reference's two-pass covariance, the eigen solver and the
// selected features (thread-level work, done by the whole warp at once). No
// neighbour table reaches global memory.
#include <algorithm>
#include <cstdlib>

#include "eig3.cuh"
#include "kernels.cuh"

namespace pgeof {

namespace {

constexpr unsigned FULL = 0xffffffffu;
constexpr int kSearchWarps = 4;
constexpr int kMaxLevels = 40;

template <typename T>
struct Bits;
template <>
struct Bits<float> {
    using U = uint32_t;
    static __device__ __forceinline__ U of(float x) { return __float_as_uint(x); }
    static __device__ __forceinline__ float val(U u) { return __uint_as_float(u); }
    static constexpr U kMax = 0xffffffffu;
};
template <>
struct Bits<double> {
    using U = unsigned long long;
    static __device__ __forceinline__ U of(double x) { return (U)__double_as_longlong(x); }
    static __device__ __forceinline__ double val(U u) { return __longlong_as_double((long long)u); }
    static constexpr U kMax = 0xffffffffffffffffull;
};

template <typename T>
struct Entry {
    T d2;
    uint32_t idx;
};

template <typename T>
__device__ __forceinline__ bool entry_less(const Entry<T>& a, const Entry<T>& b) {
    return a.d2 < b.d2 || (a.d2 == b.d2 && a.idx < b.idx);
}

// One refinement level: candidates whose bin under (type, lo, scale / shift)
// is below `b` are kept for sure, above are dropped, equal go deeper.
template <typename T>
struct Level {
    T lo, scale;
    uint32_t ilo;
    int shift;
    int type;  // 0: bins on d^2 in [lo, lo + 32/scale], 1: bins on the index
    int b;
};

template <typename T>
struct WarpSmem {
    uint32_t hist[32];
    typename Bits<T>::U dmin[32], dmax[32];
    uint32_t imin[32], imax[32];
    uint32_t run_start[32], run_len[32];
    Level<T> lev[kMaxLevels];
};

template <typename T>
struct GridView {
    GridParams g;
    const uint32_t* cell_start;
    const SPoint<T>* pts;
};

template <typename T>
struct SearchArgs {
    GridView<T> gv;
    CloudTable ct;
    const SPoint<T>* queries;
    uint64_t m;
    const uint32_t* qlist;   // optional: positions in `queries` to process
    const uint32_t* qcount;  // with qlist: number of entries (device)
    int mode;
    uint32_t k;
    T r2;
    uint32_t cap;
    int buf_in_smem;
    Entry<T>* gbuf;
    void* out_idx;
    T* out_d2;
    uint32_t* out_found;
    int fill_last;
    int rows_sorted;  // output row = position in `queries`
    uint32_t* err;
    SelSpec<T> sel;   // SEL instantiations
};

struct Box {
    int lo[3], hi[3];
};

__device__ __forceinline__ int cell_floor(float v, int gdim) {
    // floor(v) clamped to [-1, gdim] before the int conversion
    return (int)floorf(fminf(fmaxf(v, -1.0f), (float)gdim));
}

template <typename T>
__device__ __forceinline__ T dist2(const T (&q)[3], const SPoint<T>& p) {
    using O = XOps<T>;
    const T tx = O::sub(q[0], p.x);
    const T ty = O::sub(q[1], p.y);
    const T tz = O::sub(q[2], p.z);
    T d = O::mul(tx, tx);
    d = O::add(d, O::mul(ty, ty));
    d = O::add(d, O::mul(tz, tz));
    return d;
}

// distance from coordinate v to cell c's interval along one axis, shrunk by
// the index margin (never overestimates)
__device__ __forceinline__ float axis_gap(float v, int c, float o, float h, float margin) {
    const float lo = o + (float)c * h, hi = o + (float)(c + 1) * h;
    const float gap = fmaxf(0.0f, fmaxf(lo - v, v - hi));
    return fmaxf(0.0f, gap - margin);
}

// Visit every point of the cells in `bx` (rows clipped to the sphere of radius
// Rf around q when prune). All lanes call visit(valid, d2, idx) together.
// U > 1 loads U batches of 32 points before visiting them (U loads in flight
// per lane: for the few, large queries of the list passes, whose warps
// otherwise wait on one load at a time; 1M-point scene, k = 50: both list
// passes 0.131 ms with U = 1, 0.110 ms with U = 4, 0.113 ms with U = 8).
template <typename T, typename F, int U = 1>
__device__ __forceinline__ void visit_box(const GridView<T>& gv, uint32_t* run_start, uint32_t* run_len,
                                          const T (&q)[3], const Box& bx, bool prune, float Rf, F&& visit) {
    const GridParams& g = gv.g;
    const int lane = threadIdx.x & 31;
    const int ny = bx.hi[1] - bx.lo[1] + 1, nz = bx.hi[2] - bx.lo[2] + 1;
    if (ny <= 0 || nz <= 0 || bx.hi[0] < bx.lo[0]) return;
    const int R = ny * nz;
    const float qf0 = (float)q[0], qf1 = (float)q[1], qf2 = (float)q[2];
    const float Rf2 = Rf * Rf;
    for (int rg = 0; rg < R; rg += 32) {
        const int row = rg + lane;
        uint32_t st = 0, len = 0;
        if (row < R) {
            const int cy = bx.lo[1] + row % ny, cz = bx.lo[2] + row / ny;
            int xa = bx.lo[0], xb = bx.hi[0];
            bool keep = true;
            if (prune) {
                const float gy = axis_gap(qf1, cy, g.oy, g.h, g.margin);
                const float gz = axis_gap(qf2, cz, g.oz, g.h, g.margin);
                const float dyz2 = gy * gy + gz * gz;
                if (dyz2 > Rf2) {
                    keep = false;
                } else {
                    const float bxr = sqrtf(Rf2 - dyz2) + g.margin;
                    xa = max(xa, cell_floor((qf0 - bxr - g.ox) * g.inv_hx, g.gx));
                    xb = min(xb, cell_floor((qf0 + bxr - g.ox) * g.inv_hx, g.gx));
                }
            }
            if (keep && xa <= xb) {
                const uint32_t base = ((uint32_t)cz * (uint32_t)g.gy + (uint32_t)cy) * (uint32_t)g.gx;
                st = __ldg(gv.cell_start + base + xa);
                len = __ldg(gv.cell_start + base + xb + 1) - st;
            }
        }
        // pack the non-empty runs into lanes 0..nrows-1
        const uint32_t ne = __ballot_sync(FULL, len > 0);
        const int nrows = __popc(ne);
        if (nrows == 0) continue;
        if (len > 0) {
            const int ci = __popc(ne & ((1u << lane) - 1u));
            run_start[ci] = st;
            run_len[ci] = len;
        }
        __syncwarp();
        const uint32_t c_st = lane < nrows ? run_start[lane] : 0u;
        const uint32_t c_len = lane < nrows ? run_len[lane] : 0u;
        __syncwarp();
        uint32_t incl = c_len;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t y = __shfl_up_sync(FULL, incl, o);
            if (lane >= o) incl += y;
        }
        const uint32_t excl = incl - c_len;
        const uint32_t total = __shfl_sync(FULL, incl, 31);
        int r_base = 0;
        if constexpr (U > 1) {
            for (uint32_t base0 = 0; base0 < total; base0 += 32 * U) {
                SPoint<T> p[U];
                bool valid[U];
#pragma unroll
                for (int u = 0; u < U; ++u) {
                    const uint32_t base = base0 + 32u * u;
                    const uint32_t bit =
                        (lane < nrows && excl > base && excl < base + 32) ? (1u << (excl - base)) : 0u;
                    const uint32_t M = __reduce_or_sync(FULL, bit);
                    const int r = r_base + __popc(M & (0xffffffffu >> (31 - lane)));
                    const uint32_t pos = base + lane;
                    valid[u] = pos < total;
                    const uint32_t r_st = __shfl_sync(FULL, c_st, r);
                    const uint32_t r_ex = __shfl_sync(FULL, excl, r);
                    if (valid[u]) p[u] = gv.pts[r_st + (pos - r_ex)];
                    r_base = __popc(__ballot_sync(FULL, lane < nrows && excl <= base + 32)) - 1;
                }
#pragma unroll
                for (int u = 0; u < U; ++u) {
                    T d2 = T(0);
                    uint32_t idx = 0;
                    if (valid[u]) {
                        d2 = dist2<T>(q, p[u]);
                        idx = p[u].idx;
                    }
                    visit(valid[u], d2, idx);
                }
            }
            continue;
        }
        for (uint32_t base = 0; base < total; base += 32) {
            const uint32_t bit = (lane < nrows && excl > base && excl < base + 32) ? (1u << (excl - base)) : 0u;
            const uint32_t M = __reduce_or_sync(FULL, bit);
            const int r = r_base + __popc(M & (0xffffffffu >> (31 - lane)));
            const uint32_t pos = base + lane;
            const bool valid = pos < total;
            const uint32_t r_st = __shfl_sync(FULL, c_st, r);
            const uint32_t r_ex = __shfl_sync(FULL, excl, r);
            T d2 = T(0);
            uint32_t idx = 0;
            if (valid) {
                const SPoint<T> p = gv.pts[r_st + (pos - r_ex)];
                d2 = dist2<T>(q, p);
                idx = p.idx;
            }
            visit(valid, d2, idx);
            r_base = __popc(__ballot_sync(FULL, lane < nrows && excl <= base + 32)) - 1;
        }
    }
}

template <typename T>
__device__ __forceinline__ T warp_max(T v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = max(v, __shfl_xor_sync(FULL, v, o));
    return v;
}

__device__ __forceinline__ void query_cell(const GridParams& g, float x, float y, float z, int (&cq)[3]) {
    const float v[3] = {x, y, z};
    const float o[3] = {g.ox, g.oy, g.oz};
    const int gd[3] = {g.gx, g.gy, g.gz};
    const float inv[3] = {g.inv_hx, g.inv_h, g.inv_h};
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        const float c = (v[d] - o[d]) * inv[d];
        cq[d] = (int)floorf(fminf(fmaxf(c, 0.0f), (float)(gd[d] - 1)));
    }
}

// Pilot bound on the k-th neighbour distance: grow a block of cells around
// the query until it holds >= k points (cell counts only), then a 32-bin
// histogram of the block's squared distances gives tau^2 >= d_k^2.
template <typename T, int U = 1>
__device__ __forceinline__ T pilot_tau2(const GridView<T>& gv, uint32_t* hist32, uint32_t* run_start,
                                        uint32_t* run_len, const T (&q)[3], uint32_t k) {
    const GridParams& g = gv.g;
    const int lane = threadIdx.x & 31;
    const int gd[3] = {g.gx, g.gy, g.gz};
    const float go[3] = {g.ox, g.oy, g.oz};
    int cq[3];
    query_cell(g, (float)q[0], (float)q[1], (float)q[2], cq);
    Box bx;
    for (int r = 0;; ++r) {
        bool full = true;
#pragma unroll
        for (int d = 0; d < 3; ++d) {
            const int rd = d == 0 ? r * g.xsub + (g.xsub - 1) / 2 : r;  // the same extent in metres on every axis
            bx.lo[d] = max(0, cq[d] - rd);
            bx.hi[d] = min(gd[d] - 1, cq[d] + rd);
            full = full && bx.lo[d] == 0 && bx.hi[d] == gd[d] - 1;
        }
        const int ny = bx.hi[1] - bx.lo[1] + 1, nz = bx.hi[2] - bx.lo[2] + 1;
        uint32_t cnt = 0;
        for (int row = lane; row < ny * nz; row += 32) {
            const int cy = bx.lo[1] + row % ny, cz = bx.lo[2] + row / ny;
            const uint32_t base = ((uint32_t)cz * (uint32_t)g.gy + (uint32_t)cy) * (uint32_t)g.gx;
            cnt += __ldg(gv.cell_start + base + bx.hi[0] + 1) - __ldg(gv.cell_start + base + bx.lo[0]);
        }
        cnt = __reduce_add_sync(FULL, cnt);
        if (cnt >= k || full) break;
    }
    float F2 = 0.0f;
    const float hd[3] = {g.hx, g.h, g.h};
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        const float lo = go[d] + (float)bx.lo[d] * hd[d], hi = go[d] + (float)(bx.hi[d] + 1) * hd[d];
        const float far = fmaxf((float)q[d] - lo, hi - (float)q[d]) + g.margin;
        F2 += far * far;
    }
    const float sb = 32.0f / fmaxf(F2, 1e-30f);
    hist32[lane] = 0;
    __syncwarp();
    T dmax = T(0);
    const auto hist = [&](bool valid, T d2, uint32_t) {
        if (valid) {
            const float x = (float)d2 * sb;
            const int bin = x >= 31.0f ? 31 : (int)x;
            atomicAdd(&hist32[bin], 1u);
            dmax = max(dmax, d2);
        }
    };
    visit_box<T, decltype(hist)&, U>(gv, run_start, run_len, q, bx, false, 0.0f, hist);
    __syncwarp();
    dmax = warp_max(dmax);
    uint32_t incl = hist32[lane];
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t y = __shfl_up_sync(FULL, incl, o);
        if (lane >= o) incl += y;
    }
    __syncwarp();
    const uint32_t reach = __ballot_sync(FULL, incl >= k);
    const int b = reach ? __ffs(reach) - 1 : 31;
    T tau2 = dmax;
    if (b < 31) tau2 = min(dmax, (T)(((float)(b + 1) / sb) * 1.000004f));
    return tau2;
}

// Cells within distance tf of q (a conservative box).
__device__ __forceinline__ Box region_box(const GridParams& g, float qx, float qy, float qz, float tf) {
    const float v[3] = {qx, qy, qz};
    const float o[3] = {g.ox, g.oy, g.oz};
    const int gd[3] = {g.gx, g.gy, g.gz};
    const float inv[3] = {g.inv_hx, g.inv_h, g.inv_h};
    Box rb;
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        rb.lo[d] = max(0, cell_floor((v[d] - tf - o[d]) * inv[d], gd[d]));
        rb.hi[d] = min(gd[d] - 1, cell_floor((v[d] + tf - o[d]) * inv[d], gd[d]));
    }
    return rb;
}

template <typename T>
__device__ __forceinline__ int level_bin(const Level<T>& L, T d2, uint32_t idx) {
    if (L.type == 0) {
        const T x = (d2 - L.lo) * L.scale;
        return x >= T(31) ? 31 : (x <= T(0) ? 0 : (int)x);
    }
    return (int)min(31u, (idx - L.ilo) >> L.shift);
}

// 0 below, 1 inside the current window, 2 above
template <typename T>
__device__ __forceinline__ int classify(const WarpSmem<T>* ws, int nlev, T d2, uint32_t idx) {
    for (int l = 0; l < nlev; ++l) {
        const Level<T>& L = ws->lev[l];
        const int bin = level_bin(L, d2, idx);
        if (bin < L.b) return 0;
        if (bin > L.b) return 2;
    }
    return 1;
}

template <typename T>
__device__ __forceinline__ void bitonic_sort(Entry<T>* buf, int n, int P) {
    const int lane = threadIdx.x & 31;
    // padding sorts after every real entry: (+inf, 0xffffffff)
    for (int i = n + lane; i < P; i += 32) {
        buf[i].d2 = T(INFINITY);
        buf[i].idx = 0xffffffffu;
    }
    __syncwarp();
    for (int size = 2; size <= P; size <<= 1) {
        for (int stride = size >> 1; stride > 0; stride >>= 1) {
            for (int t = lane; t < P / 2; t += 32) {
                const int i = 2 * stride * (t / stride) + (t % stride);
                const int j = i + stride;
                const bool up = (i & size) == 0;
                const Entry<T> x = buf[i], y = buf[j];
                if (entry_less(y, x) == up) {
                    buf[i] = y;
                    buf[j] = x;
                }
            }
            __syncwarp();
        }
    }
}

// Write one query's result row (knn: k entries; radius: -1 / 0 padding and
// nanoflann's radius^2 in the last slot of a short row).
template <typename T, typename GetEntry>
__device__ __forceinline__ void emit_row(int mode, uint32_t k, uint32_t n_sel, uint32_t found, uint64_t qo,
                                         void* out_idx, T* out_d2, uint32_t* out_found, int fill_last, T r2,
                                         GetEntry&& get) {
    const int lane = threadIdx.x & 31;
    if (mode == MODE_KNN) {
        uint32_t* oi = static_cast<uint32_t*>(out_idx) + qo * k;
        T* od = out_d2 ? out_d2 + qo * k : nullptr;
        for (uint32_t j = lane; j < k; j += 32) {
            const Entry<T> e = get(j);
            oi[j] = e.idx;
            if (od) od[j] = e.d2;
        }
    } else {
        const uint32_t nk = min(n_sel, k);
        int32_t* oi = static_cast<int32_t*>(out_idx) + qo * k;
        T* od = out_d2 ? out_d2 + qo * k : nullptr;
        for (uint32_t j = lane; j < k; j += 32) {
            if (j < nk) {
                const Entry<T> e = get(j);
                oi[j] = (int32_t)e.idx;
                if (od) od[j] = e.d2;
            } else {
                oi[j] = -1;
                if (od) od[j] = (fill_last && j == k - 1) ? r2 : T(0);
            }
        }
        if (out_found && lane == 0) out_found[qo] = found;
    }
}

// ------------------------------------------------------------------ fused selected
template <typename T>
__device__ __forceinline__ void solve(const Cov<T>& c, int order, Pca<T>& p);
template <>
__device__ __forceinline__ void solve<float>(const Cov<float>& c, int order, Pca<float>& p) {
    bool res;
    pca_solve_f32(c, order, p, res);
}
template <>
__device__ __forceinline__ void solve<double>(const Cov<double>& c, int order, Pca<double>& p) {
    pca_solve_f64<double>(c, order, &p);
}

// A warp's parking area for selected-feature queries: the sorted neighbour
// indices of up to `ring` queries, stored [j][slot] with rows of ring + 1 words
// (writing one query's column and reading one lane's column are both free of
// bank conflicts), plus their uncapped counts and output rows.
struct SelRing {
    uint32_t* idx;    // [max(max_knn, 1)][ring + 1]
    uint32_t* found;  // [ring]
    uint32_t* row;    // [ring]
    int n;            // parked queries (warp-uniform)
};

__device__ __forceinline__ SelRing sel_ring_at(unsigned char* base, uint32_t max_knn, int ring) {
    SelRing r;
    r.idx = reinterpret_cast<uint32_t*>(base);
    r.found = r.idx + (size_t)(max_knn > 0 ? max_knn : 1) * (ring + 1);
    r.row = r.found + ring;
    r.n = 0;
    return r;
}

__device__ __forceinline__ void sel_point(const SelSpec<float>& sp, uint32_t id, float& x, float& y, float& z) {
    const float4 p = __ldg(sp.xyz4 + id);
    x = p.x;
    y = p.y;
    z = p.z;
}
__device__ __forceinline__ void sel_point(const SelSpec<double>& sp, uint32_t id, double& x, double& y, double& z) {
    x = __ldg(sp.xyz + 3 * (uint64_t)id);
    y = __ldg(sp.xyz + 3 * (uint64_t)id + 1);
    z = __ldg(sp.xyz + 3 * (uint64_t)id + 2);
}

// include/pgeof.hpp:354-369 for one parked query, on one lane: fewer than 2
// points in the radius -> zeros; otherwise the PCA of the nearest
// min(found, max_knn) in (distance, index) order -- two sequential sweeps, the
// operation order of include/pca.hpp:75-76 -- and the selected features.
// `idx` is the query's column of the parking area (entries `stride` apart).
template <typename T>
__device__ __noinline__ void sel_solve(const SelSpec<T>& sp, const uint32_t* idx, int stride, uint32_t found,
                                       uint32_t row) {
    using O = XOps<T>;
    T* o = sp.out + (uint64_t)row * sp.out_stride + sp.id_offset;
    if (found < 2) {
        for (int t = 0; t < sp.n_ids; ++t) o[t] = T(0);
        return;
    }
    const uint32_t k = min(found, sp.max_knn);
    T sx = 0, sy = 0, sz = 0;
#pragma unroll 4
    for (uint32_t j = 0; j < k; ++j) {
        T x, y, z;
        sel_point(sp, idx[(size_t)j * stride], x, y, z);
        sx = O::add(sx, x);
        sy = O::add(sy, y);
        sz = O::add(sz, z);
    }
    const T kk = (T)k;
    const T mx = O::div(sx, kk), my = O::div(sy, kk), mz = O::div(sz, kk);
    T xx = 0, xy = 0, xz = 0, yy = 0, yz = 0, zz = 0;
#pragma unroll 4
    for (uint32_t j = 0; j < k; ++j) {
        T x, y, z;
        sel_point(sp, idx[(size_t)j * stride], x, y, z);
        const T dx = O::sub(x, mx), dy = O::sub(y, my), dz = O::sub(z, mz);
        xx = O::add(xx, O::mul(dx, dx));
        xy = O::add(xy, O::mul(dx, dy));
        xz = O::add(xz, O::mul(dx, dz));
        yy = O::add(yy, O::mul(dy, dy));
        yz = O::add(yz, O::mul(dy, dz));
        zz = O::add(zz, O::mul(dz, dz));
    }
    Cov<T> c;
    c.xx = O::div(xx, kk);
    c.xy = O::div(xy, kk);
    c.xz = O::div(xz, kk);
    c.yy = O::div(yy, kk);
    c.yz = O::div(yz, kk);
    c.zz = O::div(zz, kk);
    Pca<T> p;
    solve<T>(c, sp.order, p);
    for (int t = 0; t < sp.n_ids; ++t) {
        T v = T(0);
        if (!selected_feature<T>(p, sp.ids[t], v)) v = T(0);
        o[t] = v;
    }
}

// Every lane takes one parked query (warp-wide call).
template <typename T>
__device__ __forceinline__ void sel_flush(const SelSpec<T>& sp, SelRing& rg) {
    const int lane = threadIdx.x & 31;
    __syncwarp();
    if (lane < rg.n) sel_solve<T>(sp, rg.idx + lane, sp.ring + 1, rg.found[lane], rg.row[lane]);
    __syncwarp();
    rg.n = 0;
}

// After the warps' loops (block-wide call): the queries still parked in the
// block's rings are solved one per thread, so the block's leftovers take
// ceil(total / 32) warps of solver instructions rather than every warp's
// partly filled one -- small clouds leave a few queries in every ring, and
// the solver's float64 instructions cost the same per warp whatever the
// number of active lanes.
template <typename T>
__device__ __forceinline__ void sel_flush_block(const SelSpec<T>& sp, SelRing& rg, unsigned char* ring_base,
                                                int n_warps) {
    __shared__ int parked[32];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    if (lane == 0) parked[w] = rg.n;
    __syncthreads();
    int t = threadIdx.x, ww = 0;
    while (ww < n_warps && t >= parked[ww]) {
        t -= parked[ww];
        ++ww;
    }
    if (ww < n_warps) {
        const SelRing r = sel_ring_at(ring_base + ww * sel_ring_bytes(sp.max_knn, sp.ring), sp.max_knn, sp.ring);
        sel_solve<T>(sp, r.idx + t, sp.ring + 1, r.found[t], r.row[t]);
    }
    rg.n = 0;
}

// Park one query (warp-wide call): its n_sel sorted entries (get(j)), its
// uncapped count and its output row; solve the parked queries once `ring` wait.
template <typename T, typename GetEntry>
__device__ __forceinline__ void sel_push(const SelSpec<T>& sp, SelRing& rg, uint32_t found, uint32_t n_sel,
                                         uint64_t row, GetEntry&& get) {
    const int lane = threadIdx.x & 31;
    const int stride = sp.ring + 1;
    const uint32_t k = min(n_sel, sp.max_knn);
    for (uint32_t j = lane; j < k; j += 32) rg.idx[(size_t)j * stride + rg.n] = get(j).idx;
    if (lane == 0) {
        rg.found[rg.n] = found;
        rg.row[rg.n] = (uint32_t)row;
    }
    ++rg.n;
    if (rg.n == sp.ring) sel_flush<T>(sp, rg);
}

// ------------------------------------------------------------------ general
template <typename T, bool SEL>
__global__ void __launch_bounds__(kSearchWarps * 32) search_kernel(const __grid_constant__ SearchArgs<T> a) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    WarpSmem<T>* ws = reinterpret_cast<WarpSmem<T>*>(smem_raw) + wib;
    Entry<T>* buf = a.buf_in_smem
                        ? reinterpret_cast<Entry<T>*>(smem_raw + kSearchWarps * sizeof(WarpSmem<T>)) + (size_t)wib * a.cap
                        : a.gbuf + ((size_t)blockIdx.x * kSearchWarps + wib) * a.cap;
    const uint64_t nwarps = (uint64_t)gridDim.x * kSearchWarps;
    const uint64_t m = a.qlist ? (uint64_t)*a.qcount : a.m;
    SelRing rg{};
    unsigned char* ring_base = smem_raw + kSearchWarps * sizeof(WarpSmem<T>) +
                               (a.buf_in_smem ? (size_t)kSearchWarps * a.cap * sizeof(Entry<T>) : 0);
    if constexpr (SEL) {
        rg = sel_ring_at(ring_base + wib * sel_ring_bytes(a.sel.max_knn, a.sel.ring), a.sel.max_knn, a.sel.ring);
    }

    for (uint64_t qi = (uint64_t)blockIdx.x * kSearchWarps + wib; qi < m; qi += nwarps) {
        const uint64_t qpos = a.qlist ? a.qlist[qi] : qi;
        const SPoint<T> qp = a.queries[qpos];
        GridView<T> gv = a.gv;
        uint64_t row_base = 0;
        if (a.ct.n) {
            const int ci = cloud_of(a.ct, qpos);
            gv.g = a.ct.g[ci];
            gv.cell_start = a.gv.cell_start + a.ct.cell_base[ci];
            row_base = a.ct.off[ci];
        }
        const GridParams& g = gv.g;
        const T q[3] = {qp.x, qp.y, qp.z};
        const uint32_t k = a.k;
        T tau2;
        bool strict;
        if (a.mode == MODE_KNN) {
            tau2 = pilot_tau2<T>(gv, ws->hist, ws->run_start, ws->run_len, q, k);
            strict = false;
        } else {
            tau2 = a.r2;
            strict = true;
        }
        // collect every point within tau (refining when the buffer overflows)
        const float tf = sqrtf((float)tau2) * 1.000001f + g.margin;
        const Box rb = region_box(g, (float)q[0], (float)q[1], (float)q[2], tf);
        Level<T> H;  // histogram spec for the current window
        H.type = 0;
        H.lo = T(0);
        H.scale = tau2 > T(0) ? T(32) / tau2 : T(0);
        H.ilo = 0;
        H.shift = 0;
        H.b = 0;
        int nlev = 0;
        uint32_t found = 0, n_sel = 0;
        for (int pass = 0;; ++pass) {
            ws->hist[lane] = 0;
            ws->dmin[lane] = Bits<T>::kMax;
            ws->dmax[lane] = 0;
            ws->imin[lane] = 0xffffffffu;
            ws->imax[lane] = 0;
            __syncwarp();
            uint32_t count = 0;
            visit_box<T>(gv, ws->run_start, ws->run_len, q, rb, true, tf, [&](bool valid, T d2, uint32_t idx) {
                const bool member = valid && (strict ? (d2 < tau2) : (d2 <= tau2));
                const int st = member ? classify<T>(ws, nlev, d2, idx) : 2;
                const bool take = st != 2;
                const uint32_t mask = __ballot_sync(FULL, take);
                if (take) {
                    const uint32_t pos = count + __popc(mask & ((1u << lane) - 1u));
                    if (pos < a.cap) {
                        buf[pos].d2 = d2;
                        buf[pos].idx = idx;
                    }
                    if (st == 1) {
                        const int bin = level_bin<T>(H, d2, idx);
                        atomicAdd(&ws->hist[bin], 1u);
                        atomicMin(&ws->dmin[bin], Bits<T>::of(d2));
                        atomicMax(&ws->dmax[bin], Bits<T>::of(d2));
                        atomicMin(&ws->imin[bin], idx);
                        atomicMax(&ws->imax[bin], idx);
                    }
                }
                count += __popc(mask);
            });
            __syncwarp();
            if (pass == 0) found = count;
            if (count <= a.cap) {
                n_sel = count;
                break;
            }
            // refine: window = the bin holding the k-th
            const uint32_t hv = ws->hist[lane];
            const uint32_t in_total = __reduce_add_sync(FULL, hv);
            const uint32_t below = count - in_total;
            uint32_t incl = hv;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const uint32_t y = __shfl_up_sync(FULL, incl, o);
                if (lane >= o) incl += y;
            }
            const uint32_t reach = __ballot_sync(FULL, below + incl >= k);
            const int b = reach ? __ffs(reach) - 1 : 31;
            if (nlev >= kMaxLevels) {
                if (lane == 0) atomicOr(a.err, ERR_INTERNAL);
                n_sel = a.cap;
                break;
            }
            if (lane == 0) {
                H.b = b;
                ws->lev[nlev] = H;
            }
            ++nlev;
            const T lo = Bits<T>::val(ws->dmin[b]), hi = Bits<T>::val(ws->dmax[b]);
            Level<T> N;
            N.b = 0;
            if (lo < hi) {
                N.type = 0;
                N.lo = lo;
                N.scale = T(32) / (hi - lo);
                N.ilo = 0;
                N.shift = 0;
            } else {
                const uint32_t ilo = ws->imin[b], span = ws->imax[b] - ilo;
                N.type = 1;
                N.lo = T(0);
                N.scale = T(0);
                N.ilo = ilo;
                N.shift = span == 0 ? 0 : max(0, 32 - __clz(span) - 5);
            }
            H = N;
            __syncwarp();
        }
        // sort the survivors and emit
        int P = 1;
        while (P < (int)n_sel) P <<= 1;
        if (n_sel > 1) bitonic_sort<T>(buf, (int)n_sel, P);
        if constexpr (SEL) {
            sel_push<T>(a.sel, rg, found, n_sel, a.rows_sorted ? qpos : row_base + qp.idx,
                        [&](uint32_t j) { return buf[j]; });
        } else {
            emit_row<T>(a.mode, k, n_sel, found, a.rows_sorted ? qpos : row_base + qp.idx, a.out_idx, a.out_d2,
                        a.out_found, a.fill_last, a.r2, [&](uint32_t j) { return buf[j]; });
        }
        __syncwarp();
    }
    if constexpr (SEL) sel_flush_block<T>(a.sel, rg, ring_base, kSearchWarps);
}

// ------------------------------------------------------------------ fast (float)
constexpr int kFastWarps = 4;
// Consecutive queries per work item. Small items keep the warps' finishing
// times even (per-query cost varies several-fold across a scene: walls and
// cylinders vs open ground), long items start fewer chunks, each of which needs
// a pilot bound for its first query. A single search uses guided items of
// remaining / (4 x warps) queries, between 4 and 64 (1M-point scene, k = 50:
// fixed 8 / 16 / 32 / 64-query items 1.354 / 1.379 / 1.479 / 1.675 ms; guided
// 1.30 ms -- long items early, short ones at the end).
constexpr int kChunkMax = 64;
constexpr int kChunkMin = 4;
constexpr int kGuide = 4;
constexpr int kSelBins = 64;     // selection histogram
constexpr int kMaxInBin = 24;    // larger bins (exact ties) fall back to a bitonic sort

struct FastArgs {
    GridView<float> gv;
    CloudTable ct;
    const SPoint<float>* queries;
    uint64_t m;
    int mode;
    uint32_t k;
    float r2;
    uint32_t cap;         // power of two, candidate keys per warp
    uint32_t cap_sorted;  // power of two, selected keys per warp
    uint32_t chunk;       // consecutive queries per work item (first pass): the largest
    uint32_t chunk_min;   // ... and the smallest: items shrink to remaining / guide_div
    uint32_t guide_div;
    const uint32_t* qlist;   // LIST pass: positions in `queries` to process ...
    const uint32_t* qcount;  // ... and their number (device)
    uint32_t* work;
    uint32_t* ovf_list;
    uint32_t* ovf_count;
    void* out_idx;
    float* out_d2;
    uint32_t* out_found;
    int fill_last;
    int rows_sorted;  // output row = position in `queries`
    uint32_t* err;
    SelSpec<float> sel;  // SEL instantiations
};

struct FastWarpSmem {
    uint32_t hist[kSelBins];
    uint32_t cursor[kSelBins];
    uint32_t run_start[32], run_len[32];
    float kth_d2;  // squared distance of the k-th neighbour of the query just solved
};

__device__ __forceinline__ uint64_t make_key(float d2, uint32_t idx) {
    return ((uint64_t)__float_as_uint(d2) << 32) | idx;
}
__device__ __forceinline__ float key_d2(uint64_t key) { return __uint_as_float((uint32_t)(key >> 32)); }

// bitonic sort of keys[0..n) padded to P with ~0 (larger than any key)
__device__ __forceinline__ void bitonic_keys(uint64_t* keys, int n, int P) {
    const int lane = threadIdx.x & 31;
    for (int i = n + lane; i < P; i += 32) keys[i] = ~0ull;
    __syncwarp();
    for (int size = 2; size <= P; size <<= 1) {
        for (int stride = size >> 1; stride > 0; stride >>= 1) {
            for (int t = lane; t < P / 2; t += 32) {
                const int i = 2 * stride * (t / stride) + (t % stride);
                const int j = i + stride;
                const bool up = (i & size) == 0;
                const uint64_t x = keys[i], y = keys[j];
                if ((y < x) == up) {
                    keys[i] = y;
                    keys[j] = x;
                }
            }
            __syncwarp();
        }
    }
}

// Hands the n_sel smallest of keys[0..count) (every key has d^2 <= tau2) to
// emit(pos, key) with their final sorted positions pos < n_sel, in no
// particular lane order. The selection histogram (ws->hist) is already
// filled. Keys of the bins up to the one holding the n_sel-th key are
// scattered into `out` by bin; a key's position is then its bin's start plus
// the number of smaller keys in its bin (bins hold a handful of keys; keys are
// unique since indices are). When exact ties crowd a bin the prefix is
// bitonic-sorted instead. Returns false, emitting nothing, when those bins
// hold more than out_cap keys.
template <typename Emit>
__device__ __forceinline__ bool select_emit(FastWarpSmem* ws, const uint64_t* keys, uint32_t count, uint32_t n_sel,
                                            float tau2, uint64_t* out, uint32_t out_cap, Emit&& emit) {
    const int lane = threadIdx.x & 31;
    const float sb = tau2 > 0.0f ? (float)kSelBins / tau2 : 0.0f;
    const auto bin_of = [&](uint64_t key) {
        const float x = key_d2(key) * sb;
        return x >= (float)(kSelBins - 1) ? kSelBins - 1 : (int)x;
    };
    // lane owns bins 2*lane, 2*lane+1
    const uint32_t h0 = ws->hist[2 * lane], h1 = ws->hist[2 * lane + 1];
    uint32_t incl = h0 + h1;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t y = __shfl_up_sync(FULL, incl, o);
        if (lane >= o) incl += y;
    }
    const uint32_t excl = incl - h0 - h1;
    ws->cursor[2 * lane] = excl;
    ws->cursor[2 * lane + 1] = excl + h0;
    // last bin needed: first bin whose inclusive count reaches n_sel
    const bool reach0 = excl + h0 >= n_sel, reach1 = incl >= n_sel;
    const uint32_t r0 = __ballot_sync(FULL, reach0), r1 = __ballot_sync(FULL, reach1);
    int bstar = kSelBins - 1;
    if (r0 | r1) {
        const int l0 = r0 ? __ffs(r0) - 1 : 64, l1 = r1 ? __ffs(r1) - 1 : 64;
        bstar = min(2 * l0, 2 * l1 + 1);
    }
    const uint32_t big = __ballot_sync(FULL, (2 * lane <= bstar && h0 > kMaxInBin) ||
                                                 (2 * lane + 1 <= bstar && h1 > kMaxInBin));
    __syncwarp();
    uint32_t n_take = 0;
    {
        const int lb = bstar >> 1;
        const uint32_t e = __shfl_sync(FULL, excl, lb), hh0 = __shfl_sync(FULL, h0, lb),
                       hh1 = __shfl_sync(FULL, h1, lb);
        n_take = (bstar & 1) ? e + hh0 + hh1 : e + hh0;
    }
    if (n_take > out_cap) return false;
    for (uint32_t i = lane; i < count; i += 32) {
        const uint64_t key = keys[i];
        const int bin = bin_of(key);
        if (bin <= bstar) out[atomicAdd(&ws->cursor[bin], 1u)] = key;
    }
    __syncwarp();
    if (big) {
        // exact ties crowd a bin: sort the whole prefix
        int P = 1;
        while (P < (int)n_take) P <<= 1;
        if (P > (int)out_cap) return false;
        bitonic_keys(out, (int)n_take, P);
        for (uint32_t p = lane; p < n_sel; p += 32) emit(p, out[p]);
        __syncwarp();
        return true;
    }
    // rank inside the bin; ws->cursor[bin] is now the bin's end
    for (uint32_t p = lane; p < n_take; p += 32) {
        const uint64_t key = out[p];
        const int bin = bin_of(key);
        const uint32_t end = ws->cursor[bin], beg = end - ws->hist[bin];
        uint32_t pos = beg;
        for (uint32_t q = beg; q < end; ++q) pos += out[q] < key;
        if (pos < n_sel) emit(pos, key);
    }
    __syncwarp();
    return true;
}

// LIST: a second pass over the queries whose key buffer overflowed in the
// first (a.qlist / a.qcount), each with its pilot bound -- the first pass's
// bound came from a solved neighbour and was too loose -- and a larger buffer.
template <bool MULTI, bool LIST, bool SEL>
__device__ __forceinline__ void fast_search_body(const FastArgs& a) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    FastWarpSmem* ws = reinterpret_cast<FastWarpSmem*>(smem_raw) + wib;
    uint64_t* keys = reinterpret_cast<uint64_t*>(smem_raw + kFastWarps * sizeof(FastWarpSmem)) +
                     (size_t)wib * (a.cap + a.cap_sorted);
    uint64_t* sorted = keys + a.cap;
    SelRing rg{};
    unsigned char* ring_base =
        smem_raw + kFastWarps * sizeof(FastWarpSmem) + (size_t)kFastWarps * (a.cap + a.cap_sorted) * sizeof(uint64_t);
    if constexpr (SEL) {
        rg = sel_ring_at(ring_base + wib * sel_ring_bytes(a.sel.max_knn, a.sel.ring), a.sel.max_knn, a.sel.ring);
    }
    const uint32_t k = a.k;
    const uint64_t m = LIST ? (uint64_t)*a.qcount : a.m;
    for (;;) {
        // Guided work items: a.chunk consecutive queries while many remain
        // (fewer chunk starts, hence fewer pilot bounds), shrinking to
        // remaining / guide_div and at least a.chunk_min towards the end, so
        // that warps finish together. List queries are few and costly: one
        // per item.
        uint32_t start = 0, len = 1;
        if (lane == 0) {
            if (!LIST) {
                len = a.chunk;
                if (a.chunk_min < a.chunk) {
                    const uint32_t seen = __ldcg(a.work);
                    const uint64_t rem = seen < m ? m - seen : 0;
                    const uint64_t g = rem / a.guide_div;
                    len = g >= a.chunk ? a.chunk : (g <= a.chunk_min ? a.chunk_min : (uint32_t)g);
                }
            }
            start = atomicAdd(a.work, len);
        }
        start = __shfl_sync(FULL, start, 0);
        len = __shfl_sync(FULL, len, 0);
        const uint64_t q0 = start;
        if (q0 >= m) break;
        const uint64_t q1 = min(q0 + (uint64_t)len, m);
        // the last 32 solved queries of this chunk, one per lane: position and d_k
        float rx = 0.0f, ry = 0.0f, rz = 0.0f, rdk = -1.0f;
        int rci = -1;
        for (uint64_t qpos = q0; qpos < q1; ++qpos) {
            const uint64_t qi = LIST ? (uint64_t)a.qlist[qpos] : qpos;
            const SPoint<float> qp = a.queries[qi];
            GridView<float> gv = a.gv;
            uint64_t row_base = 0;
            int ci = 0;
            if (MULTI) {
                ci = cloud_of(a.ct, qi);
                gv.g = a.ct.g[ci];
                gv.cell_start = a.gv.cell_start + a.ct.cell_base[ci];
                row_base = a.ct.off[ci];
            }
            const GridParams& g = gv.g;
            const float q[3] = {qp.x, qp.y, qp.z};
            bool optimistic = false;  // the first try used a triangle bound
            for (int attempt = 0; attempt < 2; ++attempt) {
                float tau2;
                bool strict;
                if (a.mode == MODE_KNN) {
                    strict = false;
                    // From a solved neighbour p, d_k(q) <= d_k(p) + |q - p|. The radius
                    // used is the optimistic d_k(p) + |q - p| / 2 (best over the lanes,
                    // neighbours within 0.9 d_k(p)): when it holds >= k points the k
                    // nearest are all among them; otherwise (count < k, ~2% of the
                    // queries of the outdoor scene) the query is collected again at
                    // once within the guaranteed d_k(p) + |q - p|. (A pilot bound for
                    // that second try measured slower: its extra box pass costs more
                    // than the list pass it saves.)
                    float bound = INFINITY;
                    if (!LIST && rdk >= 0.0f && rci == ci) {
                        const float dx = q[0] - rx, dy = q[1] - ry, dz = q[2] - rz;
                        const float dq = sqrtf(dx * dx + dy * dy + dz * dz);
                        if (attempt == 0) {
                            if (dq <= 0.9f * rdk) bound = rdk + 0.5f * dq;
                        } else {
                            bound = rdk + dq;
                        }
                    }
                    bound = __uint_as_float(__reduce_min_sync(FULL, __float_as_uint(bound)));
                    if (attempt == 0) optimistic = bound < INFINITY;
                    if (bound < INFINITY) {
                        const float t = bound * 1.00002f + 1e-30f + g.margin * 1e-3f;  // rounding slack
                        tau2 = t * t;
                    } else {
                        tau2 = pilot_tau2<float, LIST ? 4 : 1>(gv, ws->hist, ws->run_start, ws->run_len, q, k);
                    }
                } else {
                    strict = true;
                    tau2 = a.r2;
                }
                const float tf = sqrtf(tau2) * 1.000001f + g.margin;
                const Box rb = region_box(g, q[0], q[1], q[2], tf);
                uint32_t count = 0;
                // the selection histogram is filled while collecting
                const float sb = tau2 > 0.0f ? (float)kSelBins / tau2 : 0.0f;
                ws->hist[lane] = 0;
                ws->hist[lane + 32] = 0;
                __syncwarp();
                const auto collect = [&](bool valid, float d2, uint32_t idx) {
                    const bool take = valid && (strict ? (d2 < tau2) : (d2 <= tau2));
                    const uint32_t mask = __ballot_sync(FULL, take);
                    if (take) {
                        const uint32_t pos = count + __popc(mask & ((1u << lane) - 1u));
                        if (pos < a.cap) keys[pos] = make_key(d2, idx);
                        const float x = d2 * sb;
                        atomicAdd(&ws->hist[x >= (float)(kSelBins - 1) ? kSelBins - 1 : (int)x], 1u);
                    }
                    count += __popc(mask);
                };
                visit_box<float, decltype(collect)&, LIST ? 4 : 1>(gv, ws->run_start, ws->run_len, q, rb, true, tf,
                                                                   collect);
                __syncwarp();
                const bool short_knn = a.mode == MODE_KNN && count < k;  // the optimistic radius fell short
                const uint32_t n_sel = a.mode == MODE_KNN ? k : min(count, k);
                const uint64_t row = a.rows_sorted ? qi : row_base + qp.idx;
                bool ok = count <= a.cap && !short_knn;
                if (ok && n_sel > 0) {
                    // each selected key goes straight to its place in the result row
                    if constexpr (SEL) {
                        const size_t stride = (size_t)a.sel.ring + 1;
                        const uint32_t kcap = a.sel.max_knn;
                        ok = select_emit(ws, keys, count, n_sel, tau2, sorted, a.cap_sorted, [&](uint32_t pos, uint64_t key) {
                            if (pos < kcap) rg.idx[pos * stride + rg.n] = (uint32_t)key;
                        });
                    } else if (a.mode == MODE_KNN) {
                        uint32_t* oi = static_cast<uint32_t*>(a.out_idx) + row * k;
                        float* od = a.out_d2 ? a.out_d2 + row * k : nullptr;
                        ok = select_emit(ws, keys, count, n_sel, tau2, sorted, a.cap_sorted, [&](uint32_t pos, uint64_t key) {
                            oi[pos] = (uint32_t)key;
                            if (od) od[pos] = key_d2(key);
                            if (pos == k - 1) ws->kth_d2 = key_d2(key);
                        });
                    } else {
                        int32_t* oi = static_cast<int32_t*>(a.out_idx) + row * k;
                        float* od = a.out_d2 ? a.out_d2 + row * k : nullptr;
                        ok = select_emit(ws, keys, count, n_sel, tau2, sorted, a.cap_sorted, [&](uint32_t pos, uint64_t key) {
                            oi[pos] = (int32_t)(uint32_t)key;
                            if (od) od[pos] = key_d2(key);
                        });
                    }
                }
                if (!ok) {
                    if (attempt == 0 && optimistic && short_knn) continue;  // the guaranteed bound next
                    if (lane == 0) {
                        const uint32_t slot = atomicAdd(a.ovf_count, 1u);
                        a.ovf_list[slot] = (uint32_t)qi;
                    }
                    break;
                }
                if constexpr (SEL) {
                    // park the query; its lane solves it with the others of the ring
                    if (lane == 0) {
                        rg.found[rg.n] = count;
                        rg.row[rg.n] = (uint32_t)row;
                    }
                    ++rg.n;
                    if (rg.n == a.sel.ring) sel_flush<float>(a.sel, rg);
                } else if (a.mode != MODE_KNN) {
                    // nanoflann's radius row: -1 / 0 after the hits, radius^2 in the last slot of a short row
                    int32_t* oi = static_cast<int32_t*>(a.out_idx) + row * k;
                    float* od = a.out_d2 ? a.out_d2 + row * k : nullptr;
                    for (uint32_t j = n_sel + lane; j < k; j += 32) {
                        oi[j] = -1;
                        if (od) od[j] = (a.fill_last && j == k - 1) ? a.r2 : 0.0f;
                    }
                    if (a.out_found && lane == 0) a.out_found[row] = count;
                }
                if (!LIST && a.mode == MODE_KNN && lane == (int)(qi & 31)) {
                    rdk = sqrtf(ws->kth_d2);
                    rx = q[0];
                    ry = q[1];
                    rz = q[2];
                    rci = ci;
                }
                __syncwarp();
                break;
            }
        }
    }
    if constexpr (SEL) sel_flush_block<float>(a.sel, rg, ring_base, kFastWarps);
}

template <bool MULTI, bool LIST, bool SEL = false>
__global__ void __launch_bounds__(kFastWarps * 32) fast_search_kernel(const __grid_constant__ FastArgs a) {
    fast_search_body<MULTI, LIST, SEL>(a);
}

// The single-cloud kNN pass, compiled for 10 resident blocks per SM (48
// registers, a 24-byte spill: 1.5% faster at k = 50, 10% at k = 1 than its
// natural 56 registers); the radius pass keeps its natural allocation (the
// bound makes it 3-4% slower).
__global__ void __launch_bounds__(kFastWarps * 32, 10) fast_knn_kernel(const __grid_constant__ FastArgs a) {
    fast_search_body<false, false, false>(a);
}

template <typename T>
int general_smem_bytes(uint32_t cap, bool in_smem) {
    return (int)(kSearchWarps * (sizeof(WarpSmem<T>) + (in_smem ? (size_t)cap * sizeof(Entry<T>) : 0)));
}

template <typename T>
int launch_general_view(const GridView<T>& gv, const CloudTable& ct, const SPoint<T>* queries, uint64_t m,
                        const uint32_t* qlist, const uint32_t* qcount, int mode, uint32_t k, T radius,
                        const SearchOut<T>& out, cudaStream_t s) {
    const DeviceInfo* di;
    PGEOF_TRY(current_device_info(&di));
    // buffer capacity: a power of two comfortably above k
    const uint64_t want = mode == MODE_KNN ? std::max<uint64_t>(2ull * k, 128) : std::max<uint64_t>(4ull * k, 256);
    uint32_t cap = 1;
    while (cap < want) cap <<= 1;
    const int ring_smem = out.sel ? (int)(kSearchWarps * sel_ring_bytes(out.sel->max_knn, out.sel->ring)) : 0;
    const bool in_smem =
        general_smem_bytes<T>(cap, true) + ring_smem <= std::min(di->max_smem_optin, 200 * 1024);
    const int smem = general_smem_bytes<T>(cap, in_smem) + ring_smem;
    auto kern = out.sel ? search_kernel<T, true> : search_kernel<T, false>;
    int per_sm = 0;
    PGEOF_TRY(kernel_blocks_per_sm((const void*)kern, kSearchWarps * 32, smem, &per_sm));
    const uint64_t blocks = std::min<uint64_t>(ceil_div_u(m, kSearchWarps), (uint64_t)di->sm_count * per_sm);
    Scratch gbuf;
    SearchArgs<T> a{};
    if (!in_smem) {
        PGEOF_TRY(gbuf.alloc(blocks * kSearchWarps * (size_t)cap * sizeof(Entry<T>), s));
        a.gbuf = gbuf.as<Entry<T>>();
    }
    a.gv = gv;
    a.ct = ct;
    a.queries = queries;
    a.m = m;
    a.qlist = qlist;
    a.qcount = qcount;
    a.mode = mode;
    a.k = k;
    a.r2 = (T)(radius * radius);  // sq_search_radius in real_t, nn_search.hpp:98
    a.cap = cap;
    a.buf_in_smem = in_smem ? 1 : 0;
    a.out_idx = out.indices;
    a.out_d2 = out.sqr_dist;
    a.out_found = out.found;
    a.fill_last = out.radius_fill_last ? 1 : 0;
    a.rows_sorted = out.rows_in_query_order ? 1 : 0;
    a.err = device_error_word();
    if (out.sel) a.sel = *out.sel;
    KernelTimer kt(qlist ? "overflow_general_kernel"
                         : (out.sel ? "selected_search_kernel"
                                    : (mode == MODE_KNN ? "knn_search_kernel" : "radius_search_kernel")),
                   s);
    kern<<<(unsigned)blocks, kSearchWarps * 32, smem, s>>>(a);
    count_launch();
    return check_launch("search_kernel");
}

template <typename T>
int launch_general(const GridIndex<T>& grid, const SPoint<T>* queries, uint64_t m, const uint32_t* qlist,
                   const uint32_t* qcount, int mode, uint32_t k, T radius, const SearchOut<T>& out,
                   cudaStream_t s) {
    GridView<T> gv;
    gv.g = grid.g;
    gv.cell_start = grid.cell_start;
    gv.pts = grid.pts;
    return launch_general_view<T>(gv, CloudTable{}, queries, m, qlist, qcount, mode, k, radius, out, s);
}

// The fast kernel over `queries` (cell order), then the general kernel over the
// queries whose buffer overflowed. `words`: 8 + m words of scratch (work
// counter, overflow count, overflow list). With `words2` (another 2 (8 + m)
// words) the overflowing queries get two list passes of the fast kernel
// (pilot bounds, 1024- then 4096-key buffers) before the general kernel.
int launch_fast(const GridView<float>& gv, const CloudTable& ct, const SPoint<float>* queries, uint64_t m, int mode,
                uint32_t k, float radius, const SearchOut<float>& out, uint32_t* words, uint32_t* words2,
                cudaStream_t s, uint32_t chunk = 0) {
    const DeviceInfo* di;
    PGEOF_TRY(current_device_info(&di));
    // candidate buffer: 256 keys for kNN, 512 for radius (or 4k); selected
    // prefix: k plus the few keys that share the k-th key's histogram bin
    static const uint64_t knn_keys = [] {
        const char* e = getenv("PGEOF_KNN_KEYS");  // tuning override of the kNN candidate buffer
        const unsigned long v = e ? strtoul(e, nullptr, 10) : 256ul;
        return (uint64_t)std::min<unsigned long>(std::max<unsigned long>(v, 64ul), 4096ul);
    }();
    uint32_t cap = 1;
    const uint64_t want = std::max<uint64_t>(mode == MODE_KNN ? knn_keys : 512, 4ull * k);
    while (cap < want) cap <<= 1;
    uint32_t cap_sorted = 1;
    while (cap_sorted < k + k / 2 + 16) cap_sorted <<= 1;
    cap_sorted = std::min(cap_sorted, cap);
    const int ring_smem = out.sel ? (int)(kFastWarps * sel_ring_bytes(out.sel->max_knn, out.sel->ring)) : 0;
    const int smem =
        (int)(kFastWarps * (sizeof(FastWarpSmem) + (size_t)(cap + cap_sorted) * sizeof(uint64_t))) + ring_smem;
    auto kern = out.sel ? fast_search_kernel<false, false, true>
                        : (ct.n ? fast_search_kernel<true, false>
                                : (mode == MODE_KNN ? fast_knn_kernel : fast_search_kernel<false, false>));
    int per_sm = 0;
    PGEOF_TRY(kernel_blocks_per_sm((const void*)kern, kFastWarps * 32, smem, &per_sm));
    // Queries per work item: a fixed count when the caller gives one (batch
    // plans tune it), else guided items from kChunkMax down to kChunkMin
    // (PGEOF_KNN_CHUNK / PGEOF_KNN_CHUNK_MIN override them for tuning).
    static const uint32_t guided_max = [] {
        const char* e = getenv("PGEOF_KNN_CHUNK");
        const unsigned long v = e ? strtoul(e, nullptr, 10) : (unsigned long)kChunkMax;
        return (uint32_t)std::min<unsigned long>(std::max<unsigned long>(v, 1ul), 1024ul);
    }();
    static const uint32_t guided_min = [] {
        const char* e = getenv("PGEOF_KNN_CHUNK_MIN");
        const unsigned long v = e ? strtoul(e, nullptr, 10) : (unsigned long)kChunkMin;
        return (uint32_t)std::min<unsigned long>(std::max<unsigned long>(v, 1ul), 1024ul);
    }();
    // Radius searches (no pilot bounds to save) keep fixed 16-query items:
    // guided items measured no faster there and lengthened the serving
    // stream's p99 (3.4 vs 2.7 ms over 30 s).
    if (chunk == 0 && mode != MODE_KNN) chunk = 16;
    const uint32_t chunk_max = chunk ? chunk : guided_max;
    const uint32_t chunk_min = chunk ? chunk : std::min(guided_min, guided_max);
    const uint64_t items = ceil_div_u(m, chunk_min);
    const uint64_t blocks = std::min<uint64_t>(ceil_div_u(items, kFastWarps), (uint64_t)di->sm_count * per_sm);
    PGEOF_CUDA_TRY(cudaMemsetAsync(words, 0, 8 * sizeof(uint32_t), s));
    FastArgs a{};
    a.gv = gv;
    a.ct = ct;
    a.queries = queries;
    a.m = m;
    a.mode = mode;
    a.k = k;
    a.r2 = radius * radius;  // sq_search_radius in real_t, nn_search.hpp:98
    a.cap = cap;
    a.cap_sorted = cap_sorted;
    a.chunk = chunk_max;
    a.chunk_min = chunk_min;
    static const uint64_t guide = [] {
        const char* e = getenv("PGEOF_KNN_GUIDE");  // tuning override: items shrink to remaining / (guide x warps)
        const unsigned long v = e ? strtoul(e, nullptr, 10) : (unsigned long)kGuide;
        return (uint64_t)std::min<unsigned long>(std::max<unsigned long>(v, 1ul), 64ul);
    }();
    a.guide_div = (uint32_t)std::max<uint64_t>(1, guide * blocks * kFastWarps);
    a.work = words;
    a.ovf_count = words + 1;
    a.ovf_list = words + 8;
    a.out_idx = out.indices;
    a.out_d2 = out.sqr_dist;
    a.out_found = out.found;
    a.fill_last = out.radius_fill_last ? 1 : 0;
    a.rows_sorted = out.rows_in_query_order ? 1 : 0;
    a.err = device_error_word();
    if (out.sel) a.sel = *out.sel;
    {
        KernelTimer kt(out.sel ? "selected_search_kernel" : (mode == MODE_KNN ? "knn_search_kernel" : "radius_search_kernel"),
                       s);
        kern<<<(unsigned)blocks, kFastWarps * 32, smem, s>>>(a);
    }
    count_launch();
    PGEOF_TRY(check_launch("fast_search_kernel"));
    if (words2 && !ct.n) {
        // List passes over the overflowing queries (one query per work item,
        // a pilot bound, a larger buffer), sized on the device: 1024 keys, then
        // 4096 keys for the few that still overflow, and the general kernel
        // (refinement passes) for whatever is left -- usually nothing. The
        // small first list buffer keeps that pass's occupancy for its
        // thousands of queries; the second pass spares the general kernel's
        // refinement passes, whose latency made its launch long.
        const uint32_t* in_list = a.ovf_list;
        const uint32_t* in_count = a.ovf_count;
        for (int pass = 0; pass < 2; ++pass) {
            uint32_t* w = words2 + (size_t)pass * (m + 8);
            uint32_t cap2 = 1;
            while (cap2 < std::max<uint64_t>(pass == 0 ? 1024 : 4096, 4ull * k)) cap2 <<= 1;
            const int smem2 =
                (int)(kFastWarps * (sizeof(FastWarpSmem) + (size_t)(cap2 + cap_sorted) * sizeof(uint64_t))) +
                ring_smem;
            auto kern2 = out.sel ? fast_search_kernel<false, true, true> : fast_search_kernel<false, true>;
            int per_sm2 = 0;
            PGEOF_TRY(kernel_blocks_per_sm((const void*)kern2, kFastWarps * 32, smem2, &per_sm2));
            PGEOF_CUDA_TRY(cudaMemsetAsync(w, 0, 8 * sizeof(uint32_t), s));
            FastArgs a2 = a;
            a2.cap = cap2;
            a2.qlist = in_list;
            a2.qcount = in_count;
            a2.work = w;
            a2.ovf_count = w + 1;
            a2.ovf_list = w + 8;
            {
                KernelTimer kt("overflow_list_kernel", s);
                kern2<<<(unsigned)((uint64_t)di->sm_count * per_sm2), kFastWarps * 32, smem2, s>>>(a2);
            }
            count_launch();
            PGEOF_TRY(check_launch("fast_search_kernel(list)"));
            in_list = a2.ovf_list;
            in_count = a2.ovf_count;
        }
        return launch_general_view<float>(gv, ct, queries, m, in_list, in_count, mode, k, radius, out, s);
    }
    // queries whose key buffer overflowed: the general kernel, sized on the device
    return launch_general_view<float>(gv, ct, queries, m, a.ovf_list, a.ovf_count, mode, k, radius, out, s);
}

}  // namespace

template <typename T>
int launch_search(const GridIndex<T>& grid, const SPoint<T>* queries, const uint32_t* /*qstart*/, uint64_t m,
                  int mode, uint32_t k, T radius, const SearchOut<T>& out, cudaStream_t s) {
    if (m == 0 || k == 0) return PGEOF_OK;
    if (grid.n == 0) return fail(PGEOF_ERR_INVALID_ARGUMENT, "search over an empty point cloud");
    if constexpr (sizeof(T) != sizeof(float)) {
        return launch_general<T>(grid, queries, m, nullptr, nullptr, mode, k, radius, out, s);
    } else {
        if (k > 128 || m >= 0xfff00000ull)  // 32-bit work counters with headroom for the last items
            return launch_general<T>(grid, queries, m, nullptr, nullptr, mode, k, radius, out, s);
        Scratch ctl;
        PGEOF_TRY(ctl.alloc(3 * (m + 8) * sizeof(uint32_t), s));
        GridView<float> gv;
        gv.g = grid.g;
        gv.cell_start = grid.cell_start;
        gv.pts = grid.pts;
        return launch_fast(gv, CloudTable{}, queries, m, mode, k, radius, out, ctl.as<uint32_t>(),
                           ctl.as<uint32_t>() + m + 8, s);
    }
}

int launch_search_batch(const CloudTable& ct, const uint32_t* cell_start, const SPoint<float>* pts, uint64_t n_points,
                        uint32_t k, uint32_t* indices, float* sqr_dist, uint32_t* work, uint32_t* ovf,
                        cudaStream_t s, uint32_t chunk) {
    if (n_points == 0 || k == 0) return PGEOF_OK;
    GridView<float> gv{};
    gv.cell_start = cell_start;
    gv.pts = pts;
    SearchOut<float> out;
    out.indices = indices;
    out.sqr_dist = sqr_dist;
    if (k > 128)
        return launch_general_view<float>(gv, ct, pts, n_points, nullptr, nullptr, MODE_KNN, k, 0.0f, out, s);
    (void)ovf;
    return launch_fast(gv, ct, pts, n_points, MODE_KNN, k, 0.0f, out, work, nullptr, s, chunk);
}

template int launch_search<float>(const GridIndex<float>&, const SPoint<float>*, const uint32_t*, uint64_t, int,
                                  uint32_t, float, const SearchOut<float>&, cudaStream_t);
template int launch_search<double>(const GridIndex<double>&, const SPoint<double>*, const uint32_t*, uint64_t, int,
                                   uint32_t, double, const SearchOut<double>&, cudaStream_t);

}  // namespace pgeof
