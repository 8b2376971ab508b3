// search.cu -- exact k-nearest / radius neighbour search over the grid index
// (include/nn_search.hpp:31-132) and the radius-search + PCA path of
// compute_features_selected (include/pgeof.hpp:325-375).
//
// One warp owns one query; queries are visited in cell order so neighbouring
// warps read the same cells. Candidates are streamed as contiguous runs of the
// cell-ordered point array: every row of cells (fixed y, z; a range of x) is one
// run, runs are packed across the 32 lanes so no lane idles at row ends.
//
// Selection never keeps a sorted top-k list while scanning. Instead:
//   A. grow a block of cells around the query until it holds >= k points
//      (cell counts only, no point reads);
//   B. one pass over that block builds a 32-bin histogram of squared distances,
//      whose k-th-count bin edge tau^2 bounds the k-th neighbour distance;
//   C. one pass over every cell within tau (rows clipped to the sphere) appends
//      the points with d^2 <= tau^2 to a per-warp buffer -- usually ~1.2 k of
//      them -- which is then bitonic-sorted by (d^2, index).
// If pass C finds more points than the buffer holds, it refines instead: each
// further pass histograms only the points inside the bin that contains the
// k-th, first on d^2, then on the index when distances tie exactly, until the
// survivors fit. The result is the exact k smallest (d^2, index) pairs.
//
// Distances use nanoflann's metric_L2_Simple arithmetic: (q - p)^2 per axis,
// summed x, y, z, each operation rounded (no FMA), so values are bit-identical
// to the reference's. Ties at equal distance order by index (nanoflann keeps
// its tree-traversal order there).
#include <algorithm>

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
struct SearchArgs {
    GridParams g;
    const uint32_t* cell_start;
    const SPoint<T>* pts;
    const SPoint<T>* queries;
    uint64_t m;
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
    uint32_t* err;
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

// Visit every point of the cells in `bx` (rows clipped to the sphere of squared
// radius R2 around q when prune). All lanes call visit(valid, d2, idx) together.
template <typename T, typename F>
__device__ __forceinline__ void visit_box(const SearchArgs<T>& a, WarpSmem<T>* ws, const T (&q)[3], const Box& bx,
                                          bool prune, float Rf, F&& visit) {
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
                const float gy = axis_gap(qf1, cy, a.g.oy, a.g.h, a.g.margin);
                const float gz = axis_gap(qf2, cz, a.g.oz, a.g.h, a.g.margin);
                const float dyz2 = gy * gy + gz * gz;
                if (dyz2 > Rf2) {
                    keep = false;
                } else {
                    const float bxr = sqrtf(Rf2 - dyz2) + a.g.margin;
                    xa = max(xa, cell_floor((qf0 - bxr - a.g.ox) * a.g.inv_h, a.g.gx));
                    xb = min(xb, cell_floor((qf0 + bxr - a.g.ox) * a.g.inv_h, a.g.gx));
                }
            }
            if (keep && xa <= xb) {
                const uint32_t base = ((uint32_t)cz * (uint32_t)a.g.gy + (uint32_t)cy) * (uint32_t)a.g.gx;
                st = __ldg(a.cell_start + base + xa);
                len = __ldg(a.cell_start + base + xb + 1) - st;
            }
        }
        // pack the non-empty runs into lanes 0..nrows-1
        const uint32_t ne = __ballot_sync(FULL, len > 0);
        const int nrows = __popc(ne);
        if (nrows == 0) continue;
        if (len > 0) {
            const int ci = __popc(ne & ((1u << lane) - 1u));
            ws->run_start[ci] = st;
            ws->run_len[ci] = len;
        }
        __syncwarp();
        const uint32_t c_st = lane < nrows ? ws->run_start[lane] : 0u;
        const uint32_t c_len = lane < nrows ? ws->run_len[lane] : 0u;
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
                const SPoint<T> p = a.pts[r_st + (pos - r_ex)];
                d2 = dist2<T>(q, p);
                idx = p.idx;
            }
            visit(valid, d2, idx);
            r_base = __popc(__ballot_sync(FULL, lane < nrows && excl <= base + 32)) - 1;
        }
    }
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

template <typename T>
__device__ __forceinline__ T warp_max(T v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = max(v, __shfl_xor_sync(FULL, v, o));
    return v;
}

template <typename T>
__global__ void __launch_bounds__(kSearchWarps * 32) search_kernel(const __grid_constant__ SearchArgs<T> a) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    WarpSmem<T>* ws = reinterpret_cast<WarpSmem<T>*>(smem_raw) + wib;
    Entry<T>* buf = a.buf_in_smem
                        ? reinterpret_cast<Entry<T>*>(smem_raw + kSearchWarps * sizeof(WarpSmem<T>)) + (size_t)wib * a.cap
                        : a.gbuf + ((size_t)blockIdx.x * kSearchWarps + wib) * a.cap;
    const uint64_t nwarps = (uint64_t)gridDim.x * kSearchWarps;
    const GridParams& g = a.g;
    const int gd[3] = {g.gx, g.gy, g.gz};
    const float go[3] = {g.ox, g.oy, g.oz};

    for (uint64_t qi = (uint64_t)blockIdx.x * kSearchWarps + wib; qi < a.m; qi += nwarps) {
        const SPoint<T> qp = a.queries[qi];
        const T q[3] = {qp.x, qp.y, qp.z};
        const uint32_t k = a.k;
        int cq[3];
#pragma unroll
        for (int d = 0; d < 3; ++d) {
            const float c = ((float)q[d] - go[d]) * g.inv_h;
            cq[d] = (int)floorf(fminf(fmaxf(c, 0.0f), (float)(gd[d] - 1)));
        }
        T tau2;
        bool strict;
        if (a.mode == MODE_KNN) {
            // A. grow a cell block until it holds >= k points
            Box bx;
            for (int r = 0;; ++r) {
                bool full = true;
#pragma unroll
                for (int d = 0; d < 3; ++d) {
                    bx.lo[d] = max(0, cq[d] - r);
                    bx.hi[d] = min(gd[d] - 1, cq[d] + r);
                    full = full && bx.lo[d] == 0 && bx.hi[d] == gd[d] - 1;
                }
                const int ny = bx.hi[1] - bx.lo[1] + 1, nz = bx.hi[2] - bx.lo[2] + 1;
                uint32_t cnt = 0;
                for (int row = lane; row < ny * nz; row += 32) {
                    const int cy = bx.lo[1] + row % ny, cz = bx.lo[2] + row / ny;
                    const uint32_t base = ((uint32_t)cz * (uint32_t)g.gy + (uint32_t)cy) * (uint32_t)g.gx;
                    cnt += __ldg(a.cell_start + base + bx.hi[0] + 1) - __ldg(a.cell_start + base + bx.lo[0]);
                }
                cnt = __reduce_add_sync(FULL, cnt);
                if (cnt >= k || full) break;
            }
            // B. histogram of d^2 over the block -> tau^2 >= k-th distance^2
            float F2 = 0.0f;
#pragma unroll
            for (int d = 0; d < 3; ++d) {
                const float lo = go[d] + (float)bx.lo[d] * g.h, hi = go[d] + (float)(bx.hi[d] + 1) * g.h;
                const float far = fmaxf((float)q[d] - lo, hi - (float)q[d]) + g.margin;
                F2 += far * far;
            }
            const float sb = 32.0f / fmaxf(F2, 1e-30f);
            ws->hist[lane] = 0;
            __syncwarp();
            T dmax = T(0);
            visit_box<T>(a, ws, q, bx, false, 0.0f, [&](bool valid, T d2, uint32_t) {
                if (valid) {
                    const float x = (float)d2 * sb;
                    const int bin = x >= 31.0f ? 31 : (int)x;
                    atomicAdd(&ws->hist[bin], 1u);
                    dmax = max(dmax, d2);
                }
            });
            __syncwarp();
            dmax = warp_max(dmax);
            uint32_t hv = ws->hist[lane], incl = hv;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const uint32_t y = __shfl_up_sync(FULL, incl, o);
                if (lane >= o) incl += y;
            }
            const uint32_t reach = __ballot_sync(FULL, incl >= k);
            const int b = reach ? __ffs(reach) - 1 : 31;
            tau2 = dmax;
            if (b < 31) tau2 = min(dmax, (T)(((float)(b + 1) / sb) * 1.000004f));
            strict = false;
        } else {
            tau2 = a.r2;
            strict = true;
        }

        // C. collect every point within tau (refining when the buffer overflows)
        const float tf = sqrtf((float)tau2) * 1.000001f + g.margin;
        Box rb;
#pragma unroll
        for (int d = 0; d < 3; ++d) {
            rb.lo[d] = max(0, cell_floor(((float)q[d] - tf - go[d]) * g.inv_h, gd[d]));
            rb.hi[d] = min(gd[d] - 1, cell_floor(((float)q[d] + tf - go[d]) * g.inv_h, gd[d]));
        }
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
            visit_box<T>(a, ws, q, rb, true, tf, [&](bool valid, T d2, uint32_t idx) {
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
        const uint64_t qo = qp.idx;
        if (a.mode == MODE_KNN) {
            uint32_t* oi = static_cast<uint32_t*>(a.out_idx) + qo * k;
            T* od = a.out_d2 ? a.out_d2 + qo * k : nullptr;
            for (uint32_t j = lane; j < k; j += 32) {
                const Entry<T> e = buf[j];
                oi[j] = e.idx;
                if (od) od[j] = e.d2;
            }
        } else {
            const uint32_t nk = min(n_sel, k);
            int32_t* oi = static_cast<int32_t*>(a.out_idx) + qo * k;
            T* od = a.out_d2 ? a.out_d2 + qo * k : nullptr;
            for (uint32_t j = lane; j < k; j += 32) {
                if (j < nk) {
                    const Entry<T> e = buf[j];
                    oi[j] = (int32_t)e.idx;
                    if (od) od[j] = e.d2;
                } else {
                    oi[j] = -1;
                    if (od) od[j] = (a.fill_last && j == k - 1) ? a.r2 : T(0);
                }
            }
            if (a.out_found && lane == 0) a.out_found[qo] = found;
        }
        __syncwarp();
    }
}

// ------------------------------------------------------------------ selected
constexpr int kSelThreads = 128;
constexpr int kSelIdsPerLaunch = 32;

template <typename T>
struct SelArgs {
    const T* xyz;
    uint64_t n;
    const int32_t* nbr;
    const uint32_t* found;
    uint32_t max_knn;
    int n_ids, id_offset, out_ids;
    int ids[kSelIdsPerLaunch];
    int order;
    T* out;
};

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

// include/pgeof.hpp:354-369: fewer than 2 points in the radius -> zeros;
// otherwise PCA of the nearest min(found, max_knn) in (distance, index) order.
template <typename T>
__global__ void __launch_bounds__(kSelThreads) selected_pca_kernel(const __grid_constant__ SelArgs<T> a) {
    using O = XOps<T>;
    const uint64_t i = blockIdx.x * (uint64_t)kSelThreads + threadIdx.x;
    if (i >= a.n) return;
    T* row = a.out + i * a.out_ids + a.id_offset;
    const uint32_t found = a.found[i];
    if (found < 2) {
        for (int t = 0; t < a.n_ids; ++t) row[t] = T(0);
        return;
    }
    const uint32_t k = min(found, a.max_knn);
    const int32_t* nb = a.nbr + i * a.max_knn;
    T sx = 0, sy = 0, sz = 0;
    for (uint32_t j = 0; j < k; ++j) {
        const uint64_t id = (uint32_t)nb[j];
        sx = O::add(sx, a.xyz[3 * id]);
        sy = O::add(sy, a.xyz[3 * id + 1]);
        sz = O::add(sz, a.xyz[3 * id + 2]);
    }
    const T kk = (T)k;
    const T mx = O::div(sx, kk), my = O::div(sy, kk), mz = O::div(sz, kk);
    T xx = 0, xy = 0, xz = 0, yy = 0, yz = 0, zz = 0;
    for (uint32_t j = 0; j < k; ++j) {
        const uint64_t id = (uint32_t)nb[j];
        const T dx = O::sub(a.xyz[3 * id], mx), dy = O::sub(a.xyz[3 * id + 1], my),
                dz = O::sub(a.xyz[3 * id + 2], mz);
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
    solve<T>(c, a.order, p);
    for (int t = 0; t < a.n_ids; ++t) {
        T v = T(0);
        if (!selected_feature<T>(p, a.ids[t], v)) v = T(0);
        row[t] = v;
    }
}

template <typename T>
int smem_bytes(uint32_t cap, bool in_smem) {
    return (int)(kSearchWarps * (sizeof(WarpSmem<T>) + (in_smem ? (size_t)cap * sizeof(Entry<T>) : 0)));
}

}  // namespace

template <typename T>
int launch_search(const GridIndex<T>& grid, const SPoint<T>* queries, uint64_t m, int mode, uint32_t k, T radius,
                  const SearchOut<T>& out, cudaStream_t s) {
    if (m == 0 || k == 0) return PGEOF_OK;
    if (grid.n == 0) return fail(PGEOF_ERR_INVALID_ARGUMENT, "search over an empty point cloud");
    const DeviceInfo* di;
    PGEOF_TRY(current_device_info(&di));
    // buffer capacity: a power of two comfortably above k
    uint64_t want = mode == MODE_KNN ? std::max<uint64_t>(2ull * k, 128) : std::max<uint64_t>(4ull * k, 256);
    uint32_t cap = 1;
    while (cap < want) cap <<= 1;
    bool in_smem = smem_bytes<T>(cap, true) <= std::min(di->max_smem_optin, 200 * 1024);
    const int smem = smem_bytes<T>(cap, in_smem);
    auto kern = search_kernel<T>;
    if (smem > 48 * 1024) PGEOF_CUDA_TRY(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, smem));
    int per_sm = 0;
    PGEOF_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, kSearchWarps * 32, smem));
    per_sm = std::max(per_sm, 1);
    const uint64_t blocks = std::min<uint64_t>(ceil_div_u(m, kSearchWarps), (uint64_t)di->sm_count * per_sm);
    Scratch gbuf;
    SearchArgs<T> a{};
    if (!in_smem) {
        PGEOF_TRY(gbuf.alloc(blocks * kSearchWarps * (size_t)cap * sizeof(Entry<T>), s));
        a.gbuf = gbuf.as<Entry<T>>();
    }
    a.g = grid.g;
    a.cell_start = grid.cell_start;
    a.pts = grid.pts;
    a.queries = queries;
    a.m = m;
    a.mode = mode;
    a.k = k;
    a.r2 = (T)(radius * radius);  // sq_search_radius in real_t, nn_search.hpp:98
    a.cap = cap;
    a.buf_in_smem = in_smem ? 1 : 0;
    a.out_idx = out.indices;
    a.out_d2 = out.sqr_dist;
    a.out_found = out.found;
    a.fill_last = out.radius_fill_last ? 1 : 0;
    a.err = device_error_word();
    KernelTimer kt(mode == MODE_KNN ? "knn_search_kernel" : "radius_search_kernel", s);
    kern<<<(unsigned)blocks, kSearchWarps * 32, smem, s>>>(a);
    count_launch();
    return check_launch("search_kernel");
}

template <typename T>
int launch_selected_pca(const T* xyz, uint64_t n, const int32_t* nbr, const uint32_t* found, uint32_t max_knn,
                        const int32_t* ids, int n_ids, T* out, cudaStream_t s) {
    if (n == 0 || n_ids == 0) return PGEOF_OK;
    SelArgs<T> a{};
    a.xyz = xyz;
    a.n = n;
    a.nbr = nbr;
    a.found = found;
    a.max_knn = max_knn;
    a.out_ids = n_ids;
    a.order = eig_order();
    a.out = out;
    for (int off = 0; off < n_ids; off += kSelIdsPerLaunch) {
        a.n_ids = std::min(kSelIdsPerLaunch, n_ids - off);
        a.id_offset = off;
        for (int t = 0; t < a.n_ids; ++t) a.ids[t] = ids[off + t];
        KernelTimer kt("selected_pca_kernel", s);
        selected_pca_kernel<T><<<ceil_div_u(n, kSelThreads), kSelThreads, 0, s>>>(a);
        count_launch();
        PGEOF_TRY(check_launch("selected_pca_kernel"));
    }
    return PGEOF_OK;
}

template int launch_search<float>(const GridIndex<float>&, const SPoint<float>*, uint64_t, int, uint32_t, float,
                                  const SearchOut<float>&, cudaStream_t);
template int launch_search<double>(const GridIndex<double>&, const SPoint<double>*, uint64_t, int, uint32_t, double,
                                   const SearchOut<double>&, cudaStream_t);
template int launch_selected_pca<float>(const float*, uint64_t, const int32_t*, const uint32_t*, uint32_t,
                                        const int32_t*, int, float*, cudaStream_t);
template int launch_selected_pca<double>(const double*, uint64_t, const int32_t*, const uint32_t*, uint32_t,
                                         const int32_t*, int, double*, cudaStream_t);

}  // namespace pgeof
