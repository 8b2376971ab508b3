// features.cu -- fused CSR gather -> covariance -> eigen -> feature kernels for
// compute_features, compute_features_multiscale and compute_features_optimal
// (include/pgeof.hpp:75-117, 123-211, 243-310).
//
// One thread owns one point. Its neighbours are swept twice in CSR order: the
// first sweep forms the float mean, the second the centred float products, the
// exact operation order of include/pca.hpp:75-76 (Eigen's column sums run
// sequentially), so the covariance is the one the reference forms. Multiscale
// fills every scale prefix in the same two sweeps (the reference re-gathers
// each prefix): the first keeps one running sum and takes each scale's mean
// after that scale's last neighbour -- the value the reference's own sum over
// the prefix produces -- the second keeps one product accumulator set per
// scale; the scales' covariances then wait in shared memory and one copy of
// the eigen solver handles them in turn. Output rows are staged in shared
// memory and leave the block as one coalesced slab. The few neighbourhoods
// whose float eigenvectors are ill-conditioned are queued and solved exactly
// afterwards by features_exact_kernel.
#include <algorithm>
#include <atomic>
#include <mutex>
#include <string>

#include "eig3.cuh"
#include "kernels.cuh"

namespace pgeof {

namespace {

constexpr int kFeatThreads = 128;
constexpr int kMaxScalesPerLaunch = 8;

struct FeatArgs {
    const float4* xyz4;
    uint32_t n_xyz;
    const uint32_t* nn;
    uint64_t nnz;
    const uint32_t* ptr;
    uint32_t n_points;
    uint32_t k_min;      // FULL mode gate
    int full;            // 1: compute_features (one scale = all neighbours)
    int n_scales;        // scales handled by this launch
    int scale_offset;    // first output scale column of this launch
    int out_scales;      // scales per output row
    uint32_t scales[kMaxScalesPerLaunch];
    int order;
    float* out;
    uint32_t* err;
    // multi-cloud batches: row r belongs to the cloud c with off[c] <= r < off[c+1];
    // its neighbour indices are local to that cloud's slice of xyz4
    const uint64_t* cloud_off;
    int n_clouds;
    const SPoint<float>* row_map;  // optional: row r's output row is row_map[r].idx
    uint32_t uniform_k;            // ptr == nullptr: row r is nn[r * uniform_k, (r + 1) * uniform_k)
    uint32_t row_base;             // this launch covers rows [row_base, row_base + n_points)
    int row_map_input;             // with row_map: row r also reads CSR row row_map[r].idx
    uint32_t slab_words;           // SLAB kernel: index words per warp in shared memory
    // neighbourhoods left to the exact solve: defer[0] counts them, defer[1 ..]
    // holds their output blocks (row * out_scales + scale), whose first six
    // floats carry the covariance until features_exact_kernel replaces them
    unsigned long long* defer;
    uint64_t defer_cap;
};

// Float solve and features of one neighbourhood into f[0..10]; a neighbourhood
// that needs the exact solve gets its covariance in f[0..5] and its output
// block queued for features_exact_kernel. EXACT_INLINE runs the exact solve in
// place instead (callers without a queue).
template <bool EXACT_INLINE>
__device__ __forceinline__ void solve_or_defer(const FeatArgs& a, const Cov<float>& c, uint64_t block, float (&f)[11],
                                               uint32_t& flags) {
    Pca<float> p;
    if constexpr (EXACT_INLINE) {
        bool res;
        pca_solve_f32(c, a.order, p, res);
        features11(p, f);
        return;
    }
    if (pca_solve_f32_fast(c, a.order, p)) {
        features11(p, f);
        return;
    }
    f[0] = c.xx;
    f[1] = c.xy;
    f[2] = c.xz;
    f[3] = c.yy;
    f[4] = c.yz;
    f[5] = c.zz;
#pragma unroll
    for (int q = 6; q < 11; ++q) f[q] = 0.0f;
    const unsigned long long slot = atomicAdd(a.defer, 1ull);
    if (slot < a.defer_cap) a.defer[1 + slot] = block;
    else flags |= ERR_INTERNAL;
}

struct RowCloud {
    const float4* xyz4;
    uint32_t n;
};

__device__ __forceinline__ float4 gather_nb(const float4* xyz4, uint32_t n_xyz, uint32_t id, uint32_t& flags) {
    if (id >= n_xyz) {
        flags |= ERR_NN_RANGE;
        id = 0;
    }
    return __ldg(xyz4 + id);
}

// Calls f(j, point) for the neighbours j = 0 .. count-1 of the CSR row at
// nn + b, in order. Indices are read four at a time (16-byte loads once the
// row pointer is aligned), which quarters the L1 requests for them, and each
// group's four gathers are issued before any is used.
template <typename F>
__device__ __forceinline__ void gather_row(const uint32_t* nn_all, uint64_t b, uint32_t count, const float4* xyz4,
                                           uint32_t n_xyz, uint32_t& flags, F&& f) {
    const uint32_t* nn = nn_all + b;
    uint32_t j = 0;
    while (j < count && (reinterpret_cast<uintptr_t>(nn + j) & 15u)) {
        f(j, gather_nb(xyz4, n_xyz, __ldg(nn + j), flags));
        ++j;
    }
    for (; j + 4 <= count; j += 4) {
        const uint4 ids = __ldg(reinterpret_cast<const uint4*>(nn + j));
        const float4 p0 = gather_nb(xyz4, n_xyz, ids.x, flags), p1 = gather_nb(xyz4, n_xyz, ids.y, flags);
        const float4 p2 = gather_nb(xyz4, n_xyz, ids.z, flags), p3 = gather_nb(xyz4, n_xyz, ids.w, flags);
        f(j, p0);
        f(j + 1, p1);
        f(j + 2, p2);
        f(j + 3, p3);
    }
    for (; j < count; ++j) f(j, gather_nb(xyz4, n_xyz, __ldg(nn + j), flags));
}


// gather_row over indices already in shared memory (idx[0 .. count)).
template <typename F>
__device__ __forceinline__ void gather_row_slab(const uint32_t* idx, uint32_t count, const float4* xyz4,
                                                uint32_t n_xyz, uint32_t& flags, F&& f) {
    uint32_t j = 0;
    for (; j + 4 <= count; j += 4) {
        const uint32_t i0 = idx[j], i1 = idx[j + 1], i2 = idx[j + 2], i3 = idx[j + 3];
        const float4 p0 = gather_nb(xyz4, n_xyz, i0, flags), p1 = gather_nb(xyz4, n_xyz, i1, flags);
        const float4 p2 = gather_nb(xyz4, n_xyz, i2, flags), p3 = gather_nb(xyz4, n_xyz, i3, flags);
        f(j, p0);
        f(j + 1, p1);
        f(j + 2, p2);
        f(j + 3, p3);
    }
    for (; j < count; ++j) f(j, gather_nb(xyz4, n_xyz, idx[j], flags));
}

// SLAB: the CSR indices of a warp's 32 consecutive rows (one contiguous range
// of nn when the rows are in CSR order) are read once into shared memory with
// coalesced loads, and both sweeps take them from there -- instead of each
// thread reading its own row's indices from global memory in both sweeps.
// Rows outside the slab (too long, out of order) read global memory.
//
// EXACT_INLINE: neighbourhoods that need the exact solve get it in place.
// Otherwise they are queued for features_exact_kernel, which keeps the rare
// exact solve (and the stack frame its call needs) out of this kernel: on the
// 1M-point scene the k = 50 single-scale kernel drops from 76 to 44 registers
// and from 0.449 to 0.387 ms, and the few hundred queued solves take one
// double-float solve's latency (~0.016 ms) in features_exact_kernel.
template <int S, bool MULTI, bool SLAB = false, bool EXACT_INLINE = false>
__device__ __forceinline__ void features_body(const FeatArgs& a) {
    extern __shared__ __align__(16) float smem_f[];
    float* stage = smem_f;  // kFeatThreads * n_scales * 11, then SLAB: a.slab_words per warp
    const int tid = threadIdx.x;
    const uint32_t i = a.row_base + blockIdx.x * kFeatThreads + tid;
    const int row_w = a.n_scales * 11;
    for (int f = 0; f < row_w; ++f) stage[f * kFeatThreads + tid] = 0.0f;  // column-major staging

    uint32_t flags = 0;
    const bool row_ok = i < a.row_base + a.n_points;
    uint64_t b = 0, e = 0;
    if (row_ok) {
        const uint32_t ri = a.row_map_input ? a.row_map[i].idx : i;
        if (a.ptr) {
            b = __ldg(a.ptr + ri);
            e = __ldg(a.ptr + ri + 1);
        } else {
            b = (uint64_t)i * a.uniform_k;
            e = b + a.uniform_k;
        }
    }
    const uint32_t* slab_idx = nullptr;  // this row's indices in shared memory
    if constexpr (SLAB) {
        const int lane = tid & 31;
        const uint32_t vmask = __ballot_sync(0xffffffffu, row_ok);
        if (vmask && !a.row_map_input) {
            const int last = 31 - __clz(vmask);  // valid rows are a prefix of the warp
            const uint64_t s0 = __shfl_sync(0xffffffffu, b, 0), s1 = __shfl_sync(0xffffffffu, e, last);
            if (s1 >= s0 && s1 - s0 <= a.slab_words && s1 <= a.nnz) {
                uint32_t* slab = reinterpret_cast<uint32_t*>(stage + (size_t)kFeatThreads * row_w) +
                                 (size_t)(tid >> 5) * a.slab_words;
                for (uint32_t w = lane; w < (uint32_t)(s1 - s0); w += 32) slab[w] = __ldg(a.nn + s0 + w);
                __syncwarp();
                if (row_ok && b >= s0 && e <= s1 && e >= b) slab_idx = slab + (b - s0);
            }
        }
    }
    if (row_ok) {
        uint32_t k_nn = 0;
        if (e < b || e > a.nnz) {
            flags |= ERR_PTR_RANGE;
        } else {
            k_nn = (uint32_t)(e - b);
        }
        RowCloud rc{a.xyz4, a.n_xyz};
        if (MULTI) {
            int lo = 0, hi = a.n_clouds - 1;
            while (lo < hi) {
                const int mid = (lo + hi + 1) >> 1;
                if (a.cloud_off[mid] <= i) lo = mid;
                else hi = mid - 1;
            }
            rc.xyz4 = a.xyz4 + a.cloud_off[lo];
            rc.n = (uint32_t)(a.cloud_off[lo + 1] - a.cloud_off[lo]);
        }
        uint32_t ks[S];
        int n_active = 0;
        uint32_t kmax = 0;
#pragma unroll
        for (int s = 0; s < S; ++s) {
            ks[s] = a.full ? k_nn : a.scales[s];
            bool act;
            if (a.full) {
                act = s == 0 && k_nn >= a.k_min;
            } else {
                act = s < a.n_scales && k_nn >= ks[s] && n_active == s;  // break at the first short scale
            }
            if (act) {
                n_active = s + 1;
                kmax = ks[s] > kmax ? ks[s] : kmax;
            }
        }
        // output block of scale s of this row
        const auto out_block = [&](int s) -> uint64_t {
            const uint64_t dst = a.row_map ? (uint64_t)a.row_map[i].idx : (uint64_t)i;
            return dst * (uint64_t)a.out_scales + (uint64_t)(a.scale_offset + s);
        };
        if (n_active > 0) {
            // neighbours [j0, j1) of the row in order, indices from the slab or global memory
            const auto sweep = [&](uint32_t j0, uint32_t j1, auto&& f) {
                if (SLAB && slab_idx) {
                    gather_row_slab(slab_idx + j0, j1 - j0, rc.xyz4, rc.n, flags, f);
                } else {
                    gather_row(a.nn, b + j0, j1 - j0, rc.xyz4, rc.n, flags, f);
                }
            };
            // sweep 1: one sequential float sum over the neighbours; every scale
            // is a prefix of the same list summed from the first neighbour, so
            // its sum is this running sum after its last neighbour
            float rx = 0.0f, ry = 0.0f, rz = 0.0f;
            float mx[S], my[S], mz[S];
#pragma unroll
            for (int s = 0; s < S; ++s) mx[s] = my[s] = mz[s] = 0.0f;
            // both sweeps run in segments [ks[t-1], ks[t]) between the (ascending)
            // scale sizes, so each neighbour updates only the scales that contain it
            uint32_t j0 = 0;
#pragma unroll
            for (int t = 0; t < S; ++t) {
                if (t < n_active) {
                    const uint32_t j1 = ks[t];
                    sweep(j0, j1, [&](uint32_t, const float4& p) {
                        rx = FADD(rx, p.x);
                        ry = FADD(ry, p.y);
                        rz = FADD(rz, p.z);
                    });
                    const float kk = (float)j1;
                    mx[t] = FDIV(rx, kk);
                    my[t] = FDIV(ry, kk);
                    mz[t] = FDIV(rz, kk);
                    j0 = j1;
                }
            }
            // sweep 2: centred products, sequential sums
            float cxx[S], cxy[S], cxz[S], cyy[S], cyz[S], czz[S];
#pragma unroll
            for (int s = 0; s < S; ++s) cxx[s] = cxy[s] = cxz[s] = cyy[s] = cyz[s] = czz[s] = 0.0f;
            j0 = 0;
#pragma unroll
            for (int t = 0; t < S; ++t) {
                if (t < n_active) {
                    const uint32_t j1 = ks[t];
                    sweep(j0, j1, [&](uint32_t, const float4& p) {
#pragma unroll
                        for (int s = t; s < S; ++s) {
                            if (s < n_active) {
                                const float dx = FSUB(p.x, mx[s]);
                                const float dy = FSUB(p.y, my[s]);
                                const float dz = FSUB(p.z, mz[s]);
                                cxx[s] = FADD(cxx[s], FMUL(dx, dx));
                                cxy[s] = FADD(cxy[s], FMUL(dx, dy));
                                cxz[s] = FADD(cxz[s], FMUL(dx, dz));
                                cyy[s] = FADD(cyy[s], FMUL(dy, dy));
                                cyz[s] = FADD(cyz[s], FMUL(dy, dz));
                                czz[s] = FADD(czz[s], FMUL(dz, dz));
                            }
                        }
                    });
                    j0 = j1;
                }
            }
            if constexpr (S == 1) {
                const float kk = (float)ks[0];
                Cov<float> c;
                c.xx = FDIV(cxx[0], kk);
                c.xy = FDIV(cxy[0], kk);
                c.xz = FDIV(cxz[0], kk);
                c.yy = FDIV(cyy[0], kk);
                c.yz = FDIV(cyz[0], kk);
                c.zz = FDIV(czz[0], kk);
                float f[11];
                solve_or_defer<EXACT_INLINE>(a, c, out_block(0), f, flags);
#pragma unroll
                for (int q = 0; q < 11; ++q) stage[q * kFeatThreads + tid] = f[q];
            } else {
                // park each scale's covariance in its staging slot, then solve the
                // scales one at a time (one copy of the solver, not S)
#pragma unroll
                for (int s = 0; s < S; ++s) {
                    if (s < n_active) {
                        const float kk = (float)ks[s];
                        float* st = stage + (s * 11) * kFeatThreads + tid;
                        st[0 * kFeatThreads] = FDIV(cxx[s], kk);
                        st[1 * kFeatThreads] = FDIV(cxy[s], kk);
                        st[2 * kFeatThreads] = FDIV(cxz[s], kk);
                        st[3 * kFeatThreads] = FDIV(cyy[s], kk);
                        st[4 * kFeatThreads] = FDIV(cyz[s], kk);
                        st[5 * kFeatThreads] = FDIV(czz[s], kk);
                    }
                }
#pragma unroll 1
                for (int s = 0; s < n_active; ++s) {
                    float* st = stage + (s * 11) * kFeatThreads + tid;
                    Cov<float> c;
                    c.xx = st[0 * kFeatThreads];
                    c.xy = st[1 * kFeatThreads];
                    c.xz = st[2 * kFeatThreads];
                    c.yy = st[3 * kFeatThreads];
                    c.yz = st[4 * kFeatThreads];
                    c.zz = st[5 * kFeatThreads];
                    float f[11];
                    solve_or_defer<EXACT_INLINE>(a, c, out_block(s), f, flags);
#pragma unroll
                    for (int q = 0; q < 11; ++q) st[q * kFeatThreads] = f[q];
                }
            }
        }
    }
    if (flags) atomicOr(a.err, flags);
    __syncthreads();
    // coalesced write-out of the block's rows
    const uint32_t row0 = a.row_base + blockIdx.x * kFeatThreads;
    const uint32_t rows = min((uint32_t)kFeatThreads, a.row_base + a.n_points - row0);
    if (a.row_map) {
        // rows processed in another order: each row goes to its mapped output row
        const int out_w = a.out_scales * 11;
        for (int t = tid; t < (int)rows * row_w; t += kFeatThreads) {
            const int r = t / row_w, c = t - r * row_w;
            const uint64_t dst = a.row_map[row0 + r].idx;
            a.out[dst * out_w + a.scale_offset * 11 + c] = stage[c * kFeatThreads + r];
        }
    } else if (a.n_scales == a.out_scales) {
        float* dst = a.out + (uint64_t)row0 * row_w;
        const int total = rows * row_w;
        for (int t = tid; t < total; t += kFeatThreads) {
            const int r = t / row_w, c = t - r * row_w;
            dst[t] = stage[c * kFeatThreads + r];
        }
    } else {
        const int out_w = a.out_scales * 11;
        for (int t = tid; t < (int)rows * row_w; t += kFeatThreads) {
            const int r = t / row_w, c = t - r * row_w;
            a.out[(uint64_t)(row0 + r) * out_w + a.scale_offset * 11 + c] = stage[c * kFeatThreads + r];
        }
    }
}

template <int S, bool MULTI, bool SLAB = false, bool EXACT_INLINE = false>
__global__ void __launch_bounds__(kFeatThreads) features_kernel(const __grid_constant__ FeatArgs a) {
    features_body<S, MULTI, SLAB, EXACT_INLINE>(a);
}

// The 3-scale pass (compute_features_multiscale with three scales, the
// 1M-point benchmark's case) compiled for 8 resident blocks per SM: 64
// registers and a 44-byte spill instead of 76 registers and 6 blocks (0.607 ->
// 0.591 ms on the 1M-point scene).
template <bool MULTI>
__global__ void __launch_bounds__(kFeatThreads, 8) features3_kernel(const __grid_constant__ FeatArgs a) {
    features_body<3, MULTI, false, false>(a);
}


// Coordinates of each CSR row's first neighbour (point 0's for an empty or
// invalid row): the key by which rows are ordered in space.
__global__ void first_nb_kernel(const float* __restrict__ xyz, uint64_t n_xyz, const uint32_t* __restrict__ nn,
                                uint64_t nnz, const uint32_t* __restrict__ ptr, uint64_t n_rows,
                                float* __restrict__ out) {
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n_rows;
         i += (uint64_t)gridDim.x * blockDim.x) {
        const uint64_t b = ptr[i], e = ptr[i + 1];
        uint64_t id = 0;
        if (e > b && b < nnz) {
            id = nn[b];
            if (id >= n_xyz) id = 0;
        }
        out[3 * i] = xyz[3 * id];
        out[3 * i + 1] = xyz[3 * id + 1];
        out[3 * i + 2] = xyz[3 * id + 2];
    }
}

// The exact (float64) solve of the neighbourhoods features_kernel queued: each
// queued output block holds its float covariance in its first six floats and
// gets its 11 features in their place.
__global__ void __launch_bounds__(128) features_exact_kernel(float* __restrict__ out,
                                                             const unsigned long long* __restrict__ defer,
                                                             uint64_t cap, int order, unsigned long long* resolved) {
    const uint64_t n = min((uint64_t)defer[0], cap);
    if (resolved && blockIdx.x == 0 && threadIdx.x == 0 && n) atomicAdd(resolved, (unsigned long long)n);
    // one solve per thread: the kernel's time is one solve's latency
    for (uint64_t t = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += (uint64_t)gridDim.x * blockDim.x) {
        float* o = out + defer[1 + t] * 11;
        const Cov<float> c{o[0], o[1], o[2], o[3], o[4], o[5]};
        Pca<float> p;
        pca_solve_refined(c, order, p);
        float f[11];
        features11(p, f);
#pragma unroll
        for (int q = 0; q < 11; ++q) o[q] = f[q];
    }
}

__global__ void pad_xyz_kernel(const float* __restrict__ xyz, uint64_t n, float4* __restrict__ out) {
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
        out[i] = make_float4(xyz[3 * i], xyz[3 * i + 1], xyz[3 * i + 2], 0.0f);
    }
}

// ------------------------------------------------------------------ optimal
constexpr int kOptThreads = 128;
constexpr int kOptSlots = 64;  // eigentropy values kept per point for the near-tie pass

struct OptArgs {
    const float4* xyz4;
    uint32_t n_xyz;
    const uint32_t* nn;
    uint64_t nnz;
    const uint32_t* ptr;
    uint32_t n_points;
    uint32_t k_min, k_step, k_min_search;
    int order;
    float* out;  // (n, 12)
    uint32_t* err;
    unsigned long long* stats;  // [0] exact tie re-evaluations, [1] double re-solves
};

// Kahan-compensated running sum.
struct KSum {
    float s = 0.0f, c = 0.0f;
    __device__ __forceinline__ void add(float x) {
        const float y = FSUB(x, c);
        const float t = FADD(s, y);
        c = FSUB(FSUB(t, s), y);
        s = t;
    }
};

// Eigenvalues of a symmetric 3x3 by the trigonometric closed form (O. K.
// Smith, "Eigenvalues of a symmetric 3x3 matrix", CACM 4(4), 1961), used only
// to rank candidate neighbourhood sizes. The scan ranks candidate sizes and every size within
// kTieBand (3e-5) of its minimum is re-evaluated exactly, so the scan's values
// need only stay within half the band of the exact ones. The hardware cosine
// and logarithm (__cosf: absolute error < 2^-21 on [-pi, pi]; __logf) add about
// 1e-6 to the eigentropy -- well inside it.
__device__ __forceinline__ void eigvals_closed_form_scan(const Cov<float>& c, float (&w)[3]) {
    const float q = (c.xx + c.yy + c.zz) * (1.0f / 3.0f);
    const float b00 = c.xx - q, b11 = c.yy - q, b22 = c.zz - q;
    const float off = c.xy * c.xy + c.xz * c.xz + c.yz * c.yz;
    const float p2 = (b00 * b00 + b11 * b11 + b22 * b22 + 2.0f * off) * (1.0f / 6.0f);
    if (!(p2 > 0.0f)) {
        w[0] = w[1] = w[2] = q;
        return;
    }
    const float p = sqrtf(p2);
    const float det = b00 * (b11 * b22 - c.yz * c.yz) - c.xy * (c.xy * b22 - c.yz * c.xz) +
                      c.xz * (c.xy * c.yz - b11 * c.xz);
    float r = __fdividef(det, 2.0f * p2 * p);
    r = fminf(1.0f, fmaxf(-1.0f, r));
    const float phi = acosf(r) * (1.0f / 3.0f);
    const float e2 = q + 2.0f * p * __cosf(phi);
    const float e0 = q + 2.0f * p * __cosf(phi + 2.0943951023931953f);
    w[0] = e0;
    w[2] = e2;
    w[1] = 3.0f * q - e0 - e2;
}

// include/pca.hpp:140-150 with the hardware logarithm (scan ranking only).
__device__ __forceinline__ float eigentropy_scan(const float (&val)[3]) {
    const float eps = 1e-3f;
    const float inv = __fdividef(1.0f, val[0] + val[1] + val[2] + eps);
    const float e0 = val[0] * inv, e1 = val[1] * inv, e2 = val[2] * inv;
    return -(e0 * __logf(e0 + eps) + e1 * __logf(e1 + eps) + e2 * __logf(e2 + eps));
}

// Covariance of the first k neighbours exactly as include/pca.hpp:75-76.
__device__ __forceinline__ Cov<float> literal_cov(const OptArgs& a, uint32_t b, uint32_t k, uint32_t& flags) {
    // scalar index loads here: the 4-wide form costs this kernel ~20 registers
    float sx = 0.0f, sy = 0.0f, sz = 0.0f;
    for (uint32_t j = 0; j < k; ++j) {
        const float4 p = gather_nb(a.xyz4, a.n_xyz, __ldg(a.nn + b + j), flags);
        sx = FADD(sx, p.x);
        sy = FADD(sy, p.y);
        sz = FADD(sz, p.z);
    }
    const float kk = (float)k;
    const float mx = FDIV(sx, kk), my = FDIV(sy, kk), mz = FDIV(sz, kk);
    float xx = 0.0f, xy = 0.0f, xz = 0.0f, yy = 0.0f, yz = 0.0f, zz = 0.0f;
    for (uint32_t j = 0; j < k; ++j) {
        const float4 p = gather_nb(a.xyz4, a.n_xyz, __ldg(a.nn + b + j), flags);
        const float dx = FSUB(p.x, mx), dy = FSUB(p.y, my), dz = FSUB(p.z, mz);
        xx = FADD(xx, FMUL(dx, dx));
        xy = FADD(xy, FMUL(dx, dy));
        xz = FADD(xz, FMUL(dx, dz));
        yy = FADD(yy, FMUL(dy, dy));
        yz = FADD(yz, FMUL(dy, dz));
        zz = FADD(zz, FMUL(dz, dz));
    }
    Cov<float> c;
    c.xx = FDIV(xx, kk);
    c.xy = FDIV(xy, kk);
    c.xz = FDIV(xz, kk);
    c.yy = FDIV(yy, kk);
    c.yz = FDIV(yz, kk);
    c.zz = FDIV(zz, kk);
    return c;
}

__device__ __forceinline__ bool evaluated(uint32_t k, uint32_t k0, uint32_t k_nn, uint32_t step) {
    return k == k0 || k % step == 0 || k == k_nn;
}

// include/pgeof.hpp:264-299. Candidate sizes are ranked by eigentropy from
// compensated prefix moments (O(k) gathers instead of the reference's O(k^2));
// every size whose fast eigentropy lies within kTieBand of the fast minimum is
// then re-evaluated from the reference's own covariance and an exact eigen
// solve, and the smallest exact eigentropy wins (first k on equality -- the
// reference's strict '<' scan). Features come from the winning size's
// reference covariance.
__global__ void __launch_bounds__(kOptThreads) optimal_kernel(const __grid_constant__ OptArgs a) {
    constexpr float kTieBand = 3e-5f;
    __shared__ float ent[kOptSlots * kOptThreads];
    __shared__ float stage[12 * kOptThreads];
    const int tid = threadIdx.x;
    const uint32_t i = blockIdx.x * kOptThreads + tid;
#pragma unroll
    for (int f = 0; f < 12; ++f) stage[f * kOptThreads + tid] = 0.0f;
    uint32_t flags = 0;
    unsigned n_exact = 0, n_resolved = 0;
    if (i < a.n_points) {
        const uint32_t b = __ldg(a.ptr + i), e = __ldg(a.ptr + i + 1);
        uint32_t k_nn = 0;
        bool ok = true;
        if (e < b || (uint64_t)e > a.nnz) {
            flags |= ERR_PTR_RANGE;
            ok = false;
        } else {
            k_nn = e - b;
        }
        if (ok && k_nn >= a.k_min && k_nn >= a.k_min_search && k_nn > 0) {
            uint32_t k0 = max(a.k_min, a.k_min_search);
            k0 = min(k0, k_nn);
            // fast scan over prefix moments, shifted by the first neighbour
            uint32_t id0 = __ldg(a.nn + b);
            if (id0 >= a.n_xyz) {
                flags |= ERR_NN_RANGE;
                id0 = 0;
            }
            const float4 p0 = __ldg(a.xyz4 + id0);
            KSum s1x, s1y, s1z, sxx, sxy, sxz, syy, syz, szz;
            float best = 0.0f;
            int slot = 0;
            bool stored_all = true;
            for (uint32_t k = 1; k <= k_nn; ++k) {
                const float4 p = gather_nb(a.xyz4, a.n_xyz, __ldg(a.nn + b + k - 1), flags);
                const float dx = p.x - p0.x, dy = p.y - p0.y, dz = p.z - p0.z;
                s1x.add(dx);
                s1y.add(dy);
                s1z.add(dz);
                sxx.add(dx * dx);
                sxy.add(dx * dy);
                sxz.add(dx * dz);
                syy.add(dy * dy);
                syz.add(dy * dz);
                szz.add(dz * dz);
                if (k < k0 || !evaluated(k, k0, k_nn, a.k_step)) continue;
                const float inv = 1.0f / (float)k;
                const float mx = s1x.s * inv, my = s1y.s * inv, mz = s1z.s * inv;
                Cov<float> c;
                c.xx = sxx.s * inv - mx * mx;
                c.xy = sxy.s * inv - mx * my;
                c.xz = sxz.s * inv - mx * mz;
                c.yy = syy.s * inv - my * my;
                c.yz = syz.s * inv - my * mz;
                c.zz = szz.s * inv - mz * mz;
                float w[3];
                eigvals_closed_form_scan(c, w);
                float val[3];
#pragma unroll
                for (int q = 0; q < 3; ++q) val[q] = fmaxf(w[a.order ? 2 - q : q], 0.0f);
                const float ent_k = eigentropy_scan(val);
                if (k == k0 || ent_k < best) best = ent_k;
                if (slot < kOptSlots) {
                    ent[slot * kOptThreads + tid] = ent_k;
                } else {
                    stored_all = false;
                }
                ++slot;
            }
            // candidates within the tie band of the fast minimum
            int n_cand = 0;
            for (int sidx = 0; sidx < min(slot, kOptSlots); ++sidx)
                if (ent[sidx * kOptThreads + tid] <= best + kTieBand) ++n_cand;
            uint32_t k_opt = k0;
            if (stored_all && n_cand == 1) {
                // unique winner: find its k
                int sidx = 0;
                for (uint32_t k = k0; k <= k_nn; ++k) {
                    if (!evaluated(k, k0, k_nn, a.k_step)) continue;
                    if (ent[sidx * kOptThreads + tid] <= best + kTieBand) {
                        k_opt = k;
                        break;
                    }
                    ++sidx;
                }
            } else {
                // near-ties (or too many sizes to store): exact re-evaluation
                float best_exact = 0.0f;
                bool have = false;
                int sidx = 0;
                for (uint32_t k = k0; k <= k_nn; ++k) {
                    if (!evaluated(k, k0, k_nn, a.k_step)) continue;
                    bool cand = true;
                    if (stored_all) cand = ent[sidx * kOptThreads + tid] <= best + kTieBand;
                    ++sidx;
                    if (!cand) continue;
                    ++n_exact;
                    const Cov<float> c = literal_cov(a, b, k, flags);
                    Pca<float> pk;
                    pca_solve_f64<float>(c, a.order, &pk);
                    const float ek = eigentropy_of<float>(pk.val);
                    if (!have || ek < best_exact) {
                        best_exact = ek;
                        k_opt = k;
                        have = true;
                    }
                }
            }
            const Cov<float> c = literal_cov(a, b, k_opt, flags);
            Pca<float> p;
            bool res;
            pca_solve_f32(c, a.order, p, res);
            n_resolved += res;
            float f[11];
            features11(p, f);
#pragma unroll
            for (int q = 0; q < 11; ++q) stage[q * kOptThreads + tid] = f[q];
            stage[11 * kOptThreads + tid] = (float)k_opt;
        }
    }
    if (flags) atomicOr(a.err, flags);
    if (a.stats) {
        if (n_exact) atomicAdd(a.stats, (unsigned long long)n_exact);
        if (n_resolved) atomicAdd(a.stats + 1, (unsigned long long)n_resolved);
    }
    __syncthreads();
    const uint32_t row0 = blockIdx.x * kOptThreads;
    const uint32_t rows = min((uint32_t)kOptThreads, a.n_points - row0);
    float* dst = a.out + (uint64_t)row0 * 12;
    for (int t = tid; t < (int)rows * 12; t += kOptThreads) {
        const int r = t / 12, c = t - r * 12;
        dst[t] = stage[c * kOptThreads + r];
    }
}

}  // namespace

int pad_xyz(const float* xyz, uint64_t n, float4* out, cudaStream_t s) {
    if (n == 0) return PGEOF_OK;
    const DeviceInfo* di;
    PGEOF_TRY(current_device_info(&di));
    const unsigned blocks = (unsigned)std::min<uint64_t>(ceil_div_u(n, 256), (uint64_t)di->sm_count * 8);
    KernelTimer kt("pad_xyz_kernel", s);
    pad_xyz_kernel<<<blocks, 256, 0, s>>>(xyz, n, out);
    count_launch();
    return check_launch("pad_xyz_kernel");
}

// Index slabs (SLAB kernel) for single-scale passes; PGEOF_FEATURE_SLAB=0
// turns them off.
bool use_index_slab() {
    static const bool v = [] {
        const char* e = getenv("PGEOF_FEATURE_SLAB");
        return e ? atoi(e) != 0 : true;
    }();
    return v;
}

template <int S>
static int launch_features_s(const FeatArgs& a, cudaStream_t s) {
    const size_t stage_bytes = (size_t)kFeatThreads * a.n_scales * 11 * sizeof(float);
    const unsigned blocks = ceil_div_u(a.n_points, kFeatThreads);
    KernelTimer kt("features_kernel", s);
    const bool slab = a.slab_words > 0;
    using Kern = void (*)(const FeatArgs);
    Kern kern = slab ? (a.n_clouds > 0 ? features_kernel<S, true, true> : features_kernel<S, false, true>)
                     : (a.n_clouds > 0 ? features_kernel<S, true> : features_kernel<S, false>);
    if constexpr (S == 3) {
        if (!slab) kern = a.n_clouds > 0 ? features3_kernel<true> : features3_kernel<false>;
    }
    const size_t smem = stage_bytes + (slab ? (size_t)(kFeatThreads / 32) * a.slab_words * sizeof(uint32_t) : 0);
    PGEOF_TRY(cap_smem_carveout((const void*)kern, kFeatThreads, (int)smem));
    kern<<<blocks, kFeatThreads, smem, s>>>(a);
    count_launch();
    return check_launch("features_kernel");
}

static int launch_features_exact(float* out, const unsigned long long* defer, uint64_t cap,
                                 unsigned long long* resolved, cudaStream_t s) {
    const DeviceInfo* di;
    PGEOF_TRY(current_device_info(&di));
    const unsigned blocks = (unsigned)std::min<uint64_t>(ceil_div_u(cap, 128), (uint64_t)di->sm_count * 2);
    KernelTimer kt("features_exact_kernel", s);
    features_exact_kernel<<<blocks, 128, 0, s>>>(out, defer, cap, eig_order(), resolved);
    count_launch();
    return check_launch("features_exact_kernel");
}

static int launch_features_impl(FeatArgs& a, uint64_t n_points, bool full, uint64_t k_min, const uint32_t* scales,
                                int n_scales, uint64_t nnz, uint32_t uniform_k, cudaStream_t s);

int launch_features(const float4* xyz4, uint64_t n_xyz, const uint32_t* nn, uint64_t nnz, const uint32_t* ptr,
                    uint64_t n_points, bool full, uint64_t k_min, const uint32_t* scales, int n_scales,
                    float* out, unsigned long long* resolved, cudaStream_t s, const uint64_t* cloud_off,
                    int n_clouds, const SPoint<float>* row_map, uint32_t uniform_k, uint64_t row_base,
                    bool row_map_input, unsigned long long* defer) {
    if (n_points == 0) return PGEOF_OK;
    if (!full && n_scales <= 0) return PGEOF_OK;
    // queue for the exact solves: a count and one slot per output block
    const uint64_t cap = n_points * (uint64_t)(full ? 1 : n_scales);
    Scratch own;
    if (!defer) {
        PGEOF_TRY(own.alloc((cap + 1) * sizeof(unsigned long long), s));
        defer = own.as<unsigned long long>();
    }
    PGEOF_CUDA_TRY(cudaMemsetAsync(defer, 0, sizeof(unsigned long long), s));
    FeatArgs a{};
    a.defer = defer;
    a.defer_cap = cap;
    a.row_map = row_map;
    a.row_map_input = row_map && row_map_input ? 1 : 0;
    a.uniform_k = uniform_k;
    a.row_base = (uint32_t)row_base;
    a.cloud_off = cloud_off;
    a.n_clouds = cloud_off ? n_clouds : 0;
    a.xyz4 = xyz4;
    a.n_xyz = (uint32_t)n_xyz;
    a.nn = nn;
    a.nnz = nnz;
    a.ptr = ptr;
    a.n_points = (uint32_t)n_points;
    a.order = eig_order();
    a.err = device_error_word();
    a.out = out;
    PGEOF_TRY(launch_features_impl(a, n_points, full, k_min, scales, n_scales, nnz, uniform_k, s));
    return launch_features_exact(out, defer, cap, resolved, s);
}

static int launch_features_impl(FeatArgs& a, uint64_t n_points, bool full, uint64_t k_min, const uint32_t* scales,
                                int n_scales, uint64_t nnz, uint32_t uniform_k, cudaStream_t s) {
    if (full) {
        a.full = 1;
        a.k_min = (uint32_t)std::min<uint64_t>(k_min, 0xffffffffull);
        a.n_scales = 1;
        a.out_scales = 1;
        a.scale_offset = 0;
        // Index slab sized for the average row (warps whose rows run longer
        // read global memory). Single-scale passes only: on the 1M-point scene
        // it takes the k = 50 compute_features pass from 0.437 to 0.388 ms and
        // k = 20 from 0.172 to 0.171 ms, but the 3-scale pass from 0.607 to
        // 0.613 ms. A larger slab than the rows need costs resident blocks
        // (k = 50 rows in a 64-neighbour slab: 0.399 ms).
        const uint64_t ks = uniform_k ? uniform_k : (nnz + n_points - 1) / n_points;
        a.slab_words = use_index_slab() && !a.row_map_input && ks >= 1 && ks <= 128 ? 32u * (uint32_t)ks + 4u : 0u;
        return launch_features_s<1>(a, s);
    }
    a.full = 0;
    a.out_scales = n_scales;
    for (int s0 = 0; s0 < n_scales; s0 += kMaxScalesPerLaunch) {
        const int cnt = std::min(kMaxScalesPerLaunch, n_scales - s0);
        a.n_scales = cnt;
        a.scale_offset = s0;
        for (int q = 0; q < cnt; ++q) a.scales[q] = scales[s0 + q];
        a.slab_words = 0;
        int st;
        if (cnt == 1) st = launch_features_s<1>(a, s);
        else if (cnt == 2) st = launch_features_s<2>(a, s);
        else if (cnt == 3) st = launch_features_s<3>(a, s);
        else if (cnt == 4) st = launch_features_s<4>(a, s);
        else if (cnt <= 6) st = launch_features_s<6>(a, s);
        else st = launch_features_s<8>(a, s);
        if (st != PGEOF_OK) return st;
    }
    return PGEOF_OK;
}

int first_neighbour_xyz(const float* xyz, uint64_t n_xyz, const uint32_t* nn, uint64_t nnz, const uint32_t* ptr,
                        uint64_t n_rows, float* out, cudaStream_t s) {
    if (n_rows == 0) return PGEOF_OK;
    const DeviceInfo* di;
    PGEOF_TRY(current_device_info(&di));
    KernelTimer kt("row_order_kernels", s);
    first_nb_kernel<<<std::min<unsigned>(ceil_div_u(n_rows, 256), (unsigned)di->sm_count * 8), 256, 0, s>>>(
        xyz, n_xyz, nn, nnz, ptr, n_rows, out);
    count_launch();
    return check_launch("first_nb_kernel");
}

int launch_optimal(const float4* xyz4, uint64_t n_xyz, const uint32_t* nn, uint64_t nnz, const uint32_t* ptr,
                   uint64_t n_points, uint32_t k_min, uint32_t k_step, uint32_t k_min_search, float* out,
                   unsigned long long* stats, cudaStream_t s) {
    if (n_points == 0) return PGEOF_OK;
    OptArgs a{};
    a.xyz4 = xyz4;
    a.n_xyz = (uint32_t)n_xyz;
    a.nn = nn;
    a.nnz = nnz;
    a.ptr = ptr;
    a.n_points = (uint32_t)n_points;
    a.k_min = k_min;
    a.k_step = k_step;
    a.k_min_search = k_min_search;
    a.order = eig_order();
    a.out = out;
    a.err = device_error_word();
    a.stats = stats;
    KernelTimer kt("optimal_kernel", s);
    optimal_kernel<<<ceil_div_u(n_points, kOptThreads), kOptThreads, 0, s>>>(a);
    count_launch();
    return check_launch("optimal_kernel");
}

}  // namespace pgeof

// ===========================================================================
// compute_features without any allocation (pgeof_compute_features_f32_noalloc)
//
// Some callers cannot allocate GPU memory while they call us: code running
// under a fixed device-memory budget that was reserved up front (a serving
// process that pre-sizes every buffer so it can never fail mid-request), hosts
// whose own allocator owns the device heap and forbids foreign cudaMalloc /
// pool traffic, and real-time loops where an allocation's latency or
// implicit synchronisation is not acceptable. For them this entry point
// keeps its only scratch -- the float4-padded copy of xyz that the feature
// kernel gathers from -- in the fixed array below instead of in freshly
// allocated memory. The caller still owns and passes every input and output.
//
// The array is file-scope device memory: every GPU that loads this library
// holds it (16 MiB) until the process exits, and every call shares it. Calls
// that overlap on the GPU (two streams, or two host threads) race on it and
// must be serialised by the caller. Host code only ever sees a host-side
// stand-in for the array's name, so the device address is fetched with
// cudaGetSymbolAddress on the first call on each device, with that device
// current; make that first call before any stream capture.
// ===========================================================================
static __device__ __align__(256) float4 g_noalloc_xyz4[1u << 20];
static __device__ __align__(256) uint32_t g_noalloc_err[64];

namespace pgeof {
namespace {

constexpr uint64_t kNoAllocMaxPoints = 1u << 20;  // capacity of g_noalloc_xyz4, in points
constexpr int kNoAllocMaxDevices = 64;

struct NoAllocSetup {
    std::mutex mu;
    std::atomic<bool> ready{false};
    float4* xyz4 = nullptr;   // device address of g_noalloc_xyz4
    uint32_t* err = nullptr;  // device address of g_noalloc_err
};
NoAllocSetup g_noalloc_setup[kNoAllocMaxDevices];

// Looks the arrays' device addresses up once per device. Only success is
// cached: a failed lookup (e.g. attempted during a stream capture) clears the
// error it left and is retried by the next call.
cudaError_t noalloc_setup(NoAllocSetup& st) {
    if (st.ready.load(std::memory_order_acquire)) return cudaSuccess;
    std::lock_guard<std::mutex> lk(st.mu);
    if (st.ready.load(std::memory_order_relaxed)) return cudaSuccess;
    float4* xyz4 = nullptr;
    uint32_t* err = nullptr;
    cudaError_t e = cudaGetSymbolAddress((void**)&xyz4, g_noalloc_xyz4);
    if (e == cudaSuccess) e = cudaGetSymbolAddress((void**)&err, g_noalloc_err);
    if (e != cudaSuccess) {
        (void)cudaGetLastError();
        return e;
    }
    st.xyz4 = xyz4;
    st.err = err;
    st.ready.store(true, std::memory_order_release);
    return cudaSuccess;
}

}  // namespace
}  // namespace pgeof

namespace pgeof {
int noalloc_take_errors(uint32_t* bits) {
    *bits = 0;
    int dev = -1;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kNoAllocMaxDevices) {
        (void)cudaGetLastError();
        return PGEOF_OK;  // no device: nothing was ever recorded
    }
    NoAllocSetup& st = g_noalloc_setup[dev];
    if (!st.ready.load(std::memory_order_acquire)) return PGEOF_OK;  // no call on this device yet
    PGEOF_CUDA_TRY(cudaMemcpy(bits, st.err, sizeof(uint32_t), cudaMemcpyDeviceToHost));
    if (*bits) PGEOF_CUDA_TRY(cudaMemset(st.err, 0, sizeof(uint32_t)));
    return PGEOF_OK;
}
}  // namespace pgeof

extern "C" int pgeof_compute_features_f32_noalloc(const float* xyz, int64_t n_xyz, const uint32_t* nn, int64_t nnz,
                                                  const uint32_t* nn_ptr, int64_t n_points, uint64_t k_min,
                                                  float* features, uint32_t* error_bits, pgeof_stream_t stream) {
    using namespace pgeof;
    // the same argument checks as pgeof_compute_features_f32, then the capacity
    if (k_min < 1) return fail(PGEOF_ERR_INVALID_ARGUMENT, "k_min should be > 1");
    if (n_xyz < 0 || nnz < 0) return fail(PGEOF_ERR_INVALID_ARGUMENT, "negative size");
    if (n_points < 0) return fail(PGEOF_ERR_INVALID_ARGUMENT, "nn_ptr must hold at least one entry");
    if ((uint64_t)n_xyz > kNoAllocMaxPoints)
        return fail(PGEOF_ERR_INVALID_ARGUMENT,
                    "xyz has " + std::to_string(n_xyz) + " points; pgeof_compute_features_f32_noalloc holds at most " +
                        std::to_string(kNoAllocMaxPoints) + " (use pgeof_compute_features_f32)");
    if ((uint64_t)n_points > 0xfffffffeull) return fail(PGEOF_ERR_INVALID_ARGUMENT, "nn_ptr is too long");
    int dev = -1;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess || dev < 0 || dev >= kNoAllocMaxDevices) {
        (void)cudaGetLastError();
        return fail(PGEOF_ERR_NO_DEVICE, std::string("no CUDA device: ") + cudaGetErrorString(e));
    }
    NoAllocSetup& st = g_noalloc_setup[dev];
    e = noalloc_setup(st);
    if (e != cudaSuccess) return fail(PGEOF_ERR_CUDA, std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e));
    const cudaStream_t s = (cudaStream_t)stream;
    // without a caller word the bits accumulate in the library's word for this
    // device until pgeof_take_device_errors reads and clears it
    uint32_t* err = error_bits ? error_bits : st.err;
    if (n_points == 0) return PGEOF_OK;
    if (n_xyz > 0) {
        const unsigned blocks = (unsigned)std::min<uint64_t>(ceil_div_u((uint64_t)n_xyz, 256), 4096);
        pad_xyz_kernel<<<blocks, 256, 0, s>>>(xyz, (uint64_t)n_xyz, st.xyz4);
        count_launch();
        PGEOF_TRY(check_launch("pad_xyz_kernel (noalloc)"));
    }
    FeatArgs a{};
    a.xyz4 = st.xyz4;
    a.n_xyz = (uint32_t)n_xyz;
    a.nn = nn;
    a.nnz = (uint64_t)nnz;
    a.ptr = nn_ptr;
    a.n_points = (uint32_t)n_points;
    a.k_min = (uint32_t)std::min<uint64_t>(k_min, 0xffffffffull);
    a.full = 1;
    a.n_scales = 1;
    a.scale_offset = 0;
    a.out_scales = 1;
    a.order = eig_order();
    a.out = features;
    a.err = err;
    const size_t smem = (size_t)kFeatThreads * 11 * sizeof(float);
    features_kernel<1, false, false, true><<<ceil_div_u((uint64_t)n_points, kFeatThreads), kFeatThreads, smem, s>>>(a);
    count_launch();
    return check_launch("features_kernel (noalloc)");
}
