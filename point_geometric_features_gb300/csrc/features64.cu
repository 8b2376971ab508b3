// features64.cu -- the CSR feature passes for float64 clouds:
// compute_features, compute_features_multiscale and compute_features_optimal
// with real_t = double. pgeof's drivers and PCA are templates on real_t
// (include/pgeof.hpp:75-117, 123-211, 243-310; include/pca.hpp:72-200) but its
// binding instantiates these three for float only; this is the double
// instantiation, evaluated literally: per neighbourhood a sequential two-pass
// mean / covariance in double (no FMA), the double Jacobi solve shared with
// the selected path, and the feature formulas in double.
//
// One thread per CSR row. FP64 arithmetic, not memory, bounds these kernels on
// GB300; they exist for precision, the float32 kernels for throughput.
#include "eig3.cuh"
#include "kernels.cuh"

namespace pgeof {
namespace {

constexpr int kF64Threads = 128;

struct F64Args {
    const double* xyz;
    uint64_t n_xyz;
    const uint32_t* nn;
    uint64_t nnz;
    const uint32_t* ptr;
    uint64_t n_points;
    int kind;  // 0 compute_features, 1 multiscale, 2 optimal
    uint64_t k_min;
    const uint32_t* scales;  // device, n_scales entries (kind 1)
    int n_scales;
    uint32_t k_step, k_min_search;
    int order;
    double* out;
    uint32_t* err;
};

// include/pca.hpp:72-77 and :113-129 for the first k neighbours of the row at
// nn + b: colwise mean (sequential sum / k), centred products summed in
// neighbour order, / k.
__device__ __forceinline__ Cov<double> cov_first_k(const F64Args& a, uint64_t b, uint32_t k, uint32_t& flags) {
    double sx = 0.0, sy = 0.0, sz = 0.0;
    for (uint32_t j = 0; j < k; ++j) {
        uint64_t id = __ldg(a.nn + b + j);
        if (id >= a.n_xyz) {
            flags |= ERR_NN_RANGE;
            id = 0;
        }
        sx = DADD(sx, __ldg(a.xyz + 3 * id));
        sy = DADD(sy, __ldg(a.xyz + 3 * id + 1));
        sz = DADD(sz, __ldg(a.xyz + 3 * id + 2));
    }
    const double kk = (double)k;
    const double mx = DDIV(sx, kk), my = DDIV(sy, kk), mz = DDIV(sz, kk);
    double xx = 0.0, xy = 0.0, xz = 0.0, yy = 0.0, yz = 0.0, zz = 0.0;
    for (uint32_t j = 0; j < k; ++j) {
        uint64_t id = __ldg(a.nn + b + j);
        if (id >= a.n_xyz) id = 0;
        const double dx = DSUB(__ldg(a.xyz + 3 * id), mx);
        const double dy = DSUB(__ldg(a.xyz + 3 * id + 1), my);
        const double dz = DSUB(__ldg(a.xyz + 3 * id + 2), mz);
        xx = DADD(xx, DMUL(dx, dx));
        xy = DADD(xy, DMUL(dx, dy));
        xz = DADD(xz, DMUL(dx, dz));
        yy = DADD(yy, DMUL(dy, dy));
        yz = DADD(yz, DMUL(dy, dz));
        zz = DADD(zz, DMUL(dz, dz));
    }
    Cov<double> c;
    c.xx = DDIV(xx, kk);
    c.xy = DDIV(xy, kk);
    c.xz = DDIV(xz, kk);
    c.yy = DDIV(yy, kk);
    c.yz = DDIV(yz, kk);
    c.zz = DDIV(zz, kk);
    return c;
}

__device__ __forceinline__ void pca_first_k(const F64Args& a, uint64_t b, uint32_t k, uint32_t& flags,
                                            Pca<double>& p) {
    pca_solve_f64<double>(cov_first_k(a, b, k, flags), a.order, &p);
}

__global__ void __launch_bounds__(kF64Threads) features_f64_kernel(const __grid_constant__ F64Args a) {
    const uint64_t i = blockIdx.x * (uint64_t)kF64Threads + threadIdx.x;
    if (i >= a.n_points) return;
    uint32_t flags = 0;
    const uint64_t b = __ldg(a.ptr + i), e = __ldg(a.ptr + i + 1);
    uint64_t k_nn = 0;
    if (e < b || e > a.nnz) flags |= ERR_PTR_RANGE;
    else k_nn = e - b;
    if (a.kind == 0) {
        // include/pgeof.hpp:93-109: rows with fewer than k_min neighbours stay 0
        double f[11];
        for (int t = 0; t < 11; ++t) f[t] = 0.0;
        if (k_nn >= a.k_min && k_nn > 0) {
            Pca<double> p;
            pca_first_k(a, b, (uint32_t)k_nn, flags, p);
            features11<double>(p, f);
        }
        double* row = a.out + i * 11;
        for (int t = 0; t < 11; ++t) row[t] = f[t];
    } else if (a.kind == 1) {
        // include/pgeof.hpp:183-199: the scales in order, stopping at the first
        // scale the row cannot fill (it and the later ones stay 0)
        double* row = a.out + i * (uint64_t)a.n_scales * 11;
        bool live = true;
        for (int s = 0; s < a.n_scales; ++s) {
            const uint32_t ks = __ldg(a.scales + s);
            double f[11];
            for (int t = 0; t < 11; ++t) f[t] = 0.0;
            live = live && k_nn >= ks;
            if (live && ks > 0) {
                Pca<double> p;
                pca_first_k(a, b, ks, flags, p);
                features11<double>(p, f);
            }
            for (int t = 0; t < 11; ++t) row[s * 11 + t] = f[t];
        }
    } else {
        // include/pgeof.hpp:264-299: eigentropy over k0, the multiples of
        // k_step above it and k_nn; the first strict minimum wins
        double f[12];
        for (int t = 0; t < 12; ++t) f[t] = 0.0;
        if (k_nn >= a.k_min && k_nn >= a.k_min_search && k_nn > 0) {
            uint64_t k0 = a.k_min > a.k_min_search ? a.k_min : a.k_min_search;
            if (k0 > k_nn) k0 = k_nn;
            Pca<double> best;
            double best_e = 1.0;
            uint64_t k_opt = k_nn;
            for (uint64_t k = k0; k <= k_nn; ++k) {
                if (k > k0 && (k % a.k_step) != 0 && k != k_nn) continue;
                Pca<double> p;
                pca_first_k(a, b, (uint32_t)k, flags, p);
                const double ent = eigentropy_of<double>(p.val);
                if (k == k0 || ent < best_e) {
                    best_e = ent;
                    k_opt = k;
                    best = p;
                }
            }
            features11<double>(best, f);
            f[11] = (double)k_opt;
        }
        double* row = a.out + i * 12;
        for (int t = 0; t < 12; ++t) row[t] = f[t];
    }
    if (flags) atomicOr(a.err, flags);
}

}  // namespace

int launch_features_f64(const double* xyz, uint64_t n_xyz, const uint32_t* nn, uint64_t nnz, const uint32_t* ptr,
                        uint64_t n_points, int kind, uint64_t k_min, const uint32_t* scales, int n_scales,
                        uint32_t k_step, uint32_t k_min_search, double* out, cudaStream_t s) {
    if (n_points == 0) return PGEOF_OK;
    if (kind == 1 && n_scales == 0) return PGEOF_OK;
    F64Args a{};
    a.xyz = xyz;
    a.n_xyz = n_xyz;
    a.nn = nn;
    a.nnz = nnz;
    a.ptr = ptr;
    a.n_points = n_points;
    a.kind = kind;
    a.k_min = k_min;
    a.n_scales = n_scales;
    a.k_step = k_step ? k_step : 1;
    a.k_min_search = k_min_search;
    a.order = eig_order();
    a.out = out;
    a.err = device_error_word();
    Scratch d_scales;
    if (kind == 1) {
        PGEOF_TRY(d_scales.alloc((size_t)n_scales * sizeof(uint32_t), s));
        PGEOF_CUDA_TRY(cudaMemcpyAsync(d_scales.p, scales, (size_t)n_scales * sizeof(uint32_t),
                                       cudaMemcpyHostToDevice, s));
        a.scales = d_scales.as<uint32_t>();
    }
    KernelTimer kt("features_f64_kernel", s);
    features_f64_kernel<<<ceil_div_u(n_points, kF64Threads), kF64Threads, 0, s>>>(a);
    count_launch();
    return check_launch("features_f64_kernel");
}

}  // namespace pgeof
