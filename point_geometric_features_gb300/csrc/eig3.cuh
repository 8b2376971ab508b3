// eig3.cuh -- per-neighbourhood PCA on the device: symmetric 3x3 eigen
// decomposition and the feature epilogues of pgeof (include/pca.hpp).
//
// Eigen-solver design. The covariance is formed in float exactly as the
// reference does (include/pca.hpp:75-76, see the feature kernels). It is then
// diagonalised by cyclic Jacobi rotations (Golub & Van Loan, "Matrix
// Computations", sec. 8.5) in float. Jacobi is backward stable, so the float
// eigenvectors are accurate to ~eps*|A|/gap; when the smallest eigen-gap is
// below kGapResolve*|A| the same float covariance is diagonalised again
// exactly: by Jacobi in double-float arithmetic (pca_solve_refined), and for
// relative gaps below kGapFloat64 -- where the eigenvectors are fixed only by
// the sequence of rotations -- in double with exactly the arithmetic of the
// CPU oracle's solver (explicit round-to-nearest ops, no FMA), so
// ill-conditioned neighbourhoods reproduce the exact solution of the float
// covariance instead of float noise. Eigenpairs
// are then ordered as Eigen's SelfAdjointEigenSolver returns them (ascending;
// for equal values the first minimum stays first), because the reference feeds
// them to the formulas unsorted (pca.hpp:79-97).
#pragma once

#include "common.cuh"

namespace pgeof {

// Smallest relative eigen-gap handled by the float solver alone.
constexpr float kGapResolve = 3e-3f;

template <typename T>
struct Pca {
    T val[3];   // eigenvalues, clamped >= 0, in the order the formulas use
    T v[3][3];  // v[r][c]: row r of eigenvector c (c = 0, 1, 2 -> v0, v1, v2)
};

template <typename T>
struct Cov {
    T xx, xy, xz, yy, yz, zz;
};

// Division and square root of a rotation's parameters: IEEE-rounded (the
// oracle's arithmetic, used by the exact solver) or the hardware reciprocal
// and reciprocal square root (FAST, float only). Any rotation angle that keeps
// c^2 + s^2 = 1 to working precision serves Jacobi; the float solver's
// eigenvalues are refined afterwards as Rayleigh quotients.
template <typename T, bool FAST>
struct RotOps {
    static __device__ __forceinline__ T div(T a, T b) { return XOps<T>::div(a, b); }
    static __device__ __forceinline__ T inv_sqrt1p(T x) { return XOps<T>::div(T(1), XOps<T>::sqrt_(XOps<T>::add(T(1), x))); }
    static __device__ __forceinline__ T sqrt1p(T x) { return XOps<T>::sqrt_(XOps<T>::add(T(1), x)); }
};
template <>
struct RotOps<float, true> {
    static __device__ __forceinline__ float div(float a, float b) { return __fdividef(a, b); }
    static __device__ __forceinline__ float inv_sqrt1p(float x) { return rsqrtf(1.0f + x); }
    static __device__ __forceinline__ float sqrt1p(float x) { return sqrtf(1.0f + x); }
};

// One Jacobi rotation annihilating a[P][Q] (P < Q). Without FAST it mirrors the
// CPU oracle's solver operation for operation (explicit rounding, no fused
// multiply-add).
template <int P, int Q, typename T, bool VEC, bool FAST = false>
__device__ __forceinline__ void jacobi_rotate(T (&a)[3][3], T (&v)[3][3], bool late) {
    using O = XOps<T>;
    using RO = RotOps<T, FAST>;
    constexpr int R = 3 - P - Q;
    const T apq = a[P][Q];
    if (apq == T(0)) return;
    const T g = O::mul(T(100), fabs(apq));
    if (late && O::add(fabs(a[P][P]), g) == fabs(a[P][P]) && O::add(fabs(a[Q][Q]), g) == fabs(a[Q][Q])) {
        a[P][Q] = a[Q][P] = T(0);
        return;
    }
    const T h = O::sub(a[Q][Q], a[P][P]);
    T t;
    if (O::add(fabs(h), g) == fabs(h)) {
        t = RO::div(apq, h);
    } else {
        const T theta = RO::div(O::mul(T(0.5), h), apq);
        t = RO::div(T(1), O::add(fabs(theta), RO::sqrt1p(O::mul(theta, theta))));
        if (theta < T(0)) t = -t;
    }
    const T c = RO::inv_sqrt1p(O::mul(t, t));
    const T s = O::mul(t, c);
    const T tau = RO::div(s, O::add(T(1), c));
    a[P][P] = O::sub(a[P][P], O::mul(t, apq));
    a[Q][Q] = O::add(a[Q][Q], O::mul(t, apq));
    a[P][Q] = a[Q][P] = T(0);
    const T arp = a[R][P], arq = a[R][Q];
    a[R][P] = a[P][R] = O::sub(arp, O::mul(s, O::add(arq, O::mul(tau, arp))));
    a[R][Q] = a[Q][R] = O::add(arq, O::mul(s, O::sub(arp, O::mul(tau, arq))));
    if (VEC) {
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            const T vkp = v[k][P], vkq = v[k][Q];
            v[k][P] = O::sub(vkp, O::mul(s, O::add(vkq, O::mul(tau, vkp))));
            v[k][Q] = O::add(vkq, O::mul(s, O::sub(vkp, O::mul(tau, vkq))));
        }
    }
}

// Cyclic Jacobi. EXACT=true runs to convergence like the oracle (64 sweeps at
// most); EXACT=false stops once the off-diagonal mass is below float
// resolution. Returns the number of sweeps that rotated something.
template <typename T, bool VEC, bool EXACT>
__device__ __forceinline__ int jacobi3(T (&a)[3][3], T (&v)[3][3]) {
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j) v[i][j] = (i == j) ? T(1) : T(0);
    int sweeps = 0;
    const int max_sweeps = EXACT ? 64 : 16;
    for (int sweep = 0; sweep < max_sweeps; ++sweep) {
        if (a[0][1] == T(0) && a[0][2] == T(0) && a[1][2] == T(0)) break;
        if constexpr (!EXACT) {
            const T off = fabs(a[0][1]) + fabs(a[0][2]) + fabs(a[1][2]);
            const T scale = fabs(a[0][0]) + fabs(a[1][1]) + fabs(a[2][2]);
            if (sweep >= 2 && off <= T(1e-9) * scale) break;
        }
        ++sweeps;
        const bool late = sweep > 4;
        constexpr bool kFast = !EXACT && sizeof(T) == sizeof(float);
        jacobi_rotate<0, 1, T, VEC, kFast>(a, v, late);
        jacobi_rotate<0, 2, T, VEC, kFast>(a, v, late);
        jacobi_rotate<1, 2, T, VEC, kFast>(a, v, late);
    }
    return sweeps;
}

template <int I, int K, typename T>
__device__ __forceinline__ void swap_cols(T (&w)[3], T (&v)[3][3]) {
    const T t = w[I];
    w[I] = w[K];
    w[K] = t;
#pragma unroll
    for (int r = 0; r < 3; ++r) {
        const T u = v[r][I];
        v[r][I] = v[r][K];
        v[r][K] = u;
    }
}

// Eigen's ascending order: position i takes the FIRST minimum of w[i..2].
template <typename T>
__device__ __forceinline__ void sort_ascending(T (&w)[3], T (&v)[3][3]) {
    int k = 0;
    if (w[1] < w[k]) k = 1;
    if (w[2] < w[k]) k = 2;
    if (k == 1) swap_cols<0, 1>(w, v);
    if (k == 2) swap_cols<0, 2>(w, v);
    if (w[2] < w[1]) swap_cols<1, 2>(w, v);
}

template <typename T>
__device__ __forceinline__ void load_cov(const Cov<T>& c, T (&a)[3][3]) {
    a[0][0] = c.xx;
    a[0][1] = a[1][0] = c.xy;
    a[0][2] = a[2][0] = c.xz;
    a[1][1] = c.yy;
    a[1][2] = a[2][1] = c.yz;
    a[2][2] = c.zz;
}

// Finish: order (ascending or reversed), clamp >= 0 (std::max(ev, 0)), flip v2
// into z >= 0 (pca.hpp:85-96).
template <typename T, typename S>
__device__ __forceinline__ void finish_pca(const S (&w)[3], const S (&v)[3][3], int order, Pca<T>& out) {
#pragma unroll
    for (int i = 0; i < 3; ++i) {
        const int src = order ? 2 - i : i;
        const T ev = (T)w[src];
        out.val[i] = (ev < T(0)) ? T(0) : ev;
#pragma unroll
        for (int r = 0; r < 3; ++r) out.v[r][i] = (T)v[r][src];
    }
    if (out.v[2][2] < T(0)) {
#pragma unroll
        for (int r = 0; r < 3; ++r) out.v[r][2] = out.v[r][2] * T(-1);
    }
}

// Double-precision solve of a covariance, identical to the oracle's solver.
template <typename T>
__device__ __noinline__ void pca_solve_f64(const Cov<T> cov, int order, Pca<T>* out) {
    double a[3][3], v[3][3], w[3];
    a[0][0] = (double)cov.xx;
    a[0][1] = a[1][0] = (double)cov.xy;
    a[0][2] = a[2][0] = (double)cov.xz;
    a[1][1] = (double)cov.yy;
    a[1][2] = a[2][1] = (double)cov.yz;
    a[2][2] = (double)cov.zz;
    jacobi3<double, true, true>(a, v);
    w[0] = a[0][0];
    w[1] = a[1][1];
    w[2] = a[2][2];
    sort_ascending(w, v);
    finish_pca<T, double>(w, v, order, *out);
}

// ---- compensated ("double-float") arithmetic on the FP32 pipes: a value is
// hi + lo with |lo| <= ulp(hi)/2 (Dekker 1971; Knuth TAOCP vol. 2, 4.2.2).
struct DFloat {
    float hi, lo;
};
__device__ __forceinline__ DFloat two_prod(float a, float b) {
    const float p = __fmul_rn(a, b);
    return {p, __fmaf_rn(a, b, -p)};
}
__device__ __forceinline__ DFloat two_sum(float a, float b) {
    const float s = __fadd_rn(a, b);
    const float bb = __fsub_rn(s, a);
    return {s, __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb))};
}
__device__ __forceinline__ DFloat quick_two_sum(float a, float b) {
    const float s = __fadd_rn(a, b);
    return {s, __fsub_rn(b, __fsub_rn(s, a))};
}
__device__ __forceinline__ DFloat df_add(DFloat x, DFloat y) {
    const DFloat s = two_sum(x.hi, y.hi);
    return quick_two_sum(s.hi, __fadd_rn(s.lo, __fadd_rn(x.lo, y.lo)));
}
__device__ __forceinline__ DFloat df_mul(DFloat x, float a) {
    const DFloat p = two_prod(x.hi, a);
    return quick_two_sum(p.hi, __fmaf_rn(x.lo, a, p.lo));
}

// ---- a double-float number type for the eigen solver: the same Jacobi
// iteration as the float64 solver, on the FP32 pipes. Addition is the
// accurate double-float sum (both halves' errors carried), products use the
// fused multiply-add for the exact error of hi * hi, division and square root
// take one correction step from the float quotient / root (Dekker 1971;
// Knuth TAOCP vol. 2, 4.2.2; Bailey's double-double arithmetic). Relative
// precision ~2^-44 down to magnitudes of ~1e-30.
struct DF {
    float hi, lo;
    DF() = default;
    __device__ __forceinline__ DF(float h) : hi(h), lo(0.0f) {}
    __device__ __forceinline__ DF(float h, float l) : hi(h), lo(l) {}
    __device__ __forceinline__ explicit operator float() const { return __fadd_rn(hi, lo); }
};
__device__ __forceinline__ DF df_norm(float h, float l) {
    const DFloat q = quick_two_sum(h, l);
    return DF(q.hi, q.lo);
}
__device__ __forceinline__ DF operator-(DF x) { return DF(-x.hi, -x.lo); }
__device__ __forceinline__ bool operator==(DF x, DF y) { return x.hi == y.hi && x.lo == y.lo; }
__device__ __forceinline__ bool operator<(DF x, DF y) { return x.hi < y.hi || (x.hi == y.hi && x.lo < y.lo); }
using ::fabs;  // the float and double overloads stay visible beside DF's
__device__ __forceinline__ DF fabs(DF x) { return x.hi < 0.0f || (x.hi == 0.0f && x.lo < 0.0f) ? -x : x; }
__device__ __forceinline__ DF df_sum(DF x, DF y) {
    const DFloat s = two_sum(x.hi, y.hi);
    const DFloat t = two_sum(x.lo, y.lo);
    DF r = df_norm(s.hi, __fadd_rn(s.lo, t.hi));
    return df_norm(r.hi, __fadd_rn(r.lo, t.lo));
}
__device__ __forceinline__ DF df_prod(DF x, DF y) {
    const DFloat p = two_prod(x.hi, y.hi);
    return df_norm(p.hi, __fmaf_rn(x.lo, y.hi, __fmaf_rn(x.hi, y.lo, p.lo)));
}
__device__ __forceinline__ DF df_quot(DF x, DF y) {
    const float q1 = __fdiv_rn(x.hi, y.hi);
    DF r = df_sum(x, -df_prod(y, DF(q1)));
    const float q2 = __fdiv_rn(r.hi, y.hi);
    r = df_sum(r, -df_prod(y, DF(q2)));
    const float q3 = __fdiv_rn(r.hi, y.hi);
    return df_sum(df_norm(q1, q2), DF(q3));
}
__device__ __forceinline__ DF df_root(DF x) {
    if (!(x.hi > 0.0f)) return DF(0.0f);
    const float r = __fsqrt_rn(x.hi);
    const DFloat r2 = two_prod(r, r);
    const DF e = df_sum(x, -DF(r2.hi, r2.lo));
    return df_norm(r, __fdiv_rn(e.hi, __fmul_rn(2.0f, r)));
}

}  // namespace pgeof

template <>
struct XOps<pgeof::DF> {
    using D = pgeof::DF;
    static __device__ __forceinline__ D add(D a, D b) { return pgeof::df_sum(a, b); }
    static __device__ __forceinline__ D sub(D a, D b) { return pgeof::df_sum(a, -b); }
    static __device__ __forceinline__ D mul(D a, D b) { return pgeof::df_prod(a, b); }
    static __device__ __forceinline__ D div(D a, D b) { return pgeof::df_quot(a, b); }
    static __device__ __forceinline__ D sqrt_(D a) { return pgeof::df_root(a); }
};

namespace pgeof {

// Rayleigh quotient v^T A v / v^T v of the float covariance, evaluated in
// double-float. With v accurate to angle t the result is within t^2 * gap of
// the exact eigenvalue, and rounding contributes ~2^-46 |A| instead of the
// ~2^-24 |A| of a plain float evaluation -- which is what a small eigenvalue
// needs: the reference's formulas divide by sqrt(lambda_min) + 1e-3.
__device__ __forceinline__ float rayleigh(const Cov<float>& c, float x, float y, float z) {
    DFloat q = df_mul(two_prod(x, x), c.xx);
    q = df_add(q, df_mul(two_prod(y, y), c.yy));
    q = df_add(q, df_mul(two_prod(z, z), c.zz));
    q = df_add(q, df_mul(two_prod(x, y), __fmul_rn(2.0f, c.xy)));
    q = df_add(q, df_mul(two_prod(x, z), __fmul_rn(2.0f, c.xz)));
    q = df_add(q, df_mul(two_prod(y, z), __fmul_rn(2.0f, c.yz)));
    DFloat n = two_prod(x, x);
    n = df_add(n, two_prod(y, y));
    n = df_add(n, two_prod(z, z));
    return __fdiv_rn(__fadd_rn(q.hi, q.lo), __fadd_rn(n.hi, n.lo));
}

// Float covariance -> PCA. `resolved` reports a re-solve in double.
// Float solve alone: returns false, with `out` unset, for a neighbourhood whose
// relative eigen-gap is below kGapResolve (its eigenvectors need the exact
// solve), so that callers can run that rare solve outside their hot loop.
__device__ __forceinline__ bool pca_solve_f32_fast(const Cov<float>& cov, int order, Pca<float>& out) {
    float a[3][3], v[3][3], w[3];
    load_cov(cov, a);
    const int sweeps = jacobi3<float, true, false>(a, v);
    w[0] = a[0][0];
    w[1] = a[1][1];
    w[2] = a[2][2];
    sort_ascending(w, v);
    const float gap = fminf(w[1] - w[0], w[2] - w[1]);
    const float scale = fmaxf(fabsf(w[0]), fabsf(w[2]));
    if (sweeps > 0 && gap < kGapResolve * scale) return false;
    if (sweeps > 0) {
        // eigenvalues to ~1e-14 |A| from the well-conditioned eigenvectors
#pragma unroll
        for (int i = 0; i < 3; ++i) w[i] = rayleigh(cov, v[0][i], v[1][i], v[2][i]);
    }
    finish_pca<float, float>(w, v, order, out);
    return true;
}


// 1 / sqrt(1 + x) in double-float: the float reciprocal root and one Newton
// step (r + r (1 - y r^2) / 2).
__device__ __forceinline__ DF df_rsqrt1p(DF x) {
    const DF y = df_sum(DF(1.0f), x);
    const float r = rsqrtf(y.hi);
    const DFloat r2 = two_prod(r, r);
    const DF e = df_sum(DF(1.0f), -df_prod(y, DF(r2.hi, r2.lo)));
    return df_norm(r, __fmul_rn(__fmul_rn(0.5f, r), e.hi));
}

// One Jacobi rotation in double-float annihilating a[P][Q]:
// t = sgn(d) 2 a_pq / (|d| + sqrt(d^2 + 4 a_pq^2)) with d = a_qq - a_pp (the
// smaller root of t^2 + 2 theta t - 1, theta = d / (2 a_pq)), c = 1/sqrt(1 + t^2),
// s = t c; one division and two roots per rotation.
template <int P, int Q>
__device__ __forceinline__ void df_rotate(DF (&a)[3][3], DF (&v)[3][3]) {
    constexpr int R = 3 - P - Q;
    const DF apq = a[P][Q];
    if (apq.hi == 0.0f) return;
    const DF d = df_sum(a[Q][Q], -a[P][P]);
    const DF two_apq(__fmul_rn(2.0f, apq.hi), __fmul_rn(2.0f, apq.lo));
    const DF root = df_root(df_sum(df_prod(d, d), df_prod(two_apq, two_apq)));
    DF t = df_quot(two_apq, df_sum(fabs(d), root));
    if (d.hi < 0.0f) t = -t;
    const DF c = df_rsqrt1p(df_prod(t, t));
    const DF sn = df_prod(t, c);
    const DF tap = df_prod(t, apq);
    a[P][P] = df_sum(a[P][P], -tap);
    a[Q][Q] = df_sum(a[Q][Q], tap);
    a[P][Q] = a[Q][P] = DF(0.0f);
    const DF arp = a[R][P], arq = a[R][Q];
    a[R][P] = a[P][R] = df_sum(df_prod(c, arp), -df_prod(sn, arq));
    a[R][Q] = a[Q][R] = df_sum(df_prod(sn, arp), df_prod(c, arq));
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        const DF vkp = v[k][P], vkq = v[k][Q];
        v[k][P] = df_sum(df_prod(c, vkp), -df_prod(sn, vkq));
        v[k][Q] = df_sum(df_prod(sn, vkp), df_prod(c, vkq));
    }
}

// Relative eigen-gap below which the double-float solve is not trusted with
// the eigenvectors (their error is ~2^-44 / gap) and the float64 solve runs.
constexpr float kGapFloat64 = 1e-7f;

// The exact solve of a small-gap neighbourhood: cyclic Jacobi in double-float
// on the float covariance, swept until the off-diagonal is below 1e-15 of the
// diagonal, whose eigenpairs agree with the float64 solver's to ~1e-7 for
// relative gaps down to kGapFloat64; below that (exactly or nearly degenerate
// neighbourhoods) the float64 solver itself. A float64 solve is one long
// chain of slow dependent operations on this GPU (~60 us); the double-float
// one runs on the FP32 pipes. Returns false when the float64 solve ran.
__device__ __forceinline__ bool pca_solve_refined(const Cov<float>& cov, int order, Pca<float>& out) {
    DF a[3][3], v[3][3], w[3];
    a[0][0] = DF(cov.xx);
    a[0][1] = a[1][0] = DF(cov.xy);
    a[0][2] = a[2][0] = DF(cov.xz);
    a[1][1] = DF(cov.yy);
    a[1][2] = a[2][1] = DF(cov.yz);
    a[2][2] = DF(cov.zz);
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j) v[i][j] = DF(i == j ? 1.0f : 0.0f);
    for (int sweep = 0; sweep < 32; ++sweep) {
        const float off = fabsf(a[0][1].hi) + fabsf(a[0][2].hi) + fabsf(a[1][2].hi);
        const float diag = fabsf(a[0][0].hi) + fabsf(a[1][1].hi) + fabsf(a[2][2].hi);
        if (!(off > 1e-15f * diag)) break;
        df_rotate<0, 1>(a, v);
        df_rotate<0, 2>(a, v);
        df_rotate<1, 2>(a, v);
    }
    w[0] = a[0][0];
    w[1] = a[1][1];
    w[2] = a[2][2];
    sort_ascending(w, v);
    const float gap = fminf((float)df_sum(w[1], -w[0]), (float)df_sum(w[2], -w[1]));
    const float scale = fmaxf(fabsf((float)w[0]), fabsf((float)w[2]));
    if (!(gap >= kGapFloat64 * scale) || !(scale > 0.0f)) {
        pca_solve_f64<float>(cov, order, &out);
        return false;
    }
    finish_pca<float, DF>(w, v, order, out);
    return true;
}

// Float solve; ill-conditioned eigenvectors get the exact solve of the same
// float matrix in place (`resolved`).
__device__ __forceinline__ void pca_solve_f32(const Cov<float>& cov, int order, Pca<float>& out, bool& resolved) {
    resolved = !pca_solve_f32_fast(cov, order, out);
    if (resolved) pca_solve_refined(cov, order, out);
}

// Eigenvalues only, float (for eigentropy scans). Approximate rotations are fine
// here: the scan only ranks candidates, the winner is re-evaluated exactly.
__device__ __forceinline__ void eigvals_f32(const Cov<float>& cov, float (&w)[3]) {
    float a[3][3], v[3][3];
    load_cov(cov, a);
    jacobi3<float, false, false>(a, v);
    w[0] = a[0][0];
    w[1] = a[1][1];
    w[2] = a[2][2];
    // ascending (values only)
    float t;
    if (w[1] < w[0]) { t = w[0]; w[0] = w[1]; w[1] = t; }
    if (w[2] < w[1]) { t = w[1]; w[1] = w[2]; w[2] = t; }
    if (w[1] < w[0]) { t = w[0]; w[0] = w[1]; w[1] = t; }
}

// --------------------------------------------------------------- epilogues
template <typename T>
__device__ __forceinline__ T dev_pow(T x, T y);
template <>
__device__ __forceinline__ float dev_pow<float>(float x, float y) { return powf(x, y); }
template <>
__device__ __forceinline__ double dev_pow<double>(double x, double y) { return pow(x, y); }
template <typename T>
__device__ __forceinline__ T dev_log(T x);
template <>
__device__ __forceinline__ float dev_log<float>(float x) { return logf(x); }
template <>
__device__ __forceinline__ double dev_log<double>(double x) { return log(x); }

// include/pca.hpp:140-150
template <typename T>
__device__ __forceinline__ T eigentropy_of(const T (&val)[3]) {
    using O = XOps<T>;
    const T eps = T(1e-3);
    const T val_sum = O::add(O::add(O::add(val[0], val[1]), val[2]), eps);
    const T e0 = O::div(val[0], val_sum);
    const T e1 = O::div(val[1], val_sum);
    const T e2 = O::div(val[2], val_sum);
    T r = O::mul(-e0, dev_log<T>(O::add(e0, eps)));
    r = O::sub(r, O::mul(e1, dev_log<T>(O::add(e1, eps))));
    r = O::sub(r, O::mul(e2, dev_log<T>(O::add(e2, eps))));
    return r;
}

// include/pca.hpp:189-199
template <typename T>
__device__ __forceinline__ T verticality_pgeof(const Pca<T>& p) {
    using O = XOps<T>;
    T u[3];
#pragma unroll
    for (int j = 0; j < 3; ++j)
        u[j] = O::add(O::add(O::mul(p.val[0], fabs(p.v[j][0])), O::mul(p.val[1], fabs(p.v[j][1]))),
                      O::mul(p.val[2], fabs(p.v[j][2])));
    const T nrm = O::sqrt_(O::add(O::add(O::mul(u[0], u[0]), O::mul(u[1], u[1])), O::mul(u[2], u[2])));
    return O::div(u[2], nrm);
}

// include/pca.hpp:160-200; writes f[0..10] in EFeatureID order.
template <typename T>
__device__ __forceinline__ void features11(const Pca<T>& p, T* f) {
    using O = XOps<T>;
    const T eps = T(1e-3);
    const T val0 = O::sqrt_(p.val[0]);
    const T val1 = O::sqrt_(p.val[1]);
    const T val2 = O::sqrt_(p.val[2]);
    const T val0_fact = O::div(T(1), O::add(val0, eps));
    f[4] = p.v[0][2];
    f[5] = p.v[1][2];
    f[6] = p.v[2][2];
    f[0] = O::mul(O::sub(val0, val1), val0_fact);
    f[1] = O::mul(O::sub(val1, val2), val0_fact);
    f[2] = O::mul(val2, val0_fact);
    f[7] = val0;
    f[8] = O::sqrt_(O::add(O::mul(val0, val1), T(1e-6)));
    f[9] = dev_pow<T>(O::add(O::mul(O::mul(val0, val1), val2), T(1e-9)), T(1) / T(3));
    f[10] = O::div(val2, O::add(O::add(O::add(val0, val1), val2), eps));
    f[3] = (val0 > T(0)) ? verticality_pgeof(p) : T(0);
}

// include/pca.hpp:212-295 for one feature id (returns false = write nothing).
template <typename T>
__device__ __forceinline__ bool selected_feature(const Pca<T>& p, int id, T& out) {
    using O = XOps<T>;
    const T eps = T(1e-3);
    const T val0 = O::sqrt_(p.val[0]);
    const T val1 = O::sqrt_(p.val[1]);
    const T val2 = O::sqrt_(p.val[2]);
    const T val0_fact = O::div(T(1), O::add(val0, eps));
    switch (id) {
        case PGEOF_NORMAL_X: out = p.v[0][2]; return true;
        case PGEOF_NORMAL_Y: out = p.v[1][2]; return true;
        case PGEOF_NORMAL_Z: out = p.v[2][2]; return true;
        case PGEOF_LINEARITY: out = O::mul(O::sub(val0, val1), val0_fact); return true;
        case PGEOF_PLANARITY: out = O::mul(O::sub(val1, val2), val0_fact); return true;
        case PGEOF_SCATTERING: out = O::mul(val2, val0_fact); return true;
        case PGEOF_LENGTH: out = val0; return true;
        // pca.hpp:252 adds the float literal 1e-6f in both precisions
        case PGEOF_SURFACE: out = O::sqrt_(O::add(O::mul(val0, val1), (T)1e-6f)); return true;
        case PGEOF_VOLUME:
            out = dev_pow<T>(O::add(O::mul(O::mul(val0, val1), val2), T(1e-9)), T(1) / T(3));
            return true;
        case PGEOF_CURVATURE: out = O::div(val2, O::add(O::add(O::add(val0, val1), val2), eps)); return true;
        case PGEOF_VERTICALITY_PGEOF:
            if (val0 > T(0)) {
                out = verticality_pgeof(p);
                return true;
            }
            return false;
        case PGEOF_VERTICALITY: out = O::sub(T(1), fabs(p.v[2][2])); return true;
        case PGEOF_EIGENTROPY: out = eigentropy_of<T>(p.val); return true;
        default: return false;
    }
}

}  // namespace pgeof
