/*
 * pca_body.h -- PCA and feature formulas, instantiated by pgeof_oracle.c once
 * for float (REAL=float, SFX(x)=x##_f32) and once for double. Test
 * infrastructure only (see pgeof_oracle.c).
 */

typedef struct {
    REAL val[3];
    REAL v0[3];
    REAL v1[3];
    REAL v2[3];
} SFX(pca);

/* include/pca.hpp:75-76: centred = cloud - colwise mean; cov = centred^T centred / k.
 * Sums run sequentially over the neighbours, as Eigen's column reductions do. */
static void SFX(covariance)(const REAL* pts, size_t k, REAL c[3][3]) {
    REAL mean[3] = {0, 0, 0};
    for (size_t j = 0; j < k; ++j)
        for (int a = 0; a < 3; ++a) mean[a] = mean[a] + pts[3 * j + a];
    const REAL kk = (REAL)k;
    for (int a = 0; a < 3; ++a) mean[a] = mean[a] / kk;
    REAL s[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
    for (size_t j = 0; j < k; ++j) {
        const REAL cx = pts[3 * j + 0] - mean[0];
        const REAL cy = pts[3 * j + 1] - mean[1];
        const REAL cz = pts[3 * j + 2] - mean[2];
        s[0][0] = s[0][0] + cx * cx;
        s[0][1] = s[0][1] + cx * cy;
        s[0][2] = s[0][2] + cx * cz;
        s[1][1] = s[1][1] + cy * cy;
        s[1][2] = s[1][2] + cy * cz;
        s[2][2] = s[2][2] + cz * cz;
    }
    c[0][0] = s[0][0] / kk;
    c[0][1] = c[1][0] = s[0][1] / kk;
    c[0][2] = c[2][0] = s[0][2] / kk;
    c[1][1] = s[1][1] / kk;
    c[1][2] = c[2][1] = s[1][2] / kk;
    c[2][2] = s[2][2] / kk;
}

/* include/pca.hpp:72-98. Eigenpairs come back in Eigen's ascending order (the
 * reference does not sort); ORACLE_EIG_DESCENDING reverses them. */
static void SFX(pca_from_pointcloud)(const REAL* pts, size_t k, int order, SFX(pca) * out) {
    REAL c[3][3];
    SFX(covariance)(pts, k, c);
    double a[3][3], v[3][3], w[3];
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) a[i][j] = (double)c[i][j];
    jacobi3(a, v);
    w[0] = a[0][0];
    w[1] = a[1][1];
    w[2] = a[2][2];
    sort_ascending(w, v);
    int col[3] = {0, 1, 2};
    if (order == ORACLE_EIG_DESCENDING) {
        col[0] = 2;
        col[2] = 0;
    }
    for (int i = 0; i < 3; ++i) {
        const REAL ev = (REAL)w[col[i]];
        /* std::max(ev, 0): returns ev unless ev < 0 */
        out->val[i] = (ev < (REAL)0) ? (REAL)0 : ev;
    }
    for (int r = 0; r < 3; ++r) {
        out->v0[r] = (REAL)v[r][col[0]];
        out->v1[r] = (REAL)v[r][col[1]];
        out->v2[r] = (REAL)v[r][col[2]];
    }
    if (out->v2[2] < (REAL)0) {
        for (int r = 0; r < 3; ++r) out->v2[r] = out->v2[r] * (REAL)(-1);
    }
}

/* include/pca.hpp:140-150 */
static REAL SFX(compute_eigentropy)(const SFX(pca) * p) {
    const REAL eps = (REAL)1e-3;
    const REAL val_sum = p->val[0] + p->val[1] + p->val[2] + eps;
    const REAL e0 = p->val[0] / val_sum;
    const REAL e1 = p->val[1] / val_sum;
    const REAL e2 = p->val[2] / val_sum;
    return -e0 * RLOG(e0 + eps) - e1 * RLOG(e1 + eps) - e2 * RLOG(e2 + eps);
}

/* include/pca.hpp:189-199 and :262-278 */
static REAL SFX(verticality_pgeof)(const SFX(pca) * p) {
    const REAL u0 = p->val[0] * RABS(p->v0[0]) + p->val[1] * RABS(p->v1[0]) + p->val[2] * RABS(p->v2[0]);
    const REAL u1 = p->val[0] * RABS(p->v0[1]) + p->val[1] * RABS(p->v1[1]) + p->val[2] * RABS(p->v2[1]);
    const REAL u2 = p->val[0] * RABS(p->v0[2]) + p->val[1] * RABS(p->v1[2]) + p->val[2] * RABS(p->v2[2]);
    return u2 / RSQRT(u0 * u0 + u1 * u1 + u2 * u2);
}

/* include/pca.hpp:160-200. Index order = EFeatureID 0..10. */
static void SFX(compute_features)(const SFX(pca) * p, REAL* f) {
    const REAL eps = (REAL)1e-3;
    const REAL sq_eps = (REAL)1e-6;
    const REAL cub_eps = (REAL)1e-9;
    const REAL one_third = (REAL)1.0 / (REAL)3.0;
    const REAL val0 = RSQRT(p->val[0]);
    const REAL val1 = RSQRT(p->val[1]);
    const REAL val2 = RSQRT(p->val[2]);
    const REAL val0_fact = (REAL)1.0 / (val0 + eps);
    f[4] = p->v2[0];
    f[5] = p->v2[1];
    f[6] = p->v2[2];
    f[0] = (val0 - val1) * val0_fact;
    f[1] = (val1 - val2) * val0_fact;
    f[2] = val2 * val0_fact;
    f[7] = val0;
    f[8] = RSQRT(val0 * val1 + sq_eps);
    f[9] = RPOW(val0 * val1 * val2 + cub_eps, one_third);
    f[10] = val2 / (val0 + val1 + val2 + eps);
    if (val0 > (REAL)0) f[3] = SFX(verticality_pgeof)(p);
}

/* include/pca.hpp:212-295. ids are EFeatureID integers; K_optimal (11) and
 * unknown ids write nothing. */
static void SFX(compute_selected_features)(const SFX(pca) * p, const int32_t* ids, size_t n_ids, REAL* f) {
    const REAL eps = (REAL)1e-3;
    const REAL val0 = RSQRT(p->val[0]);
    const REAL val1 = RSQRT(p->val[1]);
    const REAL val2 = RSQRT(p->val[2]);
    const REAL val0_fact = (REAL)1.0 / (val0 + eps);
    for (size_t i = 0; i < n_ids; ++i) {
        switch (ids[i]) {
            case 4: f[i] = p->v2[0]; break;
            case 5: f[i] = p->v2[1]; break;
            case 6: f[i] = p->v2[2]; break;
            case 0: f[i] = (val0 - val1) * val0_fact; break;
            case 1: f[i] = (val1 - val2) * val0_fact; break;
            case 2: f[i] = val2 * val0_fact; break;
            case 7: f[i] = val0; break;
            case 8: f[i] = RSQRT(val0 * val1 + (REAL)1e-6f); break;
            case 9: f[i] = RPOW(val0 * val1 * val2 + (REAL)1e-9, (REAL)1.0 / (REAL)3.0); break;
            case 10: f[i] = val2 / (val0 + val1 + val2 + eps); break;
            case 3:
                if (val0 > (REAL)0) f[i] = SFX(verticality_pgeof)(p);
                break;
            case 12: f[i] = (REAL)1.0 - RABS(p->v2[2]); break;
            case 13: f[i] = SFX(compute_eigentropy)(p); break;
            default: break;
        }
    }
}
