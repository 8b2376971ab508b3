"""The oracle itself, pinned before it is trusted (CPU only).

* neighbour search against scipy's KDTree -- the reference's own tests
  (tests/test_pgeof.py:8-27) and their committed seeded fixtures;
* the reference's multiscale self-consistency test (tests/test_pgeof.py:30-46);
* features against hand-derived known answers of include/pca.hpp's formulas
  and against the independent FP64 numpy restatement.
"""

import numpy as np
import pytest
from scipy.spatial import KDTree

from oracle import oracle


def test_knn_matches_scipy_fixture(golden):
    g = golden("knn_1000_k10.npz")
    idx, d2 = oracle.knn_search(g["xyz"], g["xyz"], 10)
    np.testing.assert_equal(idx.astype(np.int64), g["scipy_idx"])
    assert np.all(np.diff(d2, axis=1) >= 0)


def test_radius_matches_scipy_fixture(golden):
    g = golden("radius_1000_r02_k10.npz")
    idx, d2 = oracle.radius_search(g["xyz"], g["xyz"], 0.2, 10)
    np.testing.assert_equal(idx.astype(np.int64), g["scipy_idx"])


@pytest.mark.parametrize("seed", [1, 2, 3])
def test_knn_matches_scipy_random(seed):
    """tests/test_pgeof.py:8-15 with fresh seeds."""
    rng = np.random.default_rng(seed)
    xyz = rng.uniform(0.0, 200.0, size=(1000, 3)).astype(np.float32)
    _, ref = KDTree(xyz).query(xyz, k=10)
    idx, _ = oracle.knn_search(xyz, xyz, 10)
    np.testing.assert_equal(idx.astype(np.int64), ref)


def test_radius_fill_and_last_slot():
    rng = np.random.default_rng(5)
    xyz = rng.random((500, 3), dtype=np.float32)
    r = np.float32(0.17)
    idx, d2 = oracle.radius_search(xyz, xyz, r, 12)
    cnt = (idx >= 0).sum(1)
    short = cnt < 12
    assert short.any() and (~short).any()
    # missing entries: index -1, distance 0, except nanoflann RKNN's r^2 in the last slot
    for i in np.nonzero(short)[0][:50]:
        assert np.all(idx[i, cnt[i]:] == -1)
        assert np.all(d2[i, cnt[i]:-1] == 0)
        assert d2[i, -1] == np.float32(r * r)
    assert np.all(d2[idx >= 0] < r * r)


def test_golden_features_reproduce(golden):
    g = golden("features_2000_k20.npz")
    xyz, idx = g["xyz"], g["idx"]
    k = idx.shape[1]
    nn = idx.reshape(-1).astype(np.uint32)
    nn_ptr = (np.arange(xyz.shape[0] + 1) * k).astype(np.uint32)
    np.testing.assert_array_equal(oracle.compute_features(xyz, nn, nn_ptr, 1), g["features"])
    np.testing.assert_array_equal(oracle.compute_features_multiscale(xyz, nn, nn_ptr, [5, 10, 20]), g["multiscale"])
    np.testing.assert_array_equal(oracle.compute_features_optimal(xyz, nn, nn_ptr, 1, 1, 5), g["optimal"])


def test_multiscale_self_consistency():
    """tests/test_pgeof.py:30-46 on the oracle (rtol 1e-1, atol 1e-5 there)."""
    rng = np.random.default_rng(4)
    xyz = rng.uniform(0.0, 200.0, size=(3000, 3)).astype(np.float32)
    _, kn = KDTree(xyz).query(xyz, k=50)
    nn = kn.flatten().astype(np.uint32)
    nn_ptr = (np.arange(xyz.shape[0] + 1) * 50).astype(np.uint32)
    multi = oracle.compute_features_multiscale(xyz, nn, nn_ptr, [20, 50])
    simple = oracle.compute_features(xyz, nn, nn_ptr, 50)
    multi_simple = oracle.compute_features_multiscale(xyz, nn, nn_ptr, [20])
    np.testing.assert_array_equal(multi[:, 0], multi_simple[:, 0])
    np.testing.assert_array_equal(multi[:, 1], simple)


def test_fp32_oracle_vs_fp64(golden):
    """The FP32-literal oracle agrees with the FP64 restatement where the
    eigenvectors are well conditioned."""
    g = golden("features_2000_k20.npz")
    xyz, idx = g["xyz"], g["idx"]
    gap = oracle.fp64_relative_gap(xyz[idx])
    ok = gap > 1e-2
    f32, f64 = g["features"][ok], g["features_fp64"][ok]
    err = np.abs(f32 - f64) / np.maximum(1.0, np.abs(f64))
    assert err.max() < 2e-4, err.max()


def _line(n=11):
    t = np.linspace(-1.0, 1.0, n, dtype=np.float32)
    d = np.array([3.0, 4.0, 12.0], np.float32) / 13.0
    return (t[:, None] * d[None, :]).astype(np.float32), d


def test_known_answer_line():
    """Collinear points: eigenvalues (0, 0, s^2) ascending; as written in
    include/pca.hpp:160-200 with val0 = sqrt(lambda_min) = 0."""
    pts, d = _line()
    r = oracle.pca_features(pts)
    var = float(np.var(np.linspace(-1.0, 1.0, 11), ddof=0))
    np.testing.assert_allclose(r["val"], [0.0, 0.0, var], atol=1e-6)
    f = r["features"]
    s = np.sqrt(var)
    np.testing.assert_allclose(f[0], 0.0, atol=1e-3)  # (val0 - val1) / (val0 + 1e-3)
    np.testing.assert_allclose(f[1], -s / 1e-3, rtol=2e-3)  # (val1 - val2) / (val0 + 1e-3)
    np.testing.assert_allclose(f[2], s / 1e-3, rtol=2e-3)  # val2 / (val0 + 1e-3)
    np.testing.assert_allclose(np.abs(f[4:7]), d, atol=1e-5)  # v2 = principal axis
    assert f[6] >= 0  # z >= 0 flip
    np.testing.assert_allclose(f[7], 0.0, atol=1e-3)  # length = sqrt(lambda_min)
    np.testing.assert_allclose(f[8], 1e-3, rtol=1e-2)  # sqrt(0 + 1e-6)
    np.testing.assert_allclose(f[10], s / (s + 1e-3), rtol=1e-4)
    assert f[3] == 0.0  # verticality only when val0 > 0


def test_known_answer_plane_descending():
    """A planar square with the descending order: v2 = normal, planarity ~ 1."""
    g = np.linspace(-1.0, 1.0, 7, dtype=np.float32)
    X, Y = np.meshgrid(g, g)
    pts = np.stack([X.ravel(), Y.ravel(), np.zeros(X.size, np.float32)], 1).astype(np.float32)
    r = oracle.pca_features(pts, order=oracle.EIG_DESCENDING)
    np.testing.assert_allclose(r["val"][2], 0.0, atol=1e-7)
    np.testing.assert_allclose(r["features"][4:7], [0.0, 0.0, 1.0], atol=1e-6)
    s = np.sqrt(r["val"][0])
    np.testing.assert_allclose(r["features"][1], (s - 0.0) / (s + 1e-3), rtol=1e-5)


def test_known_answer_single_point():
    """k=1: zero covariance -> Eigen returns the identity basis; v2 = e_z."""
    r = oracle.pca_features(np.array([[1.0, 2.0, 3.0]], np.float32))
    f = r["features"]
    np.testing.assert_array_equal(r["val"], [0, 0, 0])
    np.testing.assert_array_equal(f[4:7], [0, 0, 1])
    np.testing.assert_allclose(f[8], 1e-3, rtol=1e-6)
    np.testing.assert_allclose(f[9], np.float32(1e-9) ** np.float32(1 / 3), rtol=1e-5)
    assert f[0] == 0 and f[1] == 0 and f[2] == 0 and f[3] == 0


def test_covariance_is_sequential_float():
    rng = np.random.default_rng(9)
    pts = (rng.random((37, 3)) * 10).astype(np.float32)
    mean = np.zeros(3, np.float32)
    for p in pts:
        mean = (mean + p).astype(np.float32)
    mean = (mean / np.float32(37)).astype(np.float32)
    c = (pts - mean).astype(np.float32)
    s = np.zeros((3, 3), np.float32)
    for row in c:
        s = (s + np.outer(row, row).astype(np.float32)).astype(np.float32)
    s = (s / np.float32(37)).astype(np.float32)
    cov = oracle.covariance(pts)
    np.testing.assert_array_equal(cov, [s[0, 0], s[0, 1], s[0, 2], s[1, 1], s[1, 2], s[2, 2]])


def test_optimal_rule_first_minimum():
    """k_opt = first k reaching the minimal eigentropy, col 11 = k_opt."""
    rng = np.random.default_rng(3)
    xyz = rng.random((400, 3), dtype=np.float32)
    idx, _ = oracle.knn_search(xyz, xyz, 30)
    nn = idx.reshape(-1).astype(np.uint32)
    nn_ptr = (np.arange(401) * 30).astype(np.uint32)
    out = oracle.compute_features_optimal(xyz, nn, nn_ptr, 1, 3, 10)
    for i in range(0, 400, 37):
        ks = [k for k in range(10, 31) if k == 10 or k % 3 == 0 or k == 30]
        ents = [oracle.pca_features(xyz[idx[i, :k]])["eigentropy"] for k in ks]
        best = ks[int(np.argmin(ents))]
        assert out[i, 11] == best
        np.testing.assert_array_equal(out[i, :11], oracle.pca_features(xyz[idx[i, :best]])["features"])


def test_selected_matches_features():
    rng = np.random.default_rng(8)
    xyz = rng.random((600, 3), dtype=np.float32)
    ids = [0, 1, 2, 3, 4, 5, 6, 7, 8, 9, 10]
    sel = oracle.compute_features_selected(xyz, 0.15, 16, ids)
    idx, _ = oracle.radius_search(xyz, xyz, 0.15, 16)
    for i in range(0, 600, 41):
        row = idx[i][idx[i] >= 0]
        if row.size < 2:
            assert np.all(sel[i] == 0)
            continue
        np.testing.assert_array_equal(sel[i], oracle.pca_features(xyz[row])["features"])


def test_f64_oracle_vs_numpy_fp64(golden):
    """The double-instantiation drivers (real_t = double) agree with the
    independent numpy FP64 restatement (eigh) on the golden cloud, and their
    multiscale / optimal drivers keep the float drivers' rules."""
    g = golden("features_2000_k20.npz")
    xyz, idx = g["xyz"].astype(np.float64), g["idx"]
    n, k = idx.shape
    nn = idx.reshape(-1).astype(np.uint32)
    ptr = (np.arange(n + 1) * k).astype(np.uint32)
    f = oracle.compute_features_f64(xyz, nn, ptr)
    ref = g["features_fp64"]
    gap = oracle.fp64_relative_gap(g["xyz"][idx])
    ok = gap > 1e-6
    err = np.abs(f - ref) / np.maximum(1.0, np.abs(ref))
    assert err[ok].max() < 1e-9, err[ok].max()
    assert np.abs(f[:, 7] - ref[:, 7]).max() < 1e-12  # Length: eigenvalue only
    m = oracle.compute_features_f64(xyz, nn, ptr, kind="multi", k_scales=[5, 10, k])
    np.testing.assert_array_equal(m[:, 2], f)
    # ragged rows: scales the row cannot fill stay 0 and so do the later ones
    nn_r = np.concatenate([nn[ptr[i]:ptr[i] + 7] for i in range(n)])
    ptr_r = (np.arange(n + 1) * 7).astype(np.uint32)
    m = oracle.compute_features_f64(xyz, nn_r, ptr_r, kind="multi", k_scales=[5, 10, 20])
    assert np.all(m[:, 1:] == 0) and np.all(m[:, 0, 7] > 0)
    o = oracle.compute_features_f64(xyz, nn, ptr, 1, kind="optimal", k_step=3, k_min_search=6)
    o32 = oracle.compute_features_optimal(g["xyz"], nn, ptr, 1, 3, 6)
    assert np.mean(o[:, 11] == o32[:, 11]) > 0.99
    assert set(np.unique(o[:, 11])) <= {6, 9, 12, 15, 18, 20}
    with pytest.raises(ValueError):
        oracle.compute_features_f64(xyz, nn, ptr, 0)
