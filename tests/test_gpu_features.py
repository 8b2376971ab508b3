"""GPU feature-pass parity (include/pgeof.hpp:75-310, include/pca.hpp) against
the oracle, through the drop-in Python API (pgeof_ext -> C ABI).

Tolerance: the GPU forms the covariance with the reference's exact float
operation order (bit-identical to the oracle's), so differences come only from
the eigen solver: |gpu - oracle| <= 1e-4 * max(1, |oracle|) per value (the
ascending-order ratios reach ~1e3, hence relative above 1). Each test prints
the per-feature maximum of that scaled error. Normals are compared after sign
alignment where the reference's z-flip is undefined (|n_z| < 1e-4). Optimal-k
tests print the fraction of rows whose k_opt differs from the oracle's.
"""

import os

import numpy as np
import pytest

from conftest import align_normals, feature_close, feature_report
from oracle import oracle
from point_geometric_features_gb300.synthetic import outdoor_scene, uniform_cube

pytestmark = pytest.mark.gpu


def _csr(idx):
    k = idx.shape[1]
    return idx.reshape(-1).astype(np.uint32), (np.arange(idx.shape[0] + 1) * k).astype(np.uint32)


def _radius_csr(idx):
    cnt = (idx >= 0).sum(axis=1)
    return idx[idx >= 0].astype(np.uint32), np.r_[0, np.cumsum(cnt)].astype(np.uint32)


def _assert_features(gpu, ref, label=""):
    g = align_normals(gpu, ref)
    feature_report(g, ref, label=label)
    ok = feature_close(g, ref)
    rate = ok.all(axis=-1).mean() if ok.size else 1.0
    assert rate == 1.0, f"{label}: only {rate:.6f} of rows within tolerance"


def _k_opt_mismatch(gpu, ref, label, limit=1e-3):
    """Fraction of rows whose optimal k differs from the oracle's (printed)."""
    diff = gpu[:, 11] != ref[:, 11]
    rate = float(diff.mean())
    print(f"[parity] {label} k_opt mismatch {int(diff.sum())}/{diff.size} rows = {rate:.2e}")
    assert rate <= limit, f"{label}: k_opt differs on {rate:.2e} of rows"
    return ~diff


def test_golden_features(cuda, pgeof, golden):
    g = golden("features_2000_k20.npz")
    nn, nn_ptr = _csr(g["idx"])
    _assert_features(pgeof.compute_features(g["xyz"], nn, nn_ptr), g["features"], "golden features")
    _assert_features(pgeof.compute_features_multiscale(g["xyz"], nn, nn_ptr, [5, 10, 20]), g["multiscale"],
                     "golden multiscale")
    opt = pgeof.compute_features_optimal(g["xyz"], nn, nn_ptr, 1, 1, 5)
    same = _k_opt_mismatch(opt, g["optimal"], "golden optimal")
    _assert_features(opt[same], g["optimal"][same], "golden optimal")


def test_c1_uniform_10k_k20(cuda, pgeof):
    """10k uniform points, knn k=20 -> CSR -> compute_features(k_min=1)."""
    xyz = uniform_cube(10_000, seed=0)
    idx, _ = pgeof.knn_search(xyz, xyz, 20)
    nn, nn_ptr = _csr(idx)
    f = pgeof.compute_features(xyz, nn, nn_ptr)
    assert f.shape == (10_000, 11) and f.dtype == np.float32
    _assert_features(f, oracle.compute_features(xyz, nn, nn_ptr), "C1 10k cube k=20")
    # against the FP64 oracle, well-conditioned rows
    f64 = oracle.fp64_compute_features(xyz, nn, nn_ptr)
    gap = oracle.fp64_relative_gap(xyz[idx])
    sel = gap > 1e-2
    err = np.abs(f[sel] - f64[sel]) / np.maximum(1.0, np.abs(f64[sel]))
    assert err.max() < 5e-4


def test_scene_multiscale(cuda, pgeof):
    """The outdoor scene at 50k points: knn k=50 -> multiscale [10, 20, 50]."""
    xyz = outdoor_scene(50_000, seed=1)
    idx, _ = pgeof.knn_search(xyz, xyz, 50)
    nn, nn_ptr = _csr(idx)
    m = pgeof.compute_features_multiscale(xyz, nn, nn_ptr, [10, 20, 50])
    assert m.shape == (50_000, 3, 11)
    _assert_features(m, oracle.compute_features_multiscale(xyz, nn, nn_ptr, [10, 20, 50]), "scene 50k multiscale")
    # reference self-consistency (tests/test_pgeof.py:30-46)
    single = pgeof.compute_features(xyz, nn, nn_ptr, 50)
    np.testing.assert_array_equal(m[:, 2], single)


def test_k_min_gating_and_ragged_rows(cuda, pgeof):
    xyz = uniform_cube(3000, seed=2)
    idx, _ = pgeof.radius_search(xyz, xyz, 0.06, 40)
    nn, nn_ptr = _radius_csr(idx)
    for k_min in (1, 3, 10, 25):
        f = pgeof.compute_features(xyz, nn, nn_ptr, k_min)
        ref = oracle.compute_features(xyz, nn, nn_ptr, k_min)
        _assert_features(f, ref, f"ragged k_min={k_min}")
        short = np.diff(nn_ptr) < k_min
        assert np.all(f[short] == 0)
    m = pgeof.compute_features_multiscale(xyz, nn, nn_ptr, [2, 5, 5, 12, 30])
    _assert_features(m, oracle.compute_features_multiscale(xyz, nn, nn_ptr, [2, 5, 5, 12, 30]), "ragged multiscale")


def test_many_scales(cuda, pgeof):
    """more scales than one launch handles (chunks of 8)."""
    xyz = uniform_cube(2000, seed=3)
    idx, _ = pgeof.knn_search(xyz, xyz, 40)
    nn, nn_ptr = _csr(idx)
    scales = [2, 3, 4, 5, 6, 8, 10, 12, 15, 20, 25, 30, 40]
    m = pgeof.compute_features_multiscale(xyz, nn, nn_ptr, scales)
    _assert_features(m, oracle.compute_features_multiscale(xyz, nn, nn_ptr, scales), "13 scales")
    empty = pgeof.compute_features_multiscale(xyz, nn, nn_ptr, [])
    assert empty.shape == (2000, 0, 11)


def test_optimal_radius_csr(cuda, pgeof):
    """The outdoor scene at 40k points: radius 0.5 / max 64 -> optimal(k_min=1, k_step=1, k_min_search=10)."""
    xyz = outdoor_scene(40_000, seed=2)
    idx, _ = pgeof.radius_search(xyz, xyz, 0.5, 64)
    nn, nn_ptr = _radius_csr(idx)
    f = pgeof.compute_features_optimal(xyz, nn, nn_ptr, 1, 1, 10)
    ref = oracle.compute_features_optimal(xyz, nn, nn_ptr, 1, 1, 10)
    same = _k_opt_mismatch(f, ref, "optimal scene 40k radius")
    _assert_features(f[same], ref[same], "optimal scene 40k radius")
    short = np.diff(nn_ptr) < 10
    assert np.all(f[short] == 0)


@pytest.mark.parametrize("k_step", [2, 5])
def test_optimal_steps(cuda, pgeof, k_step):
    xyz = uniform_cube(3000, seed=k_step)
    idx, _ = pgeof.knn_search(xyz, xyz, 33)
    nn, nn_ptr = _csr(idx)
    f = pgeof.compute_features_optimal(xyz, nn, nn_ptr, 3, k_step, 7)
    ref = oracle.compute_features_optimal(xyz, nn, nn_ptr, 3, k_step, 7)
    same = _k_opt_mismatch(f, ref, f"optimal k_step={k_step}")
    _assert_features(f[same], ref[same], f"optimal k_step={k_step}")


def test_degenerate_neighbourhoods(cuda, pgeof):
    """k = 1, 2, 3, collinear, coplanar and duplicate points."""
    rng = np.random.default_rng(11)
    pts = [rng.random((1, 3)), rng.random((2, 3)), rng.random((3, 3))]
    t = rng.random(9)
    pts.append(np.stack([t, 2 * t, -t], 1))  # line
    p = rng.random((12, 3))
    p[:, 2] = 0.25
    pts.append(p)  # horizontal plane
    pts.append(np.repeat(rng.random((1, 3)), 6, axis=0))  # duplicates
    xyz = np.concatenate(pts).astype(np.float32)
    sizes = [len(p) for p in pts]
    nn = np.arange(xyz.shape[0], dtype=np.uint32)
    nn_ptr = np.r_[0, np.cumsum(sizes)].astype(np.uint32)
    f = pgeof.compute_features(xyz, nn, nn_ptr)
    ref = oracle.compute_features(xyz, nn, nn_ptr)
    _assert_features(f, ref, "degenerate neighbourhoods")


def test_near_degenerate_neighbourhoods(cuda, pgeof):
    """Neighbourhoods whose two largest or two smallest eigenvalues differ by a
    relative 1e-2 ... 1e-7 (regular polygons and octahedra, stretched by 1 + eps
    and rotated): the eigenvectors there are ill-conditioned, which is where
    the small-gap solves (double-float, float64 below 1e-7) take over."""
    rng = np.random.default_rng(23)
    blocks = []
    for eps in (1e-2, 1e-3, 1e-4, 1e-5, 1e-6, 1e-7, 0.0):
        for _ in range(40):
            m = int(rng.integers(8, 40))
            a = np.linspace(0.0, 2.0 * np.pi, m, endpoint=False) + rng.random()
            if rng.random() < 0.5:  # polygon: two equal large eigenvalues, small normal one
                p = np.stack([np.cos(a) * (1.0 + eps), np.sin(a), 1e-3 * rng.standard_normal(m)], 1)
            else:  # polygon plus poles: the two small eigenvalues nearly equal
                p = np.stack([np.cos(a), np.sin(a), np.zeros(m)], 1) * np.array([0.2, 0.2 * (1.0 + eps), 0.0])
                p[:, 0] += np.linspace(-1.0, 1.0, m)
            q, _ = np.linalg.qr(rng.standard_normal((3, 3)))
            blocks.append(p @ q.T * rng.uniform(0.1, 10.0) + rng.uniform(-50.0, 50.0, 3))
    xyz = np.concatenate(blocks).astype(np.float32)
    sizes = [len(b) for b in blocks]
    nn = np.arange(xyz.shape[0], dtype=np.uint32)
    nn_ptr = np.r_[0, np.cumsum(sizes)].astype(np.uint32)
    f = pgeof.compute_features(xyz, nn, nn_ptr)
    ref = oracle.compute_features(xyz, nn, nn_ptr)
    _assert_features(f, ref, "near-degenerate neighbourhoods")
    f3 = pgeof.compute_features_multiscale(xyz, nn, nn_ptr, [4, 8])
    ref3 = oracle.compute_features_multiscale(xyz, nn, nn_ptr, [4, 8])
    _assert_features(f3, ref3, "near-degenerate neighbourhoods, scales 4 and 8")


def test_csr_validation(cuda, pgeof):
    xyz = uniform_cube(100, seed=1)
    nn = np.arange(100, dtype=np.uint32)
    with pytest.raises(ValueError):
        pgeof.compute_features(xyz, np.r_[nn[:-1], 100].astype(np.uint32), np.array([0, 50, 100], np.uint32))
    with pytest.raises(ValueError):
        pgeof.compute_features(xyz, nn, np.array([0, 60, 50, 100], np.uint32))
    with pytest.raises(ValueError):
        pgeof.compute_features(xyz, nn, np.array([0, 50, 101], np.uint32))
    with pytest.raises(ValueError):
        pgeof.compute_features_multiscale(xyz, nn, np.array([0, 50, 100], np.uint32), [20, 10])
    with pytest.raises(ValueError):
        pgeof.compute_features_optimal(xyz, nn, np.array([0, 50, 100], np.uint32), 0, 1, 0)
    with pytest.raises(TypeError):
        pgeof.compute_features(xyz, nn.astype(np.int64), np.array([0, 50, 100], np.uint32))
    out = pgeof.compute_features(xyz, nn, np.array([0], np.uint32))
    assert out.shape == (0, 11)
    # the device stays usable after a data error
    ok = pgeof.compute_features(xyz, nn, np.array([0, 50, 100], np.uint32))
    assert np.isfinite(ok).all()


def test_descending_order_switch(cuda, pgeof):
    xyz = outdoor_scene(20_000, seed=4)
    idx, _ = pgeof.knn_search(xyz, xyz, 20)
    nn, nn_ptr = _csr(idx)
    try:
        pgeof.set_eig_order("descending")
        f = pgeof.compute_features(xyz, nn, nn_ptr)
    finally:
        pgeof.set_eig_order("ascending")
    ref = oracle.compute_features(xyz, nn, nn_ptr, order=oracle.EIG_DESCENDING)
    _assert_features(f, ref, "descending order")
    ground = np.abs(xyz[:, 2]) < 0.03
    assert np.median(f[ground, 6]) > 0.99  # normals of the ground plane point up


def test_full_size_multiscale_properties(cuda, pgeof):
    """1M-point scene, k=50, scales [10, 20, 50]: finite, row-consistent with
    the single-scale call, and a 5000-row sample equal to the oracle."""
    xyz = outdoor_scene(1_000_000, seed=1)
    idx, _ = pgeof.knn_search(xyz, xyz, 50)
    nn, nn_ptr = _csr(idx)
    m = pgeof.compute_features_multiscale(xyz, nn, nn_ptr, [10, 20, 50])
    assert np.isfinite(m).all()
    rng = np.random.default_rng(1)
    rows = rng.choice(xyz.shape[0], 5000, replace=False)
    sub_nn = idx[rows].reshape(-1).astype(np.uint32)
    sub_ptr = (np.arange(rows.size + 1) * 50).astype(np.uint32)
    ref = oracle.compute_features_multiscale(xyz, sub_nn, sub_ptr, [10, 20, 50])
    _assert_features(m[rows], ref, "1M scene multiscale, 5000-row sample")


@pytest.mark.parametrize("k", [8, 50])
def test_knn_features_equals_separate_calls(cuda, pgeof, k):
    """The fused feature-only pipeline writes exactly what knn_search followed
    by compute_features / compute_features_multiscale writes."""
    torch = cuda
    for xyz in (outdoor_scene(60_000, seed=21), uniform_cube(30_000, seed=22)):
        t = torch.from_numpy(xyz).cuda()
        idx, _ = pgeof.knn_search(t, t, k)
        ptr = torch.arange(0, k * (xyz.shape[0] + 1), k, dtype=torch.int32, device="cuda")
        ref = pgeof.compute_features(t, idx.reshape(-1), ptr)
        got = pgeof.knn_features(t, k)
        assert torch.equal(got, ref)
        scales = [max(1, k // 4), k // 2, k]
        ref3 = pgeof.compute_features_multiscale(t, idx.reshape(-1), ptr, scales)
        got3 = pgeof.knn_features(t, k, scales)
        assert torch.equal(got3, ref3)
    # numpy in, numpy out
    small = uniform_cube(2_000, seed=23)
    got = pgeof.knn_features(small, 10)
    i, _ = pgeof.knn_search(small, small, 10)
    ref = pgeof.compute_features(small, i.reshape(-1), (np.arange(2_001) * 10).astype(np.uint32))
    np.testing.assert_array_equal(got, ref)
    with pytest.raises(ValueError):
        pgeof.knn_features(small, 2_001)
    with pytest.raises(ValueError):
        pgeof.knn_features(small, 10, [5, 20])


def test_host_pipeline_large_csr_matches_device_path(cuda, pgeof):
    """Neighbour lists of >= 64 MB go through the chunked host pipeline (upload,
    feature pass and download of successive row chunks overlapped); results
    must equal the device path's, and bad offsets still raise."""
    torch = cuda
    n, k = 400_000, 50
    xyz = outdoor_scene(n, seed=31)
    t = torch.from_numpy(xyz).cuda()
    idx, _ = pgeof.knn_search(t, t, k)
    nn_h = idx.cpu().numpy().astype(np.uint32).reshape(-1)
    assert nn_h.nbytes >= 64 << 20
    ptr_h = (np.arange(n + 1, dtype=np.int64) * k).astype(np.uint32)
    ptr_d = torch.from_numpy(ptr_h.view(np.int32)).cuda()
    ref1 = pgeof.compute_features(t, idx.reshape(-1), ptr_d).cpu().numpy()
    np.testing.assert_array_equal(pgeof.compute_features(xyz, nn_h, ptr_h), ref1)
    ref3 = pgeof.compute_features_multiscale(t, idx.reshape(-1), ptr_d, [10, 20, 50]).cpu().numpy()
    np.testing.assert_array_equal(pgeof.compute_features_multiscale(xyz, nn_h, ptr_h, [10, 20, 50]), ref3)
    bad = ptr_h.copy()
    bad[n // 2] = bad[n // 2 + 1] + 7  # a decreasing step in the middle chunk
    with pytest.raises(ValueError):
        pgeof.compute_features(xyz, nn_h, bad)


def test_row_order_is_invisible(cuda, tmp_path):
    """Large clouds process CSR rows in the spatial order of their first
    neighbour; forcing that on a small cloud (threshold 1 point) must give
    the same bits as the plain order (threshold 0)."""
    import subprocess
    import sys

    child = os.path.join(os.path.dirname(os.path.abspath(__file__)), "_row_order_child.py")
    outs = {}
    for thr in ("0", "1"):
        path = str(tmp_path / f"rows_{thr}.npz")
        env = dict(os.environ, PGEOF_ROW_ORDER_POINTS=thr)
        subprocess.run([sys.executable, child, path], env=env, check=True, timeout=300)
        outs[thr] = np.load(path)
    for key in ("f1", "f3", "g"):
        np.testing.assert_array_equal(outs["0"][key], outs["1"][key])
