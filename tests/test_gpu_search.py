"""GPU neighbour search parity (include/nn_search.hpp:31-132) against the
oracle and scipy, through the drop-in Python API (pgeof_ext -> C ABI)."""

import numpy as np
import pytest
from scipy.spatial import KDTree

from conftest import feature_close
from oracle import oracle
from point_geometric_features_gb300.synthetic import outdoor_scene, uniform_cube

pytestmark = pytest.mark.gpu


def test_reference_test_knn(cuda, pgeof, golden):
    """tests/test_pgeof.py:8-15 with the committed seeded fixture."""
    g = golden("knn_1000_k10.npz")
    idx, d2 = pgeof.knn_search(g["xyz"], g["xyz"], 10)
    assert idx.dtype == np.uint32 and d2.dtype == np.float32 and idx.shape == (1000, 10)
    np.testing.assert_equal(idx.astype(np.int64), g["scipy_idx"])


def test_reference_test_radius(cuda, pgeof, golden):
    """tests/test_pgeof.py:18-27 with the committed seeded fixture."""
    g = golden("radius_1000_r02_k10.npz")
    idx, d2 = pgeof.radius_search(g["xyz"], g["xyz"], 0.2, 10)
    assert idx.dtype == np.int32 and idx.shape == (1000, 10)
    np.testing.assert_equal(idx.astype(np.int64), g["scipy_idx"])


@pytest.mark.parametrize("k", [1, 2, 7, 20, 50, 64, 100])
def test_knn_exact_uniform(cuda, pgeof, k):
    xyz = uniform_cube(10_000, seed=k)
    idx, d2 = pgeof.knn_search(xyz, xyz, k)
    ri, rd = oracle.knn_search(xyz, xyz, k)
    np.testing.assert_array_equal(d2, rd)  # bit-identical float distances
    np.testing.assert_array_equal(idx, ri)


def test_knn_exact_scene(cuda, pgeof):
    xyz = outdoor_scene(40_000, seed=1)
    idx, d2 = pgeof.knn_search(xyz, xyz, 50)
    ri, rd = oracle.knn_search(xyz, xyz, 50)
    np.testing.assert_array_equal(d2, rd)
    np.testing.assert_array_equal(idx, ri)


def test_knn_separate_queries_outside_box(cuda, pgeof):
    rng = np.random.default_rng(3)
    data = rng.random((5000, 3), dtype=np.float32)
    query = (rng.random((777, 3), dtype=np.float32) * 3.0 - 1.0).astype(np.float32)  # many outside the data box
    idx, d2 = pgeof.knn_search(data, query, 12)
    ri, rd = oracle.knn_search(data, query, 12)
    np.testing.assert_array_equal(d2, rd)
    np.testing.assert_array_equal(idx, ri)


def test_knn_k_equals_n(cuda, pgeof):
    xyz = uniform_cube(300, seed=4)
    idx, d2 = pgeof.knn_search(xyz, xyz, 300)
    ri, rd = oracle.knn_search(xyz, xyz, 300)
    np.testing.assert_array_equal(idx, ri)
    np.testing.assert_array_equal(d2, rd)


def test_knn_duplicates_ties_by_index(cuda, pgeof):
    """Many exact duplicates force the refinement passes (equal distances are
    ordered by index)."""
    rng = np.random.default_rng(5)
    base = rng.random((200, 3), dtype=np.float32)
    xyz = np.concatenate([base, np.repeat(base[:3], 400, axis=0), rng.random((2000, 3), dtype=np.float32)])
    xyz = np.ascontiguousarray(xyz.astype(np.float32))
    for k in (5, 64, 450):
        idx, d2 = pgeof.knn_search(xyz, xyz, k)
        ri, rd = oracle.knn_search(xyz, xyz, k)
        np.testing.assert_array_equal(d2, rd)
        np.testing.assert_array_equal(idx, ri)


def test_knn_planar_and_single_axis(cuda, pgeof):
    rng = np.random.default_rng(6)
    plane = rng.random((4000, 3), dtype=np.float32)
    plane[:, 2] = 0.0
    line = np.zeros((1000, 3), np.float32)
    line[:, 0] = rng.random(1000, dtype=np.float32)
    for xyz in (plane, line):
        idx, d2 = pgeof.knn_search(xyz, xyz, 16)
        ri, rd = oracle.knn_search(xyz, xyz, 16)
        np.testing.assert_array_equal(d2, rd)
        np.testing.assert_array_equal(idx, ri)


def test_knn_errors_and_empty(cuda, pgeof):
    xyz = uniform_cube(10, seed=1)
    with pytest.raises(ValueError):
        pgeof.knn_search(xyz, xyz, 11)
    with pytest.raises(TypeError):
        pgeof.knn_search(xyz.astype(np.float64), xyz, 2)
    idx, d2 = pgeof.knn_search(xyz, np.zeros((0, 3), np.float32), 3)
    assert idx.shape == (0, 3)
    idx, d2 = pgeof.knn_search(xyz, xyz, 0)
    assert idx.shape == (10, 0)
    one = np.array([[0.5, 0.5, 0.5]], np.float32)
    idx, d2 = pgeof.knn_search(one, one, 1)
    assert idx[0, 0] == 0 and d2[0, 0] == 0


@pytest.mark.parametrize("r,k", [(0.05, 30), (0.1, 16), (0.02, 64), (0.3, 8)])
def test_radius_exact(cuda, pgeof, r, k):
    xyz = uniform_cube(8000, seed=int(r * 1000))
    idx, d2 = pgeof.radius_search(xyz, xyz, r, k)
    ri, rd = oracle.radius_search(xyz, xyz, r, k)
    np.testing.assert_array_equal(idx, ri)
    np.testing.assert_array_equal(d2, rd)  # includes nanoflann's r^2 in the last slot of short rows


def test_radius_scene_and_queries(cuda, pgeof):
    data = outdoor_scene(30_000, seed=2)
    rng = np.random.default_rng(2)
    query = data[rng.choice(data.shape[0], 3000, replace=False)] + rng.normal(0, 0.3, (3000, 3)).astype(np.float32)
    query = np.ascontiguousarray(query.astype(np.float32))
    idx, d2 = pgeof.radius_search(data, query, 0.5, 64)
    ri, rd = oracle.radius_search(data, query, 0.5, 64)
    np.testing.assert_array_equal(idx, ri)
    np.testing.assert_array_equal(d2, rd)


def test_radius_errors(cuda, pgeof):
    xyz = uniform_cube(10, seed=1)
    with pytest.raises(ValueError):
        pgeof.radius_search(xyz, xyz, 0.1, 11)
    idx, d2 = pgeof.radius_search(xyz, xyz, 0.1, 0)
    assert idx.shape == (10, 0)


def test_knn_matches_scipy_large(cuda, pgeof):
    """bench_knn.py shapes at 200k points: identical to scipy except at exact ties."""
    rng = np.random.default_rng(21)
    xyz = rng.uniform(0.0, 200.0, size=(200_000, 3)).astype(np.float32)
    idx, _ = pgeof.knn_search(xyz, xyz, 50)
    _, ref = KDTree(xyz).query(xyz[:5000], k=50, workers=-1)
    mism = (idx[:5000].astype(np.int64) != ref).any(axis=1).mean()
    assert mism < 1e-3, mism


def test_knn_full_size_properties(cuda, pgeof):
    """1M-point outdoor scene, k=50: sorted rows, self first, distances that
    recompute exactly from the returned indices, and a 2000-query spot check
    against the oracle's brute force."""
    xyz = outdoor_scene(1_000_000, seed=1)
    idx, d2 = pgeof.knn_search(xyz, xyz, 50)
    assert np.all(np.diff(d2, axis=1) >= 0)
    assert np.all(d2[:, 0] == 0)
    rng = np.random.default_rng(0)
    rows = rng.choice(xyz.shape[0], 2000, replace=False)
    diff = (xyz[rows][:, None, :] - xyz[idx[rows]]).astype(np.float32)
    rec = (diff[..., 0] * diff[..., 0] + diff[..., 1] * diff[..., 1]).astype(np.float32)
    rec = (rec + diff[..., 2] * diff[..., 2]).astype(np.float32)
    np.testing.assert_array_equal(rec, d2[rows])
    ri, rd = oracle.knn_search(xyz, xyz[rows], 50)
    np.testing.assert_array_equal(d2[rows], rd)
    np.testing.assert_array_equal(idx[rows], ri)


def test_knn_deterministic(cuda, pgeof):
    xyz = outdoor_scene(50_000, seed=9)
    a = pgeof.knn_search(xyz, xyz, 32)
    b = pgeof.knn_search(xyz, xyz, 32)
    np.testing.assert_array_equal(a[0], b[0])
    np.testing.assert_array_equal(a[1], b[1])


def _csr_from_table(idx):
    """pgeof README.md:157-163: drop the -1 padding, row counts -> offsets."""
    idx = np.asarray(idx)
    mask = idx >= 0
    ptr = np.zeros(idx.shape[0] + 1, np.uint32)
    ptr[1:] = np.cumsum(mask.sum(1))
    return idx[mask].astype(np.uint32), ptr


@pytest.mark.parametrize("max_knn", [1, 7, 64])
def test_radius_search_csr_matches_padded_table(cuda, pgeof, max_knn):
    torch = cuda
    xyz = outdoor_scene(60_000, seed=13)
    t = torch.from_numpy(xyz).cuda()
    for q, r in ((t, 0.5), (torch.from_numpy(uniform_cube(5_000, seed=3, side=100.0)).cuda(), 2.0)):
        idx, _ = pgeof.radius_search(t, q, r, max_knn)
        nn, ptr = pgeof.radius_search_csr(t, q, r, max_knn)
        ref_nn, ref_ptr = _csr_from_table(idx.cpu().numpy())
        np.testing.assert_array_equal(ptr.view(torch.int32).cpu().numpy().view(np.uint32), ref_ptr)
        np.testing.assert_array_equal(nn.view(torch.int32).cpu().numpy().view(np.uint32), ref_nn)
    # numpy in, numpy out; against the oracle's own table on a small case
    small = xyz[:3_000]
    nn, ptr = pgeof.radius_search_csr(small, small, 0.7, 16)
    o_idx, _ = oracle.radius_search(small, small, 0.7, 16)
    ref_nn, ref_ptr = _csr_from_table(o_idx)
    assert nn.dtype == np.uint32 and ptr.dtype == np.uint32
    np.testing.assert_array_equal(ptr, ref_ptr)
    np.testing.assert_array_equal(nn, ref_nn)


def test_radius_search_csr_edges(cuda, pgeof):
    torch = cuda
    xyz = torch.from_numpy(uniform_cube(1_000, seed=2)).cuda()
    far = xyz + 1000.0  # no neighbour within the radius for any query
    nn, ptr = pgeof.radius_search_csr(xyz, far, 0.1, 8)
    assert nn.numel() == 0 and int(ptr.view(torch.int32).max()) == 0 and ptr.numel() == 1_001
    nn, ptr = pgeof.radius_search_csr(xyz, xyz[:0], 0.1, 8)
    assert nn.numel() == 0 and ptr.numel() == 1
    with pytest.raises(ValueError):
        pgeof.radius_search_csr(xyz, xyz, 0.1, 2_000)  # max_knn > n
    # the CSR feeds compute_features_optimal directly
    nn, ptr = pgeof.radius_search_csr(xyz, xyz, 0.3, 32)
    out = pgeof.compute_features_optimal(xyz, nn, ptr, 1, 1, 5)
    idx, _ = pgeof.radius_search(xyz, xyz, 0.3, 32)
    ref_nn, ref_ptr = _csr_from_table(idx.cpu().numpy())
    ref = pgeof.compute_features_optimal(xyz.cpu().numpy(), ref_nn, ref_ptr, 1, 1, 5)
    np.testing.assert_array_equal(out.cpu().numpy(), ref)


def test_host_knn_pipeline_large_matches_device_path(cuda, pgeof):
    """Results of >= 128 MB take the chunked host path (query row chunks sorted
    and searched in turn, downloads overlapped): identical to the device path,
    for the cloud itself and for separate queries."""
    torch = cuda
    xyz = outdoor_scene(400_000, seed=41)
    t = torch.from_numpy(xyz).cuda()
    i_d, d_d = pgeof.knn_search(t, t, 50)
    i_h, d_h = pgeof.knn_search(xyz, xyz, 50)
    np.testing.assert_array_equal(i_h, i_d.cpu().numpy().astype(np.uint32))
    np.testing.assert_array_equal(d_h, d_d.cpu().numpy())
    q = uniform_cube(420_000, seed=42, side=100.0)
    q[:, 2] *= 0.2
    qt = torch.from_numpy(q).cuda()
    i_d, d_d = pgeof.knn_search(t, qt, 40)
    i_h, d_h = pgeof.knn_search(xyz, q, 40)
    np.testing.assert_array_equal(i_h, i_d.cpu().numpy().astype(np.uint32))
    np.testing.assert_array_equal(d_h, d_d.cpu().numpy())


def test_all_points_identical(cuda, pgeof):
    """A cloud collapsed to one position: every distance is 0, so every row is
    the lowest indices in order (include/nn_search.hpp:31-132 with the
    (distance, index) tie order) and the grid has a single cell."""
    xyz = np.full((3000, 3), 0.25, np.float32)
    for k in (1, 50, 200):
        idx, d2 = pgeof.knn_search(xyz, xyz, k)
        assert np.all(d2 == 0)
        np.testing.assert_array_equal(idx, np.broadcast_to(np.arange(k, dtype=np.uint32), idx.shape))
    idx, d2 = pgeof.radius_search(xyz, xyz, 0.1, 64)
    np.testing.assert_array_equal(idx, np.broadcast_to(np.arange(64, dtype=np.int32), idx.shape))
    ri, rd = oracle.radius_search(xyz, xyz[:50], 0.1, 64)
    np.testing.assert_array_equal(idx[:50], ri)
    np.testing.assert_array_equal(d2[:50], rd)
    nn = idx[:, :20].reshape(-1).astype(np.uint32)
    ptr = (np.arange(xyz.shape[0] + 1) * 20).astype(np.uint32)
    assert feature_close(pgeof.compute_features(xyz, nn, ptr), oracle.compute_features(xyz, nn, ptr)).all()
