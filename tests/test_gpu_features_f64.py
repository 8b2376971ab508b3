"""Float64 CSR feature passes (compute_features*_f64) against the oracle's
double instantiation of include/pgeof.hpp:75-310.

The device runs the oracle's arithmetic in double (sequential two-pass
covariance without FMA, the same cyclic Jacobi with explicit rounding), so
most values are bit-identical; pow (Volume) and log (eigentropy, hence the
optimal k on exact ties) come from CUDA's libdevice instead of glibc and may
differ in the last bits. Tolerance: |gpu - oracle| <= 1e-12 * max(1, |oracle|)
on every value of rows whose optimal k agrees."""

import numpy as np
import pytest

from oracle import oracle
from point_geometric_features_gb300.synthetic import outdoor_scene, uniform_cube

pytestmark = pytest.mark.gpu

TOL = 1e-12


def _close(a, b):
    return np.abs(a - b) <= TOL * np.maximum(1.0, np.abs(b))


def _knn_csr(xyz32, k):
    idx, _ = oracle.knn_search(xyz32, xyz32, k)
    return idx.reshape(-1).astype(np.uint32), (np.arange(xyz32.shape[0] + 1) * k).astype(np.uint32)


def _radius_csr(xyz32, r, max_knn, n_rows=None):
    """CSR of radius neighbourhoods of the first n_rows points (all by default)
    in the whole cloud: ragged rows, from 1 to max_knn neighbours."""
    idx, _ = oracle.radius_search(xyz32, xyz32[:n_rows], r, max_knn)
    cnt = (idx >= 0).sum(1)
    return idx[idx >= 0].astype(np.uint32), np.r_[0, np.cumsum(cnt)].astype(np.uint32)


@pytest.fixture(scope="module")
def scene():
    xyz32 = outdoor_scene(20_000, seed=21)
    return xyz32, xyz32.astype(np.float64)


def test_f64_compute_features_matches_oracle(cuda, pgeof, scene):
    xyz32, xyz = scene
    nn, ptr = _knn_csr(xyz32, 20)
    got = pgeof.compute_features_f64(xyz, nn, ptr)
    want = oracle.compute_features_f64(xyz, nn, ptr)
    assert got.dtype == np.float64 and got.shape == want.shape
    assert _close(got, want).all()
    exact = (got == want).mean(0)
    assert np.delete(exact, 9).min() > 0.99, exact  # all but Volume (pow) bit-identical almost everywhere
    # against the independent numpy FP64 restatement (eigh) on well-separated
    # eigenvalues: the float64 path is exact to ~1e-9, while the float32 path
    # loses digits to the 100 m coordinate offset (x - mean in float)
    ref = oracle.fp64_compute_features(xyz32, nn, ptr)
    ok = oracle.fp64_relative_gap(xyz32[nn.reshape(-1, 20)]) > 1e-6
    cols = [0, 1, 2, 3, 7, 8, 9, 10]
    f32 = pgeof.compute_features(xyz32, nn, ptr)

    def err(a):
        return (np.abs(a[ok][:, cols] - ref[ok][:, cols]) / np.maximum(1.0, np.abs(ref[ok][:, cols]))).max()

    e64, e32 = err(got), err(f32)
    print(f"\nmax scaled error vs numpy FP64: float64 path {e64:.3e}, float32 path {e32:.3e}")
    assert e64 < 1e-8 and e64 < e32


def test_f64_k_min_and_ragged_rows(cuda, pgeof, scene):
    xyz32, xyz = scene
    nn, ptr = _radius_csr(xyz32, 3.0, 24, 5000)
    for k_min in (1, 3, 10):
        got = pgeof.compute_features_f64(xyz, nn, ptr, k_min)
        want = oracle.compute_features_f64(xyz, nn, ptr, k_min)
        assert _close(got, want).all()
        short = np.diff(ptr) < k_min
        assert np.all(got[short] == 0)


def test_f64_multiscale_matches_oracle(cuda, pgeof, scene):
    xyz32, xyz = scene
    nn, ptr = _radius_csr(xyz32, 3.5, 40)
    scales = [4, 10, 10, 25, 40]
    got = pgeof.compute_features_multiscale_f64(xyz, nn, ptr, scales)
    want = oracle.compute_features_f64(xyz, nn, ptr, kind="multi", k_scales=scales)
    assert got.shape == (xyz.shape[0], len(scales), 11)
    assert _close(got, want).all()
    sizes = np.diff(ptr)
    for s, ks in enumerate(scales):  # include/pgeof.hpp:183-199: the first unfillable scale stops the row
        assert np.all(got[sizes < ks, s:] == 0)


@pytest.mark.parametrize("k_min,k_step,k_min_search", [(1, 1, 10), (5, 4, 1)])
def test_f64_optimal_matches_oracle(cuda, pgeof, scene, k_min, k_step, k_min_search):
    xyz32, xyz = scene
    nn, ptr = _radius_csr(xyz32, 3.5, 48, 8000)
    got = pgeof.compute_features_optimal_f64(xyz, nn, ptr, k_min, k_step, k_min_search)
    want = oracle.compute_features_f64(xyz, nn, ptr, k_min, kind="optimal", k_step=k_step,
                                       k_min_search=k_min_search)
    agree = got[:, 11] == want[:, 11]
    print(f"[parity] f64 optimal ({k_min},{k_step},{k_min_search}) k_opt mismatch "
          f"{int((~agree).sum())}/{agree.size} rows = {1.0 - agree.mean():.2e}")
    assert agree.mean() >= 0.999
    assert _close(got[agree], want[agree]).all()
    assert (got[:, 11] > 0).mean() > 0.5  # most rows reach k_min_search


def test_f64_device_tensors_equal_numpy(cuda, pgeof, scene):
    torch = cuda
    xyz32, xyz = scene
    nn, ptr = _knn_csr(xyz32, 16)
    t = torch.from_numpy(xyz).cuda()
    tn = torch.from_numpy(nn.view(np.int32)).cuda()
    tp = torch.from_numpy(ptr.view(np.int32)).cuda()
    for dev, host in (
        (pgeof.compute_features(t, tn, tp), pgeof.compute_features_f64(xyz, nn, ptr)),
        (pgeof.compute_features_multiscale(t, tn, tp, [8, 16]),
         pgeof.compute_features_multiscale_f64(xyz, nn, ptr, [8, 16])),
        (pgeof.compute_features_optimal_f64(t, tn, tp, 1, 2, 8),
         pgeof.compute_features_optimal_f64(xyz, nn, ptr, 1, 2, 8)),
    ):
        assert dev.dtype == torch.float64 and dev.is_cuda
        np.testing.assert_array_equal(dev.cpu().numpy(), host)


def test_f64_data_errors(cuda, pgeof):
    xyz = uniform_cube(50, seed=22).astype(np.float64)
    nn = np.arange(50, dtype=np.uint32)
    nn[7] = 50
    ptr = np.array([0, 25, 50], np.uint32)
    with pytest.raises(ValueError, match="nn holds an index"):
        pgeof.compute_features_f64(xyz, nn, ptr)
    with pytest.raises(ValueError, match="nn_ptr"):
        pgeof.compute_features_optimal_f64(xyz, np.arange(50, dtype=np.uint32), np.array([0, 30, 20], np.uint32))
