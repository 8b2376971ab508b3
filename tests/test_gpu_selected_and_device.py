"""compute_features_selected (include/pgeof.hpp:325-375, float and double) and
the device-resident entry points: torch CUDA tensors, and the C ABI called
directly with ctypes."""

import ctypes

import numpy as np
import pytest

from conftest import feature_close, feature_report
from oracle import oracle
from point_geometric_features_gb300.synthetic import outdoor_scene, uniform_cube

pytestmark = pytest.mark.gpu

IDS = [12, 10, 1, 6, 13, 3, 0, 2, 4, 5, 7, 8, 9, 11]


def test_golden_selected(cuda, pgeof, golden):
    g = golden("features_2000_k20.npz")
    ids = [pgeof.EFeatureID(int(i)) for i in g["selected_ids"]]
    s32 = pgeof.compute_features_selected(g["xyz"], 0.1, 20, ids)
    s64 = pgeof.compute_features_selected(g["xyz"].astype(np.float64), 0.1, 20, ids)
    assert s32.dtype == np.float32 and s64.dtype == np.float64
    feature_report(s32, g["selected_f32"], label="golden selected f32", names=[str(i) for i in g["selected_ids"]])
    assert feature_close(s32, g["selected_f32"]).all()
    assert feature_close(s64, g["selected_f64"], tol=1e-9).all()


@pytest.mark.parametrize("dtype", [np.float32, np.float64])
def test_selected_scene(cuda, pgeof, dtype):
    """The serving workload's feature list [Verticality, Curvature, Planarity, Normal_z]."""
    xyz = outdoor_scene(20_000, seed=5).astype(dtype)
    ids = [pgeof.Verticality, pgeof.Curvature, pgeof.Planarity, pgeof.Normal_z]
    out = pgeof.compute_features_selected(xyz, 0.4, 32, ids)
    ref = oracle.compute_features_selected(xyz, 0.4, 32, [int(i) for i in ids])
    feature_report(out, ref, label=f"selected scene {np.dtype(dtype).name}",
                   names=["Verticality", "Curvature", "Planarity", "Normal_z"])
    assert feature_close(out, ref, tol=1e-9 if dtype == np.float64 else 1e-4).all()


def test_selected_all_ids_and_isolated(cuda, pgeof):
    """Every EFeatureID, K_optimal stays 0, isolated points (< 2 in radius) are 0."""
    rng = np.random.default_rng(3)
    xyz = np.concatenate([rng.random((3000, 3)), rng.random((20, 3)) + 10.0]).astype(np.float32)
    ids = [pgeof.EFeatureID(i) for i in IDS]
    out = pgeof.compute_features_selected(xyz, 0.08, 24, ids)
    ref = oracle.compute_features_selected(xyz, 0.08, 24, IDS)
    feature_report(out, ref, label="selected all ids", names=[str(i) for i in IDS])
    assert feature_close(out, ref).all()
    assert np.all(out[:, IDS.index(11)] == 0)
    assert np.all(out[3000:] == 0)


def test_selected_reference_bench_shape(cuda, pgeof):
    """tests/bench_jakteristics.py:12-45: 10k float64 points in [0, 200)^3, r=5, max 50, [Verticality]."""
    rng = np.random.default_rng(12)
    xyz = rng.uniform(0.0, 200.0, size=(10_000, 3))
    out = pgeof.compute_features_selected(xyz, 5.0, 50, [pgeof.Verticality])
    ref = oracle.compute_features_selected(xyz, 5.0, 50, [12])
    assert feature_close(out, ref, tol=1e-9).all()


def test_torch_device_path(cuda, pgeof):
    torch = cuda
    xyz = outdoor_scene(30_000, seed=6)
    t = torch.from_numpy(xyz).cuda()
    idx, d2 = pgeof.knn_search(t, t, 24)
    assert idx.is_cuda and d2.is_cuda
    ri, rd = pgeof.knn_search(xyz, xyz, 24)
    np.testing.assert_array_equal(idx.cpu().numpy().astype(np.uint32), ri)
    np.testing.assert_array_equal(d2.cpu().numpy(), rd)
    nn = idx.reshape(-1)
    nn_ptr = torch.arange(0, 24 * (xyz.shape[0] + 1), 24, device="cuda", dtype=torch.int32)
    f = pgeof.compute_features_multiscale(t, nn, nn_ptr, [8, 24])
    fh = pgeof.compute_features_multiscale(xyz, ri.reshape(-1), nn_ptr.cpu().numpy().astype(np.uint32), [8, 24])
    np.testing.assert_array_equal(f.cpu().numpy(), fh)
    ridx, rd2 = pgeof.radius_search(t, t, 0.3, 16)
    hi, hd = pgeof.radius_search(xyz, xyz, 0.3, 16)
    np.testing.assert_array_equal(ridx.cpu().numpy(), hi)
    sel = pgeof.compute_features_selected(t.double(), 0.3, 16, [pgeof.Verticality])
    np.testing.assert_array_equal(sel.cpu().numpy(),
                                  pgeof.compute_features_selected(xyz.astype(np.float64), 0.3, 16, [pgeof.Verticality]))
    bad = torch.tensor([0, 5, 3], dtype=torch.int32, device="cuda")
    with pytest.raises(ValueError):
        pgeof.compute_features(t, nn, bad)


def test_c_abi_direct(cuda, pgeof):
    """Call libpgeof_cuda.so through ctypes with device pointers, like a
    non-Python caller of include/pgeof_cuda.h would."""
    torch = cuda
    lib = ctypes.CDLL(pgeof.LIBRARY_PATH)
    P, I64, U32 = ctypes.c_void_p, ctypes.c_int64, ctypes.c_uint32
    lib.pgeof_knn_search_f32.argtypes = [P, I64, P, I64, U32, P, P, P]
    lib.pgeof_compute_features_f32.argtypes = [P, I64, P, I64, P, I64, ctypes.c_uint64, P, P]
    lib.pgeof_take_device_errors.argtypes = [P, ctypes.POINTER(ctypes.c_uint32)]
    xyz = uniform_cube(5000, seed=8)
    t = torch.from_numpy(xyz).cuda()
    k = 10
    idx = torch.empty((5000, k), dtype=torch.int32, device="cuda")
    d2 = torch.empty((5000, k), dtype=torch.float32, device="cuda")
    s = torch.cuda.current_stream().cuda_stream
    assert lib.pgeof_knn_search_f32(t.data_ptr(), 5000, t.data_ptr(), 5000, k, idx.data_ptr(), d2.data_ptr(), s) == 0
    ptr = torch.arange(0, k * 5001, k, dtype=torch.int32, device="cuda")
    out = torch.empty((5000, 11), dtype=torch.float32, device="cuda")
    assert lib.pgeof_compute_features_f32(t.data_ptr(), 5000, idx.data_ptr(), 5000 * k, ptr.data_ptr(), 5000, 1,
                                          out.data_ptr(), s) == 0
    bits = ctypes.c_uint32(99)
    assert lib.pgeof_take_device_errors(s, ctypes.byref(bits)) == 0 and bits.value == 0
    ri, _ = oracle.knn_search(xyz, xyz, k)
    np.testing.assert_array_equal(idx.cpu().numpy().astype(np.uint32), ri)
    ref = oracle.compute_features(xyz, ri.reshape(-1), np.arange(0, k * 5001, k, dtype=np.uint32))
    assert feature_close(out.cpu().numpy(), ref).all()
    # argument errors come back as status codes before any device work
    assert lib.pgeof_knn_search_f32(t.data_ptr(), 5, t.data_ptr(), 5, 6, idx.data_ptr(), d2.data_ptr(), s) == 1


def test_kernels_actually_launch(cuda, pgeof):
    before = pgeof.kernel_launch_count()
    xyz = uniform_cube(1000, seed=1)
    pgeof.knn_search(xyz, xyz, 8)
    assert pgeof.kernel_launch_count() > before


def test_result_arrays_reuse_cached_host_blocks(cuda, pgeof):
    """Numpy results live in cached page-locked blocks: values are unaffected
    by reuse, a block is only recycled after its array is freed, and trimming
    the cache leaves live arrays intact."""
    xyz = uniform_cube(20_000, seed=9)
    i1, d1 = pgeof.knn_search(xyz, xyz, 16)
    keep_i, keep_d = i1.copy(), d1.copy()
    i2, d2 = pgeof.knn_search(xyz, xyz, 16)  # i1/d1 still alive: different blocks
    assert i1.ctypes.data != i2.ctypes.data
    np.testing.assert_array_equal(i2, keep_i)
    del i2, d2
    pgeof.pgeof_ext._host_pool_trim()  # releases the freed blocks only
    np.testing.assert_array_equal(i1, keep_i)
    np.testing.assert_array_equal(d1, keep_d)
    for _ in range(3):
        i3, d3 = pgeof.knn_search(xyz, xyz, 16)
        np.testing.assert_array_equal(i3, keep_i)
        np.testing.assert_array_equal(d3, keep_d)
    ptr = (np.arange(xyz.shape[0] + 1) * 16).astype(np.uint32)
    f = pgeof.compute_features(xyz, i1.reshape(-1), ptr)
    assert f.flags.c_contiguous and f.flags.writeable and f.shape == (20_000, 11)
    f[:] = 0  # writable like a fresh numpy array
