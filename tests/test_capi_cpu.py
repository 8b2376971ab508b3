"""The C ABI library and the drop-in module on a machine without a GPU:
the library loads and exports every entry point declared in
include/pgeof_cuda.h, and argument checks that precede any device work behave
like the reference (ValueError / TypeError)."""

import ctypes
import os
import re

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "pgeof_cuda.h")


def declared_functions():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(pgeof_[a-z0-9_]+)\s*\(", text)))


def test_header_declares_the_reference_surface():
    names = declared_functions()
    for want in ("knn_search_f32", "radius_search_f32", "compute_features_f32", "compute_features_multiscale_f32",
                 "compute_features_optimal_f32", "compute_features_selected_f32", "compute_features_selected_f64"):
        assert "pgeof_" + want in names
        assert "pgeof_host_" + want in names


def test_library_exports_every_declared_symbol(pgeof):
    lib = ctypes.CDLL(pgeof.LIBRARY_PATH)
    missing = [n for n in declared_functions() if not hasattr(lib, n)]
    assert not missing, missing
    lib.pgeof_status_string.restype = ctypes.c_char_p
    assert lib.pgeof_status_string(1) == b"invalid argument"
    assert lib.pgeof_abi_version() == 1


def test_enum_values_match_reference(pgeof):
    """include/pca.hpp:47-63."""
    names = ["Linearity", "Planarity", "Scattering", "VerticalityPGEOF", "Normal_x", "Normal_y", "Normal_z",
             "Length", "Surface", "Volume", "Curvature", "K_optimal", "Verticality", "Eigentropy"]
    for i, n in enumerate(names):
        assert int(getattr(pgeof.EFeatureID, n)) == i
        assert int(getattr(pgeof, n)) == i


def test_argument_errors_without_device(pgeof):
    xyz = np.random.default_rng(0).random((20, 3), dtype=np.float32)
    nn = np.arange(20, dtype=np.uint32)
    ptr = np.array([0, 10, 20], np.uint32)
    with pytest.raises(ValueError, match="knn size is greater"):
        pgeof.knn_search(xyz, xyz, 21)
    with pytest.raises(ValueError, match="max knn size is greater"):
        pgeof.radius_search(xyz, xyz, 0.1, 21)
    with pytest.raises(ValueError, match="k_min should be"):
        pgeof.compute_features(xyz, nn, ptr, 0)
    with pytest.raises(ValueError, match="k_scales"):
        pgeof.compute_features_multiscale(xyz, nn, ptr, [10, 5])
    with pytest.raises(ValueError, match="k_scales"):
        pgeof.compute_features_multiscale(xyz, nn, ptr, [0, 5])
    with pytest.raises(ValueError, match="k_min and k_min_search"):
        pgeof.compute_features_optimal(xyz, nn, ptr, 0, 1, 0)
    with pytest.raises(ValueError, match="k_step"):
        pgeof.compute_features_optimal(xyz, nn, ptr, 1, 0, 1)
    # noconvert dtype strictness (src/pgeof_ext.cpp:34-35)
    with pytest.raises(TypeError):
        pgeof.compute_features(xyz.astype(np.float64), nn, ptr)
    with pytest.raises(TypeError):
        pgeof.compute_features(xyz, nn.astype(np.int32), ptr)
    with pytest.raises(TypeError):
        pgeof.knn_search(xyz[:, :2].copy(), xyz, 2)
    with pytest.raises(TypeError):
        pgeof.compute_features_selected(xyz.astype(np.int32), 0.1, 5, [pgeof.Verticality])


def test_eig_order_switch(pgeof):
    assert pgeof.get_eig_order() == "ascending"
    pgeof.set_eig_order("descending")
    assert pgeof.get_eig_order() == "descending"
    pgeof.set_eig_order("ascending")
    with pytest.raises(KeyError):
        pgeof.set_eig_order("sideways")


def test_index_handle_argument_checks_without_device(pgeof):
    """pgeof_index_*: argument errors come back before any device work."""
    lib = ctypes.CDLL(pgeof.LIBRARY_PATH)
    h = ctypes.c_void_p(0)
    xyz = np.zeros((4, 3), np.float32)
    ptr = xyz.ctypes.data_as(ctypes.c_void_p)
    assert lib.pgeof_index_create_f32(ptr, ctypes.c_int64(0), 16, ctypes.c_float(0.0), None, ctypes.byref(h)) == 1
    assert h.value is None
    assert lib.pgeof_index_create_f32(ptr, ctypes.c_int64(4), 16, ctypes.c_float(-1.0), None, ctypes.byref(h)) == 1
    assert lib.pgeof_index_create_f32(None, ctypes.c_int64(4), 16, ctypes.c_float(0.0), None, ctypes.byref(h)) == 1
    assert lib.pgeof_index_create_f32(ptr, ctypes.c_int64(4), 16, ctypes.c_float(0.0), None, None) == 1
    n = ctypes.c_int64(-1)
    assert lib.pgeof_index_size(None, ctypes.byref(n)) == 1
    assert lib.pgeof_index_knn_search_f32(None, None, ctypes.c_int64(0), 3, None, None, None) == 1
    assert lib.pgeof_index_radius_search_f32(None, None, ctypes.c_int64(0), ctypes.c_float(0.1), 3, None, None,
                                             None) == 1
    assert lib.pgeof_index_knn_features_f32(None, 3, None, ctypes.c_int64(0), None, None) == 1
    assert lib.pgeof_index_destroy(None) == 0
    lib.pgeof_last_error_message.restype = ctypes.c_char_p
    assert b"invalid index" in lib.pgeof_last_error_message()


def test_f64_feature_argument_errors_without_device(pgeof):
    xyz = np.random.default_rng(0).random((20, 3))
    nn = np.arange(20, dtype=np.uint32)
    ptr = np.array([0, 10, 20], np.uint32)
    with pytest.raises(ValueError, match="k_min should be"):
        pgeof.compute_features_f64(xyz, nn, ptr, 0)
    with pytest.raises(ValueError, match="k_scales"):
        pgeof.compute_features_multiscale_f64(xyz, nn, ptr, [10, 5])
    with pytest.raises(ValueError, match="k_min and k_min_search"):
        pgeof.compute_features_optimal_f64(xyz, nn, ptr, 0, 1, 0)
    with pytest.raises(ValueError, match="k_step"):
        pgeof.compute_features_optimal_f64(xyz, nn, ptr, 1, 0, 1)
    with pytest.raises(TypeError):  # noconvert: float32 xyz is not cast
        pgeof.compute_features_f64(xyz.astype(np.float32), nn, ptr)
    with pytest.raises(TypeError):
        pgeof.compute_features(xyz, nn, ptr)  # the reference's float32-only entry point stays strict


def test_server_handle_argument_checks_without_device(pgeof):
    """pgeof_server_*: argument errors come back before any thread or device work."""
    lib = ctypes.CDLL(pgeof.LIBRARY_PATH)
    h = ctypes.c_void_p(0)
    assert lib.pgeof_server_create(0, ctypes.c_uint64(1 << 30), ctypes.byref(h)) == 1
    assert lib.pgeof_server_create(4, ctypes.c_uint64(0), ctypes.byref(h)) == 1
    assert lib.pgeof_server_create(4, ctypes.c_uint64(1 << 30), None) == 1
    rid = ctypes.c_uint64(0)
    assert lib.pgeof_server_submit_selected_f32(None, None, ctypes.c_int64(0), ctypes.c_float(1.0), 4, None,
                                                ctypes.c_int64(0), None, ctypes.byref(rid)) == 1
    assert lib.pgeof_server_wait(None, ctypes.c_uint64(1), None, None, None) == 1
    assert lib.pgeof_server_stats(None, None, None, None) == 1
    cid = ctypes.c_uint64(0)
    assert lib.pgeof_server_add_cloud_f32(None, None, ctypes.c_int64(10), ctypes.c_float(1.0), 16,
                                          ctypes.byref(cid)) == 1
    assert lib.pgeof_server_remove_cloud(None, ctypes.c_uint64(1)) == 1
    assert lib.pgeof_server_submit_selected_resident_f32(None, ctypes.c_uint64(1), ctypes.c_float(1.0), 16, None,
                                                         ctypes.c_int64(0), None, ctypes.byref(rid)) == 1
    assert lib.pgeof_server_destroy(None) == 0
