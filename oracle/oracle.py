"""Python face of the oracle -- TEST INFRASTRUCTURE ONLY.

Only ``tests/``, ``__graft_entry__.smoke()`` and ``bench.py``'s CPU-baseline
leg use this module, and only as the checker / the timed CPU baseline. The
shipped library never imports it.

Two restatements of pgeof 0.3.3 live here:

* ``libpgeof_oracle.so`` (``pgeof_oracle.c``): the FP32-literal restatement of
  ``include/pca.hpp`` / ``include/pgeof.hpp`` / ``include/nn_search.hpp``
  (see the C file's header for the exact arithmetic), threaded with pthreads.
* ``fp64_*`` functions below: an independent numpy FP64 restatement (gather,
  two-pass covariance, ``numpy.linalg.eigh`` -- ascending like Eigen --
  features), the "FP64 oracle" that per-feature errors are reported against.

Parity status: neighbour search is pinned by the reference's own tests
(``tests/test_pgeof.py:8-27``, scipy KDTree); feature values are
"parity unpinned" against a reference binary (none can be built here) and are
pinned by hand-derived known answers plus the FP64 restatement.
"""

from __future__ import annotations

import ctypes
import os
import subprocess
import threading

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_BUILD_DIR = os.path.join(_HERE, "_build")
_LIB_PATH = os.path.join(_BUILD_DIR, "libpgeof_oracle.so")
_SOURCES = [os.path.join(_HERE, "pgeof_oracle.c"), os.path.join(_HERE, "pca_body.h")]

EIG_ASCENDING = 0
EIG_DESCENDING = 1

_lock = threading.Lock()
_lib = None


def build(force: bool = False) -> str:
    """Compile ``libpgeof_oracle.so`` (gcc, no FMA contraction, pthreads)."""
    os.makedirs(_BUILD_DIR, exist_ok=True)
    stale = force or not os.path.exists(_LIB_PATH) or any(
        os.path.getmtime(s) > os.path.getmtime(_LIB_PATH) for s in _SOURCES
    )
    if stale:
        tmp = _LIB_PATH + f".tmp{os.getpid()}"
        cmd = [
            "gcc", "-O2", "-std=c11", "-fPIC", "-shared", "-ffp-contract=off", "-fno-fast-math",
            "-pthread", "-o", tmp, _SOURCES[0], "-lm",
        ]
        subprocess.check_call(cmd, cwd=_HERE)
        os.replace(tmp, _LIB_PATH)
    return _LIB_PATH


def _load():
    global _lib
    with _lock:
        if _lib is None:
            build()
            lib = ctypes.CDLL(_LIB_PATH)
            P = ctypes.c_void_p
            S = ctypes.c_size_t
            U = ctypes.c_uint32
            I = ctypes.c_int
            lib.oracle_compute_features.argtypes = [P, P, P, S, S, I, I, P]
            lib.oracle_compute_features_multiscale.argtypes = [P, P, P, S, P, S, I, I, P]
            lib.oracle_compute_features_optimal.argtypes = [P, P, P, S, U, U, U, I, I, P]
            lib.oracle_knn_search.argtypes = [P, S, P, S, U, I, P, P]
            lib.oracle_radius_search.argtypes = [P, S, P, S, ctypes.c_float, U, I, P, P]
            lib.oracle_selected_f32.argtypes = [P, S, ctypes.c_float, U, P, S, I, I, P]
            lib.oracle_selected_f64.argtypes = [P, S, ctypes.c_double, U, P, S, I, I, P]
            lib.oracle_compute_features_f64.argtypes = [I, P, P, P, S, S, P, S, U, U, I, I, P]
            lib.oracle_pca_features_f32.argtypes = [P, S, I, P]
            lib.oracle_pca_features_f32.restype = None
            lib.oracle_covariance_f32.argtypes = [P, S, P]
            lib.oracle_covariance_f32.restype = None
            lib.oracle_num_threads.restype = I
            for f in (
                lib.oracle_compute_features, lib.oracle_compute_features_multiscale,
                lib.oracle_compute_features_optimal, lib.oracle_knn_search, lib.oracle_radius_search,
                lib.oracle_selected_f32, lib.oracle_selected_f64, lib.oracle_compute_features_f64,
            ):
                f.restype = I
            _lib = lib
    return _lib


def _ptr(a: np.ndarray):
    return a.ctypes.data_as(ctypes.c_void_p)


def _c(a, dtype):
    return np.ascontiguousarray(a, dtype=dtype)


def num_threads() -> int:
    return int(_load().oracle_num_threads())


# ----------------------------------------------------------------------------
# FP32-literal restatement (C)
# ----------------------------------------------------------------------------
def compute_features(xyz, nn, nn_ptr, k_min=1, order=EIG_ASCENDING, threads=0):
    """include/pgeof.hpp:75-117."""
    lib = _load()
    xyz, nn, nn_ptr = _c(xyz, np.float32), _c(nn, np.uint32), _c(nn_ptr, np.uint32)
    n = nn_ptr.size - 1
    out = np.zeros((n, 11), np.float32)
    if lib.oracle_compute_features(_ptr(xyz), _ptr(nn), _ptr(nn_ptr), n, int(k_min), order, threads, _ptr(out)):
        raise ValueError("k_min should be > 1")
    return out


def compute_features_multiscale(xyz, nn, nn_ptr, k_scales, order=EIG_ASCENDING, threads=0):
    """include/pgeof.hpp:123-211."""
    lib = _load()
    xyz, nn, nn_ptr = _c(xyz, np.float32), _c(nn, np.uint32), _c(nn_ptr, np.uint32)
    scales = _c(np.asarray(k_scales), np.uint32)
    n = nn_ptr.size - 1
    out = np.zeros((n, scales.size, 11), np.float32)
    if lib.oracle_compute_features_multiscale(
        _ptr(xyz), _ptr(nn), _ptr(nn_ptr), n, _ptr(scales), scales.size, order, threads, _ptr(out)
    ):
        raise ValueError("k_scales should be > 1 and sorted in ascending order")
    return out


def compute_features_optimal(xyz, nn, nn_ptr, k_min=1, k_step=1, k_min_search=1, order=EIG_ASCENDING, threads=0):
    """include/pgeof.hpp:243-310."""
    lib = _load()
    xyz, nn, nn_ptr = _c(xyz, np.float32), _c(nn, np.uint32), _c(nn_ptr, np.uint32)
    n = nn_ptr.size - 1
    out = np.zeros((n, 12), np.float32)
    if lib.oracle_compute_features_optimal(
        _ptr(xyz), _ptr(nn), _ptr(nn_ptr), n, int(k_min), int(k_step), int(k_min_search), order, threads, _ptr(out)
    ):
        raise ValueError("k_min and k_min_search should be > 1 (and k_step >= 1)")
    return out


def compute_features_f64(xyz, nn, nn_ptr, k_min=1, kind="full", k_scales=(), k_step=1, k_min_search=1,
                         order=EIG_ASCENDING, threads=0):
    """include/pgeof.hpp:75-117 / 123-211 / 243-310 (kind "full" / "multi" /
    "optimal") with real_t = double: the same drivers and PCA in double."""
    lib = _load()
    xyz, nn, nn_ptr = _c(xyz, np.float64), _c(nn, np.uint32), _c(nn_ptr, np.uint32)
    scales = _c(np.asarray(k_scales if kind == "multi" else [1]), np.uint32)
    n = nn_ptr.size - 1
    code = {"full": 0, "multi": 1, "optimal": 2}[kind]
    shape = {"full": (n, 11), "multi": (n, scales.size, 11), "optimal": (n, 12)}[kind]
    out = np.zeros(shape, np.float64)
    if lib.oracle_compute_features_f64(code, _ptr(xyz), _ptr(nn), _ptr(nn_ptr), n, int(k_min), _ptr(scales),
                                       scales.size if kind == "multi" else 0, int(k_step), int(k_min_search), order,
                                       threads, _ptr(out)):
        raise ValueError("invalid k_min / k_scales / k_step")
    return out


def knn_search(data, query, k, threads=0):
    """include/nn_search.hpp:31-67 (brute force, (distance, index) order)."""
    lib = _load()
    data, query = _c(data, np.float32), _c(query, np.float32)
    m = query.shape[0]
    idx = np.zeros((m, k), np.uint32)
    d2 = np.zeros((m, k), np.float32)
    if lib.oracle_knn_search(_ptr(data), data.shape[0], _ptr(query), m, int(k), threads, _ptr(idx), _ptr(d2)):
        raise ValueError("knn size is greater than the data point cloud size")
    return idx, d2


def radius_search(data, query, radius, max_knn, threads=0):
    """include/nn_search.hpp:85-132 (brute force, (distance, index) order)."""
    lib = _load()
    data, query = _c(data, np.float32), _c(query, np.float32)
    m = query.shape[0]
    idx = np.zeros((m, max_knn), np.int32)
    d2 = np.zeros((m, max_knn), np.float32)
    if lib.oracle_radius_search(
        _ptr(data), data.shape[0], _ptr(query), m, float(radius), int(max_knn), threads, _ptr(idx), _ptr(d2)
    ):
        raise ValueError("max knn size is greater than the data point cloud size")
    return idx, d2


def compute_features_selected(xyz, radius, max_knn, ids, order=EIG_ASCENDING, threads=0):
    """include/pgeof.hpp:325-375, float or double by xyz dtype."""
    lib = _load()
    ids = _c([int(i) for i in ids], np.int32)
    if np.asarray(xyz).dtype == np.float64:
        xyz = _c(xyz, np.float64)
        out = np.zeros((xyz.shape[0], ids.size), np.float64)
        lib.oracle_selected_f64(_ptr(xyz), xyz.shape[0], float(radius), int(max_knn), _ptr(ids), ids.size,
                                order, threads, _ptr(out))
    else:
        xyz = _c(xyz, np.float32)
        out = np.zeros((xyz.shape[0], ids.size), np.float32)
        lib.oracle_selected_f32(_ptr(xyz), xyz.shape[0], float(radius), int(max_knn), _ptr(ids), ids.size,
                                order, threads, _ptr(out))
    return out


def pca_features(points, order=EIG_ASCENDING):
    """One neighbourhood: returns dict(val, v0, v1, v2, features[11], eigentropy)."""
    lib = _load()
    pts = _c(points, np.float32).reshape(-1, 3)
    out = np.zeros(24, np.float32)
    lib.oracle_pca_features_f32(_ptr(pts), pts.shape[0], order, _ptr(out))
    return {
        "val": out[0:3].copy(), "v0": out[3:6].copy(), "v1": out[6:9].copy(), "v2": out[9:12].copy(),
        "features": out[12:23].copy(), "eigentropy": float(out[23]),
    }


def covariance(points):
    """The float covariance (xx, xy, xz, yy, yz, zz) formed as the reference forms it."""
    lib = _load()
    pts = _c(points, np.float32).reshape(-1, 3)
    out = np.zeros(6, np.float32)
    lib.oracle_covariance_f32(_ptr(pts), pts.shape[0], _ptr(out))
    return out


# ----------------------------------------------------------------------------
# FP64 numpy restatement (independent of the C code)
# ----------------------------------------------------------------------------
def fp64_eig(points_batch: np.ndarray, order=EIG_ASCENDING):
    """points_batch (m, k, 3) -> (val (m,3), vec (m,3,3) columns, cov (m,3,3)), all float64.

    Same steps as include/pca.hpp:72-98 in double: mean-centre, C^T C / k,
    ascending eigen-decomposition, clamp >= 0, flip v2 to z >= 0.
    """
    P = np.asarray(points_batch, dtype=np.float64)
    C = P - P.mean(axis=1, keepdims=True)
    cov = np.einsum("mki,mkj->mij", C, C) / P.shape[1]
    w, V = np.linalg.eigh(cov)
    if order == EIG_DESCENDING:
        w = w[:, ::-1]
        V = V[:, :, ::-1]
    w = np.maximum(w, 0.0)
    flip = V[:, 2, 2] < 0
    V[flip, :, 2] *= -1.0
    return w, V, cov


def fp64_features_from_eig(w: np.ndarray, V: np.ndarray) -> np.ndarray:
    """include/pca.hpp:160-200 in float64, for (m,3) eigenvalues and (m,3,3) column eigenvectors."""
    eps = 1e-3
    s = np.sqrt(w)
    v0, v1, v2 = s[:, 0], s[:, 1], s[:, 2]
    fact = 1.0 / (v0 + eps)
    f = np.zeros((w.shape[0], 11))
    f[:, 0] = (v0 - v1) * fact
    f[:, 1] = (v1 - v2) * fact
    f[:, 2] = v2 * fact
    u = (w[:, None, :] * np.abs(V)).sum(axis=2)  # u_j = sum_i val_i |v_i[j]|
    nrm = np.linalg.norm(u, axis=1)
    with np.errstate(invalid="ignore", divide="ignore"):
        vert = np.where(v0 > 0, u[:, 2] / nrm, 0.0)
    f[:, 3] = vert
    f[:, 4:7] = V[:, :, 2]
    f[:, 7] = v0
    f[:, 8] = np.sqrt(v0 * v1 + 1e-6)
    f[:, 9] = np.power(v0 * v1 * v2 + 1e-9, 1.0 / 3.0)
    f[:, 10] = v2 / (v0 + v1 + v2 + eps)
    return f


def fp64_eigentropy(w: np.ndarray) -> np.ndarray:
    eps = 1e-3
    e = w / (w.sum(axis=1, keepdims=True) + eps)
    return -(e * np.log(e + eps)).sum(axis=1)


def fp64_compute_features(xyz, nn, nn_ptr, k_min=1, order=EIG_ASCENDING):
    """FP64 version of include/pgeof.hpp:75-117 (groups equal-size neighbourhoods)."""
    xyz = np.asarray(xyz, dtype=np.float64)
    nn = np.asarray(nn, dtype=np.int64)
    nn_ptr = np.asarray(nn_ptr, dtype=np.int64)
    n = nn_ptr.size - 1
    out = np.zeros((n, 11))
    sizes = np.diff(nn_ptr)
    for k in np.unique(sizes):
        if k < max(k_min, 1):
            continue
        rows = np.nonzero(sizes == k)[0]
        gather = nn[nn_ptr[rows][:, None] + np.arange(k)[None, :]]
        w, V, _ = fp64_eig(xyz[gather], order)
        out[rows] = fp64_features_from_eig(w, V)
    return out


def fp64_relative_gap(points_batch: np.ndarray) -> np.ndarray:
    """min eigen-gap / largest eigenvalue of each neighbourhood (conditioning of the eigenvectors)."""
    P = np.asarray(points_batch, dtype=np.float64)
    C = P - P.mean(axis=1, keepdims=True)
    cov = np.einsum("mki,mkj->mij", C, C) / P.shape[1]
    w = np.linalg.eigvalsh(cov)
    gap = np.minimum(w[:, 1] - w[:, 0], w[:, 2] - w[:, 1])
    return gap / np.maximum(w[:, 2], 1e-300)
