"""GB300 (sm_103a) implementation of pgeof's neighbour search and local-PCA
geometric features, with pgeof's Python API.

Drop-in for ``pgeof`` (src/pgeof/__init__.py:1-9): the same names, argument
names, defaults and numpy dtype rules. Every call runs on the GPU through
``libpgeof_cuda.so``; there is no CPU fallback -- if the native library is
missing, importing this package raises ImportError.

Besides numpy arrays, every function also accepts ``torch.cuda`` tensors: the
work then stays on the device (inputs are read in place, outputs are CUDA
tensors, the call is enqueued on the current torch stream).
"""

from __future__ import annotations

import os as _os
import sys as _sys

try:
    from . import pgeof_ext as _ext
except ImportError as _e:  # no CPU fallback: fail loudly
    raise ImportError(
        "point_geometric_features_gb300: the native library is not built "
        f"({_e}). Build it with `python point_geometric_features_gb300/_build.py` "
        "(needs nvcc for sm_103a)."
    ) from _e

from .pgeof_ext import EFeatureID  # noqa: E402

# enum values exported at module level like pgeof_ext's export_values()
for _name, _val in EFeatureID.__members__.items():
    globals()[_name] = _val

LIBRARY_PATH = _os.path.join(_os.path.dirname(_os.path.abspath(__file__)), "libpgeof_cuda.so")

__all__ = [
    "EFeatureID",
    "compute_features",
    "compute_features_multiscale",
    "compute_features_optimal",
    "compute_features_f64",
    "compute_features_multiscale_f64",
    "compute_features_optimal_f64",
    "knn_search",
    "radius_search",
    "radius_search_csr",
    "knn_features",
    "compute_features_selected",
    "set_eig_order",
    "get_eig_order",
    "kernel_launch_count",
    "check_device_errors",
    "batch_knn_features",
    "BatchPlan",
    "GridIndex",
]


def _is_torch(x) -> bool:
    return type(x).__module__.startswith("torch") and hasattr(x, "is_cuda")


def set_eig_order(order: str) -> None:
    """Eigenpair order fed to the feature formulas.

    ``"ascending"`` (default) is what pgeof 0.3.3 does: include/pca.hpp:79-97
    uses Eigen's eigenvalues unsorted, i.e. ascending. ``"descending"`` puts the
    largest eigenvalue first, which makes Normal_x/y/z the surface normal.
    """
    _ext._set_eig_order({"ascending": 0, "descending": 1}[order])


def get_eig_order() -> str:
    return ("ascending", "descending")[_ext._get_eig_order()]


def kernel_launch_count() -> int:
    """Number of CUDA kernels libpgeof_cuda has launched in this process."""
    return int(_ext._launch_count())


def profile_kernels(enabled: bool) -> None:
    """Bracket every kernel launch with CUDA events on its own stream."""
    _ext._profile_enable(bool(enabled))


def kernel_profile() -> dict:
    """{kernel name: (launches, total ms)} since the last call (waits for the events)."""
    out = {}
    for line in _ext._profile_report().splitlines():
        name, n, ms = line.split()
        out[name] = (int(n), float(ms))
    return out


def check_device_errors(stream=None) -> None:
    """Synchronise ``stream`` (torch stream, int handle or None = current torch
    stream) and raise ValueError if a device call saw invalid CSR input."""
    bits = _ext._take_device_errors(_stream_handle(stream))
    if bits & 1:
        raise ValueError("nn holds an index >= the number of points in xyz")
    if bits & 2:
        raise ValueError("nn_ptr must be non-decreasing and its values must not exceed len(nn)")
    if bits & 4:
        raise RuntimeError("neighbour selection exceeded its refinement bound")


def _stream_handle(stream=None) -> int:
    if isinstance(stream, int):
        return stream
    torch = _sys.modules.get("torch")
    if stream is None:
        if torch is None or not torch.cuda.is_available():
            return 0
        return int(torch.cuda.current_stream().cuda_stream)
    return int(stream.cuda_stream)


# --------------------------------------------------------------- device path
def _dev_cloud(t, name, dtype_name="float32"):
    torch = _sys.modules["torch"]
    want = getattr(torch, dtype_name)
    if not t.is_cuda or t.dtype != want or t.dim() != 2 or t.shape[1] != 3 or not t.is_contiguous():
        raise TypeError(f"{name} must be a contiguous CUDA {dtype_name} tensor of shape (n, 3)")
    return t


def _dev_index(t, name):
    torch = _sys.modules["torch"]
    ok_dtypes = (torch.int32,) + ((torch.uint32,) if hasattr(torch, "uint32") else ())
    if not t.is_cuda or t.dtype not in ok_dtypes or t.dim() != 1 or not t.is_contiguous():
        raise TypeError(f"{name} must be a contiguous 1-D CUDA uint32 (or int32) tensor")
    return t


def _uint32_empty(torch, shape, device):
    if hasattr(torch, "uint32"):
        return torch.empty(shape, dtype=torch.uint32, device=device)
    return torch.empty(shape, dtype=torch.int32, device=device)


def _to_host(t, as_uint32=False):
    """A CUDA tensor as a numpy array in page-locked memory from torch's cached
    host allocator: the download runs at DMA speed instead of page-faulting a
    fresh pageable array (the numpy array keeps the block alive)."""
    torch = _sys.modules["torch"]
    if as_uint32 or t.dtype not in (torch.float32, torch.float64, torch.int32, torch.int64):
        t = t.view(torch.int32)
    h = torch.empty(t.shape, dtype=t.dtype, pin_memory=True)
    h.copy_(t)
    a = h.numpy()
    return a.view("uint32") if as_uint32 else a


def _finish(check, stream):
    if check:
        check_device_errors(stream)


def _dev_features(kind, xyz, nn, nn_ptr, args, check):
    torch = _sys.modules["torch"]
    if xyz.dtype == torch.float64:
        return _dev_features_f64(kind, xyz, nn, nn_ptr, args, check)
    _dev_cloud(xyz, "xyz")
    _dev_index(nn, "nn")
    _dev_index(nn_ptr, "nn_ptr")
    n = nn_ptr.shape[0] - 1
    with torch.cuda.device(xyz.device):
        s = int(torch.cuda.current_stream().cuda_stream)
        if kind == "full":
            out = torch.empty((max(n, 0), 11), dtype=torch.float32, device=xyz.device)
            _ext._dev_compute_features(xyz.data_ptr(), xyz.shape[0], nn.data_ptr(), nn.shape[0], nn_ptr.data_ptr(),
                                       n, int(args[0]), out.data_ptr(), s)
        elif kind == "multi":
            scales = [int(v) for v in args[0]]
            out = torch.empty((max(n, 0), len(scales), 11), dtype=torch.float32, device=xyz.device)
            _ext._dev_compute_features_multiscale(xyz.data_ptr(), xyz.shape[0], nn.data_ptr(), nn.shape[0],
                                                  nn_ptr.data_ptr(), n, scales, out.data_ptr(), s)
        else:
            out = torch.empty((max(n, 0), 12), dtype=torch.float32, device=xyz.device)
            _ext._dev_compute_features_optimal(xyz.data_ptr(), xyz.shape[0], nn.data_ptr(), nn.shape[0],
                                               nn_ptr.data_ptr(), n, int(args[0]), int(args[1]), int(args[2]),
                                               out.data_ptr(), s)
        _finish(check, s)
    return out


def _dev_features_f64(kind, xyz, nn, nn_ptr, args, check):
    torch = _sys.modules["torch"]
    _dev_cloud(xyz, "xyz", "float64")
    _dev_index(nn, "nn")
    _dev_index(nn_ptr, "nn_ptr")
    n = max(nn_ptr.shape[0] - 1, 0)
    code = {"full": 0, "multi": 1, "optimal": 2}[kind]
    scales = [int(v) for v in args[0]] if kind == "multi" else []
    k_min = int(args[0]) if kind != "multi" else 1
    k_step, k_min_search = (int(args[1]), int(args[2])) if kind == "optimal" else (1, 1)
    shape = {"full": (n, 11), "multi": (n, len(scales), 11), "optimal": (n, 12)}[kind]
    with torch.cuda.device(xyz.device):
        s = int(torch.cuda.current_stream().cuda_stream)
        out = torch.zeros(shape, dtype=torch.float64, device=xyz.device)
        _ext._dev_compute_features_f64(code, xyz.data_ptr(), xyz.shape[0], nn.data_ptr(), nn.shape[0],
                                       nn_ptr.data_ptr(), nn_ptr.shape[0] - 1, k_min, scales, k_step, k_min_search,
                                       out.data_ptr(), s)
        _finish(check, s)
    return out


# --------------------------------------------------------------- public API
def compute_features(xyz, nn, nn_ptr, k_min=1, verbose=False, *, check=True):
    """include/pgeof.hpp:75-117 -- (n_points, 11) float32 features from CSR neighbours."""
    if _is_torch(xyz):
        return _dev_features("full", xyz, nn, nn_ptr, (k_min,), check)
    return _ext.compute_features(xyz, nn, nn_ptr, k_min, verbose)


def compute_features_multiscale(xyz, nn, nn_ptr, k_scales, verbose=False, *, check=True):
    """include/pgeof.hpp:123-211 -- (n_points, n_scales, 11) float32 features."""
    if _is_torch(xyz):
        return _dev_features("multi", xyz, nn, nn_ptr, (k_scales,), check)
    return _ext.compute_features_multiscale(xyz, nn, nn_ptr, k_scales, verbose)


def compute_features_optimal(xyz, nn, nn_ptr, k_min=1, k_step=1, k_min_search=1, verbose=False, *, check=True):
    """include/pgeof.hpp:243-310 -- (n_points, 12) float32, column 11 = optimal k."""
    if _is_torch(xyz):
        return _dev_features("optimal", xyz, nn, nn_ptr, (k_min, k_step, k_min_search), check)
    return _ext.compute_features_optimal(xyz, nn, nn_ptr, k_min, k_step, k_min_search, verbose)


def compute_features_f64(xyz, nn, nn_ptr, k_min=1, verbose=False, *, check=True):
    """compute_features for a float64 cloud (include/pgeof.hpp:75-117 with
    real_t = double, which pgeof's binding does not instantiate): (n_points, 11)
    float64. numpy arrays or CUDA tensors, as compute_features."""
    if _is_torch(xyz):
        return _dev_features_f64("full", xyz, nn, nn_ptr, (k_min,), check)
    return _ext.compute_features_f64(xyz, nn, nn_ptr, k_min, verbose)


def compute_features_multiscale_f64(xyz, nn, nn_ptr, k_scales, verbose=False, *, check=True):
    """compute_features_multiscale for a float64 cloud (include/pgeof.hpp:123-211
    with real_t = double): (n_points, n_scales, 11) float64."""
    if _is_torch(xyz):
        return _dev_features_f64("multi", xyz, nn, nn_ptr, (k_scales,), check)
    return _ext.compute_features_multiscale_f64(xyz, nn, nn_ptr, k_scales, verbose)


def compute_features_optimal_f64(xyz, nn, nn_ptr, k_min=1, k_step=1, k_min_search=1, verbose=False, *, check=True):
    """compute_features_optimal for a float64 cloud (include/pgeof.hpp:243-310
    with real_t = double): (n_points, 12) float64, column 11 = optimal k."""
    if _is_torch(xyz):
        return _dev_features_f64("optimal", xyz, nn, nn_ptr, (k_min, k_step, k_min_search), check)
    return _ext.compute_features_optimal_f64(xyz, nn, nn_ptr, k_min, k_step, k_min_search, verbose)


def knn_search(data, query, knn):
    """include/nn_search.hpp:31-67 -- (uint32 indices, float32 squared distances), (n_query, knn)."""
    if _is_torch(data):
        torch = _sys.modules["torch"]
        _dev_cloud(data, "data")
        _dev_cloud(query, "query")
        with torch.cuda.device(data.device):
            s = int(torch.cuda.current_stream().cuda_stream)
            idx = _uint32_empty(torch, (query.shape[0], int(knn)), data.device)
            d2 = torch.empty((query.shape[0], int(knn)), dtype=torch.float32, device=data.device)
            _ext._dev_knn_search(data.data_ptr(), data.shape[0], query.data_ptr(), query.shape[0], int(knn),
                                 idx.data_ptr(), d2.data_ptr(), s)
        return idx, d2
    return _ext.knn_search(data, query, knn)


def radius_search(data, query, search_radius, max_knn):
    """include/nn_search.hpp:85-132 -- (int32 indices, -1 = none; float32 squared distances)."""
    if _is_torch(data):
        torch = _sys.modules["torch"]
        _dev_cloud(data, "data")
        _dev_cloud(query, "query")
        with torch.cuda.device(data.device):
            s = int(torch.cuda.current_stream().cuda_stream)
            idx = torch.empty((query.shape[0], int(max_knn)), dtype=torch.int32, device=data.device)
            d2 = torch.empty((query.shape[0], int(max_knn)), dtype=torch.float32, device=data.device)
            _ext._dev_radius_search(data.data_ptr(), data.shape[0], query.data_ptr(), query.shape[0],
                                    float(search_radius), int(max_knn), idx.data_ptr(), d2.data_ptr(), s)
        return idx, d2
    return _ext.radius_search(data, query, search_radius, max_knn)


def radius_search_csr(data, query, search_radius, max_knn):
    """Radius search straight to the CSR pair that compute_features* take.

    Returns (nn, nn_ptr), both uint32: row i's neighbours are
    nn[nn_ptr[i]:nn_ptr[i + 1]], the non-padding entries of radius_search's row
    i in the same order -- what pgeof's README builds on the host from the
    padded table (README.md:157-163), done on the GPU. torch CUDA tensors stay
    on the device; numpy arrays go through it and come back as numpy.
    """
    import torch

    numpy_in = not _is_torch(data)
    if numpy_in:
        import numpy as np

        if not (isinstance(data, np.ndarray) and data.dtype == np.float32 and isinstance(query, np.ndarray)
                and query.dtype == np.float32):
            raise TypeError("radius_search_csr expects float32 numpy arrays or float32 CUDA tensors")
        data_t = torch.from_numpy(np.ascontiguousarray(data)).cuda()
        query_t = data_t if query is data else torch.from_numpy(np.ascontiguousarray(query)).cuda()
    else:
        data_t, query_t = data, query
    _dev_cloud(data_t, "data")
    _dev_cloud(query_t, "query")
    m, k = int(query_t.shape[0]), int(max_knn)
    with torch.cuda.device(data_t.device):
        s = int(torch.cuda.current_stream().cuda_stream)
        nn = _uint32_empty(torch, max(m * k, 1), data_t.device)
        nn_ptr = _uint32_empty(torch, m + 1, data_t.device)
        _ext._dev_radius_search_csr(data_t.data_ptr(), data_t.shape[0], query_t.data_ptr(), m,
                                    float(search_radius), k, nn.data_ptr(), nn_ptr.data_ptr(), s)
        nnz = int(nn_ptr[m:].view(torch.int32).item())
    nn = nn[:nnz]
    if numpy_in:
        return _to_host(nn, True), _to_host(nn_ptr, True)
    return nn, nn_ptr


def knn_features(xyz, k, k_scales=None):
    """kNN + local PCA features in one device pipeline, for callers that want
    only the features.

    Returns what compute_features(xyz, *knn_search(xyz, xyz, k) as CSR) returns
    -- (n, 11) -- or, with k_scales (ascending, each <= k),
    compute_features_multiscale over the same kNN lists -- (n, len(k_scales),
    11). The neighbour lists never leave the GPU and no distances are written.
    torch CUDA tensors stay on the device; numpy arrays go through it.
    """
    import torch

    numpy_in = not _is_torch(xyz)
    if numpy_in:
        import numpy as np

        if not (isinstance(xyz, np.ndarray) and xyz.dtype == np.float32):
            raise TypeError("knn_features expects a float32 numpy array or a float32 CUDA tensor")
        t = torch.from_numpy(np.ascontiguousarray(xyz)).cuda()
    else:
        t = xyz
    _dev_cloud(t, "xyz")
    scales = [int(v) for v in k_scales] if k_scales is not None else []
    n = int(t.shape[0])
    shape = (n, len(scales), 11) if scales else (n, 11)
    with torch.cuda.device(t.device):
        s = int(torch.cuda.current_stream().cuda_stream)
        out = torch.zeros(shape, dtype=torch.float32, device=t.device)
        _ext._dev_knn_features(t.data_ptr(), n, int(k), scales, out.data_ptr(), s)
    return _to_host(out) if numpy_in else out


def compute_features_selected(xyz, search_radius, max_knn, selected_features):
    """include/pgeof.hpp:325-375 -- (n, len(selected_features)) in xyz's precision."""
    if _is_torch(xyz):
        torch = _sys.modules["torch"]
        f64 = xyz.dtype == torch.float64
        _dev_cloud(xyz, "xyz", "float64" if f64 else "float32")
        ids = [int(v) for v in selected_features]
        with torch.cuda.device(xyz.device):
            s = int(torch.cuda.current_stream().cuda_stream)
            out = torch.empty((xyz.shape[0], len(ids)), dtype=xyz.dtype, device=xyz.device)
            _ext._dev_compute_features_selected(xyz.data_ptr(), xyz.shape[0], float(search_radius), int(max_knn),
                                                ids, f64, out.data_ptr(), s)
        return out
    return _ext.compute_features_selected(xyz, search_radius, max_knn, selected_features)


# --------------------------------------------------------------- multi-cloud batches
def _batch_inputs(clouds, offsets):
    torch = _sys.modules["torch"]
    if isinstance(clouds, (list, tuple)):
        offsets = [0]
        for c in clouds:
            _dev_cloud(c, "cloud")
            offsets.append(offsets[-1] + int(c.shape[0]))
        xyz = torch.cat(list(clouds), 0).contiguous()
    else:
        xyz = _dev_cloud(clouds, "xyz")
        offsets = [int(v) for v in offsets]
    return xyz, offsets


def batch_knn_features(clouds, k, offsets=None, features=True):
    """knn_search(cloud, cloud, k) and compute_features on its kNN CSR for many
    clouds in one device pipeline (no host round trip between kernels).

    ``clouds``: a list of contiguous CUDA float32 (n_i, 3) tensors, or one
    (N, 3) tensor with ``offsets`` (n_clouds + 1 row offsets). Returns
    ``(indices, sqr_dist, features)`` over all N rows: uint32 (N, k) indices
    local to each cloud, float32 (N, k) squared distances, float32 (N, 11)
    features (None when ``features`` is False) -- equal to the per-cloud calls.
    """
    torch = _sys.modules["torch"]
    xyz, offs = _batch_inputs(clouds, offsets)
    n = xyz.shape[0]
    with torch.cuda.device(xyz.device):
        s = int(torch.cuda.current_stream().cuda_stream)
        idx = _uint32_empty(torch, (n, int(k)), xyz.device)
        d2 = torch.empty((n, int(k)), dtype=torch.float32, device=xyz.device)
        f = torch.empty((n, 11), dtype=torch.float32, device=xyz.device) if features else None
        _ext._dev_batch_knn_features(xyz.data_ptr(), offs, int(k), idx.data_ptr(), d2.data_ptr(),
                                     f.data_ptr() if f is not None else 0, s)
    return idx, d2, f


class BatchPlan:
    """The batch pipeline captured once into a CUDA graph for a fixed batch
    shape: ``plan = BatchPlan(xyz, offsets, k)``; refill ``plan.xyz`` in place
    and call ``plan()``; results land in ``plan.indices``, ``plan.sqr_dist``,
    ``plan.features``. Creation tunes the grid cell size on the given data."""

    def __init__(self, clouds, k, offsets=None, features=True):
        torch = _sys.modules["torch"]
        self.xyz, self.offsets = _batch_inputs(clouds, offsets)
        n = self.xyz.shape[0]
        dev = self.xyz.device
        self.indices = _uint32_empty(torch, (n, int(k)), dev)
        self.sqr_dist = torch.empty((n, int(k)), dtype=torch.float32, device=dev)
        self.features = torch.empty((n, 11), dtype=torch.float32, device=dev) if features else None
        with torch.cuda.device(dev):
            s = int(torch.cuda.current_stream().cuda_stream)
            self._h = _ext._batch_plan_create(self.xyz.data_ptr(), self.offsets, int(k), self.indices.data_ptr(),
                                              self.sqr_dist.data_ptr(),
                                              self.features.data_ptr() if features else 0, s)

    def __call__(self, stream=None):
        _ext._batch_plan_launch(self._h, _stream_handle(stream))
        return self.indices, self.sqr_dist, self.features

    def info(self):
        """The speed parameters the plan runs with (chosen by the autotuner at
        creation, or reused from an earlier plan of the same shape class) and
        the pipeline times measured with them and with the defaults."""
        cell, chunk, tuned, dflt, cached = _ext._batch_plan_info(self._h)
        return {"cell_factor": round(float(cell), 3),
                "queries_per_work_item": int(chunk) if chunk else "guided (64 down to 4)",
                "warps_per_query": 1, "tuned_ms": round(float(tuned), 4), "default_ms": round(float(dflt), 4),
                "from_cache": bool(cached)}

    def close(self):
        if getattr(self, "_h", 0):
            _ext._batch_plan_destroy(self._h)
            self._h = 0

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


# --------------------------------------------------------------- resident index
class GridIndex:
    """One cloud's grid index built once and searched many times.

    pgeof rebuilds its KD-tree inside every knn_search / radius_search call
    (include/nn_search.hpp:35,39,90,97); ``GridIndex(data)`` builds the GPU
    grid once, then ``knn_search``, ``radius_search`` and ``knn_features``
    take any k or radius and return exactly what the module-level functions
    return for the same data. ``query=None`` searches the indexed points
    themselves (rows in the cloud's order). ``k_hint`` / ``radius_hint`` steer
    the cell size towards the searches that will be asked for most (speed
    only). ``data`` is a float32 (n, 3) numpy array (results come back as
    numpy) or CUDA tensor (results stay on the device, enqueued on the current
    torch stream); the index keeps its own copy of the points.
    """

    def __init__(self, data, k_hint=16, radius_hint=0.0):
        import torch

        self._numpy = not _is_torch(data)
        if self._numpy:
            import numpy as np

            if not (isinstance(data, np.ndarray) and data.dtype == np.float32):
                raise TypeError("GridIndex expects a float32 numpy array or a float32 CUDA tensor")
            data = torch.from_numpy(np.ascontiguousarray(data)).cuda()
        _dev_cloud(data, "data")
        self.device = data.device
        self.n = int(data.shape[0])
        self._h = 0
        with torch.cuda.device(self.device):
            s = int(torch.cuda.current_stream().cuda_stream)
            self._h = _ext._index_create(data.data_ptr(), self.n, int(k_hint), float(radius_hint), s)

    def __len__(self):
        return self.n

    def _query(self, torch, query):
        if query is None:
            return None, 0, self.n
        if self._numpy != (not _is_torch(query)):
            raise TypeError("query must be of the same kind (numpy or CUDA tensor) as the indexed data")
        if self._numpy:
            import numpy as np

            if not (isinstance(query, np.ndarray) and query.dtype == np.float32):
                raise TypeError("query must be a float32 numpy array")
            query = torch.from_numpy(np.ascontiguousarray(query)).to(self.device)
        _dev_cloud(query, "query")
        if query.shape[0] == 0:  # (a NULL query pointer would mean the indexed points)
            return query, None, 0
        return query, query.data_ptr(), int(query.shape[0])

    def _out(self, *ts, uint32_first=False):
        """Results as given (CUDA tensors) or as numpy arrays for numpy inputs."""
        if not self._numpy:
            return ts if len(ts) > 1 else ts[0]
        res = [_to_host(ts[0], uint32_first)] + [_to_host(t) for t in ts[1:]]
        return tuple(res) if len(res) > 1 else res[0]

    def knn_search(self, query, knn):
        """include/nn_search.hpp:31-67 on the index: (uint32 indices, float32 squared distances)."""
        import torch

        self._check_open()
        q, qp, m = self._query(torch, query)
        with torch.cuda.device(self.device):
            s = int(torch.cuda.current_stream().cuda_stream)
            idx = _uint32_empty(torch, (m, int(knn)), self.device)
            d2 = torch.empty((m, int(knn)), dtype=torch.float32, device=self.device)
            if qp is None and int(knn) > self.n:
                raise ValueError("knn size is greater than the data point cloud size")
            if qp is not None:
                _ext._dev_index_knn_search(self._h, qp, m if qp else 0, int(knn), idx.data_ptr(), d2.data_ptr(),
                                           s)
        del q
        return self._out(idx, d2, uint32_first=True)

    def radius_search(self, query, search_radius, max_knn):
        """include/nn_search.hpp:85-132 on the index: (int32 indices, -1 = none; float32 squared distances)."""
        import torch

        self._check_open()
        q, qp, m = self._query(torch, query)
        with torch.cuda.device(self.device):
            s = int(torch.cuda.current_stream().cuda_stream)
            idx = torch.empty((m, int(max_knn)), dtype=torch.int32, device=self.device)
            d2 = torch.empty((m, int(max_knn)), dtype=torch.float32, device=self.device)
            if qp is None and int(max_knn) > self.n:
                raise ValueError("max knn size is greater than the data point cloud size")
            if qp is not None:
                _ext._dev_index_radius_search(self._h, qp, m if qp else 0, float(search_radius), int(max_knn),
                                              idx.data_ptr(), d2.data_ptr(), s)
        del q
        return self._out(idx, d2)

    def knn_features(self, k, k_scales=None):
        """``knn_features(data, k, k_scales)`` on the indexed cloud."""
        import torch

        self._check_open()
        scales = [int(v) for v in k_scales] if k_scales is not None else []
        shape = (self.n, len(scales), 11) if scales else (self.n, 11)
        with torch.cuda.device(self.device):
            s = int(torch.cuda.current_stream().cuda_stream)
            out = torch.zeros(shape, dtype=torch.float32, device=self.device)
            _ext._dev_index_knn_features(self._h, int(k), scales, out.data_ptr(), s)
        return self._out(out)

    def _check_open(self):
        if not self._h:
            raise ValueError("the index is closed")

    def close(self):
        if getattr(self, "_h", 0):
            _ext._index_destroy(self._h)
            self._h = 0

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
