"""pgeof_compute_features_f32_noalloc: compute_features for callers that cannot
allocate GPU memory during the call (a pre-sized memory budget, a host that
owns the device heap, a latency-bound loop). Its only scratch is a fixed
device array inside the library, so its results must equal the allocating
entry point's -- on consecutive calls too, because every call reuses (and
overwrites) the same array.

Kept in its own file, collected last, so that a run stopping at the first
failure has run every other test before this one."""

import ctypes

import numpy as np
import pytest

from conftest import feature_close
from point_geometric_features_gb300.synthetic import outdoor_scene, uniform_cube

pytestmark = pytest.mark.gpu

CAPACITY = 1 << 20


def _lib(pgeof):
    lib = ctypes.CDLL(pgeof.LIBRARY_PATH)
    P, I64 = ctypes.c_void_p, ctypes.c_int64
    lib.pgeof_compute_features_f32.argtypes = [P, I64, P, I64, P, I64, ctypes.c_uint64, P, P]
    lib.pgeof_compute_features_f32_noalloc.argtypes = [P, I64, P, I64, P, I64, ctypes.c_uint64, P, P, P]
    lib.pgeof_device_alloc_count.restype = ctypes.c_uint64
    lib.pgeof_take_device_errors.argtypes = [P, ctypes.POINTER(ctypes.c_uint32)]
    return lib


def _case(torch, pgeof, xyz, k):
    t = torch.from_numpy(xyz).cuda()
    idx, _ = pgeof.knn_search(t, t, k)
    nn = idx.reshape(-1).to(torch.int32)
    ptr = torch.arange(0, k * (xyz.shape[0] + 1), k, dtype=torch.int32, device="cuda")
    return t, nn, ptr


def _run(lib, fn_name, t, nn, ptr, k_min, torch, err=None):
    n = ptr.shape[0] - 1
    out = torch.full((n, 11), float("nan"), dtype=torch.float32, device="cuda")
    s = torch.cuda.current_stream().cuda_stream
    args = [t.data_ptr(), t.shape[0], nn.data_ptr(), nn.shape[0], ptr.data_ptr(), n, k_min, out.data_ptr()]
    if fn_name.endswith("noalloc"):
        args.append(err.data_ptr() if err is not None else None)
    st = getattr(lib, fn_name)(*args, s)
    torch.cuda.synchronize()
    return st, out.cpu().numpy()


def test_noalloc_matches_allocating_entry_point_on_consecutive_calls(cuda, pgeof):
    torch = cuda
    lib = _lib(pgeof)
    cases = [
        (uniform_cube(20_000, seed=31), 16, 1),
        (outdoor_scene(6_000, seed=32), 24, 10),  # smaller cloud: stale scratch beyond it must not leak in
        (uniform_cube(20_000, seed=31), 16, 1),
    ]
    for xyz, k, k_min in cases:
        t, nn, ptr = _case(torch, pgeof, xyz, k)
        before = lib.pgeof_device_alloc_count()
        st_ref, ref = _run(lib, "pgeof_compute_features_f32", t, nn, ptr, k_min, torch)
        assert st_ref == 0
        assert lib.pgeof_device_alloc_count() > before  # the counter sees the allocating entry point's scratch
        before = lib.pgeof_device_alloc_count()
        st, got = _run(lib, "pgeof_compute_features_f32_noalloc", t, nn, ptr, k_min, torch)
        assert st == 0
        assert lib.pgeof_device_alloc_count() == before, "the no-allocation entry point allocated device memory"
        assert np.isfinite(got).all()
        assert feature_close(got, ref).all()


def test_noalloc_reports_data_errors_and_rejects_oversize(cuda, pgeof):
    torch = cuda
    lib = _lib(pgeof)
    xyz = uniform_cube(4_000, seed=33)
    t, nn, ptr = _case(torch, pgeof, xyz, 8)
    err = torch.zeros(1, dtype=torch.int32, device="cuda")
    st, _ = _run(lib, "pgeof_compute_features_f32_noalloc", t, nn, ptr, 1, torch, err)
    assert st == 0 and int(err.item()) == 0
    bad = nn.clone()
    bad[5] = xyz.shape[0]  # an index past the end of xyz: flagged, never read
    st, _ = _run(lib, "pgeof_compute_features_f32_noalloc", t, bad, ptr, 1, torch, err)
    assert st == 0 and int(err.item()) & 1
    # without a caller word the bits wait in the library's word for pgeof_take_device_errors
    s = torch.cuda.current_stream().cuda_stream
    bits = ctypes.c_uint32(0)
    assert lib.pgeof_take_device_errors(s, ctypes.byref(bits)) == 0  # drain anything earlier
    st, _ = _run(lib, "pgeof_compute_features_f32_noalloc", t, bad, ptr, 1, torch)
    assert st == 0
    assert lib.pgeof_take_device_errors(s, ctypes.byref(bits)) == 0 and bits.value & 1
    assert lib.pgeof_take_device_errors(s, ctypes.byref(bits)) == 0 and bits.value == 0  # read once, then cleared
    # beyond the fixed capacity: rejected before any device work
    st = lib.pgeof_compute_features_f32_noalloc(t.data_ptr(), CAPACITY + 1, nn.data_ptr(), nn.shape[0],
                                                ptr.data_ptr(), ptr.shape[0] - 1, 1, t.data_ptr(), None, s)
    assert st == 1
    lib.pgeof_last_error_message.restype = ctypes.c_char_p
    assert b"at most" in lib.pgeof_last_error_message()
