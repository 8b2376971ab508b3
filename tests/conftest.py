import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GB300 device (parity tests through the C ABI)")


@pytest.fixture(scope="session")
def golden():
    def load(name):
        return dict(np.load(os.path.join(GOLDEN, name)))

    return load


@pytest.fixture(scope="session")
def cuda():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    torch.cuda.set_device(0)
    return torch


@pytest.fixture(scope="session")
def pgeof():
    import point_geometric_features_gb300 as p

    return p


def feature_close(a, b, rtol=1e-4, atol=1e-4):
    """|a - b| <= atol + rtol * |b| elementwise (features span ~1e-3 .. 1e3)."""
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return np.abs(a - b) <= atol + rtol * np.abs(b)


def align_normals(f_gpu, f_ref, cols=(4, 5, 6)):
    """Normals are only defined up to sign when n_z is numerically 0 (the
    reference's z-flip then keeps whatever sign the solver produced); align
    those rows before comparing."""
    f_gpu = np.array(f_gpu, copy=True)
    nz = np.abs(f_ref[..., cols[2]]) < 1e-4
    dot = (f_gpu[..., cols[0]] * f_ref[..., cols[0]] + f_gpu[..., cols[1]] * f_ref[..., cols[1]])
    flip = nz & (dot < 0)
    for c in cols:
        f_gpu[..., c] = np.where(flip, -f_gpu[..., c], f_gpu[..., c])
    return f_gpu
