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


FEATURE_NAMES = ["Linearity", "Planarity", "Scattering", "VerticalityPGEOF", "Normal_x", "Normal_y", "Normal_z",
                 "Length", "Surface", "Volume", "Curvature", "K_optimal"]

# The parity bar: |gpu - ref| <= 1e-4 * max(1, |ref|) per value, i.e. 1e-4
# absolute where |ref| <= 1 and 1e-4 relative above (the ascending-order
# ratios Linearity / Planarity / Scattering reach ~1e1 .. 1e3).
FEATURE_TOL = 1e-4


def scaled_error(a, b):
    """|a - b| / max(1, |b|) elementwise, in float64."""
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return np.abs(a - b) / np.maximum(1.0, np.abs(b))


def feature_close(a, b, tol=FEATURE_TOL):
    """|a - b| <= tol * max(1, |b|) elementwise."""
    return scaled_error(a, b) <= tol


def feature_report(a, b, names=None, label=""):
    """Per-column max scaled error of a (rows, columns) feature block against
    its reference, printed (pytest -s / -rP shows it) and returned."""
    e = scaled_error(a, b)
    e = e.reshape(-1, e.shape[-1]) if e.ndim > 1 else e.reshape(-1, 1)
    cols = e.shape[1]
    names = names or (FEATURE_NAMES[:cols] if cols <= len(FEATURE_NAMES) else [str(i) for i in range(cols)])
    worst = e.max(axis=0) if e.shape[0] else np.zeros(cols)
    print(f"[parity] {label} rows={e.shape[0]} max |d|/max(1,|ref|): "
          + " ".join(f"{n}={w:.2e}" for n, w in zip(names, worst)))
    return dict(zip(names, worst.tolist()))


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
