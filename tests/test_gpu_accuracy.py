"""The 4M-point outdoor scene (seed 2), radius_search(r=0.5, max_knn=64) ->
CSR -> compute_features_optimal(k_min=1, k_step=1, k_min_search=10), with each
feature's error against the FP64 oracle (numpy float64 restatement of
include/pca.hpp / include/pgeof.hpp:243-310) on a 3,000-row sample.

Reported per feature: max |gpu - fp64| and max relative error (|x| > 1e-3),
the normal's angle error (radians, sign-agnostic), the agreement of the
optimal k with the FP32-literal oracle and with the FP64 argmin. Bounds: the
1e-4 abs target on linearity / planarity / scattering / verticality and
1e-3 rad on normals hold for the rows whose eigenvectors are well conditioned
(relative eigen-gap >= 1e-3); the ascending-order Scattering reaches ~1e3, so
the 1e-4 bound is applied relative to max(1, |x|).
"""

import numpy as np
import pytest

from oracle import oracle
from point_geometric_features_gb300.synthetic import outdoor_scene

pytestmark = pytest.mark.gpu

NAMES = ["Linearity", "Planarity", "Scattering", "VerticalityPGEOF", "Normal_x", "Normal_y", "Normal_z", "Length",
         "Surface", "Volume", "Curvature"]


def _fp64_optimal(P, k0, k_nn):
    """FP64 eigentropy argmin (first minimum) over k in [k0, k_nn] (k_step = 1) for one row."""
    best, best_k = None, k0
    for k in range(k0, k_nn + 1):
        w, _, _ = oracle.fp64_eig(P[None, :k])
        e = oracle.fp64_eigentropy(w)[0]
        if best is None or e < best:
            best, best_k = e, k
    return best_k


def test_optimal_4m_errors_vs_fp64(cuda, pgeof):
    torch = cuda
    xyz = outdoor_scene(4_000_000, seed=2)
    t = torch.from_numpy(xyz).cuda()
    idx, _ = pgeof.radius_search(t, t, 0.5, 64)
    mask = idx >= 0
    cnt = mask.sum(1)
    ptr = torch.zeros(xyz.shape[0] + 1, dtype=torch.int64, device="cuda")
    ptr[1:] = torch.cumsum(cnt, 0)
    nn = idx[mask].to(torch.int32)
    out = pgeof.compute_features_optimal(t, nn, ptr.to(torch.int32), 1, 1, 10).cpu().numpy()

    rng = np.random.default_rng(0)
    rows = rng.choice(xyz.shape[0], 3000, replace=False)
    idx_h = idx[torch.from_numpy(rows).cuda()].cpu().numpy()
    k_gpu = out[rows, 11].astype(int)
    # FP32-literal oracle on the sample's CSR
    sub_nn = np.concatenate([r[r >= 0] for r in idx_h]).astype(np.uint32)
    sub_ptr = np.r_[0, np.cumsum((idx_h >= 0).sum(1))].astype(np.uint32)
    ref32 = oracle.compute_features_optimal(xyz, sub_nn, sub_ptr, 1, 1, 10)
    agree32 = float((ref32[:, 11] == out[rows, 11]).mean())

    gaps, agree64, valid = [], [], 0
    f64_rows, gpu_rows = [], []
    for j, r in enumerate(rows):
        nb = idx_h[j][idx_h[j] >= 0]
        if nb.size < 10:
            assert np.all(out[r] == 0)
            continue
        valid += 1
        P = xyz[nb].astype(np.float64)
        k = k_gpu[j]
        w, V, _ = oracle.fp64_eig(P[None, :k])
        f64 = oracle.fp64_features_from_eig(w, V)[0]
        gaps.append(oracle.fp64_relative_gap(P[None, :k])[0])
        f64_rows.append(f64)
        gpu_rows.append(out[r, :11].astype(np.float64))
        if j < 300:
            agree64.append(_fp64_optimal(P, 10, nb.size) == k)
    F64 = np.array(f64_rows)
    G = np.array(gpu_rows)
    gaps = np.array(gaps)
    n_dot = np.abs((F64[:, 4:7] * G[:, 4:7]).sum(1)) / np.maximum(
        np.linalg.norm(F64[:, 4:7], axis=1) * np.linalg.norm(G[:, 4:7], axis=1), 1e-30)
    ang = np.arccos(np.clip(n_dot, -1.0, 1.0))
    good = gaps >= 1e-3
    lines = [f"rows {valid}, k_opt agreement: FP32 oracle {agree32:.4f}, FP64 argmin (300 rows) "
             f"{np.mean(agree64):.4f}; well-conditioned rows {good.mean():.4f}"]
    lines.append(f"{'feature':18s} {'max abs':>10s} {'max rel':>10s} {'max abs (gap>=1e-3)':>20s}")
    for i, n in enumerate(NAMES):
        d = np.abs(G[:, i] - F64[:, i])
        rel = d / np.maximum(np.abs(F64[:, i]), 1e-3)
        lines.append(f"{n:18s} {d.max():10.3e} {rel.max():10.3e} {d[good].max():20.3e}")
    lines.append(f"normal angle (rad): max {ang.max():.3e}, max well-conditioned {ang[good].max():.3e}")
    print("\n" + "\n".join(lines))
    assert agree32 >= 0.999
    scaled = np.abs(G - F64) / np.maximum(1.0, np.abs(F64))
    for i in (0, 1, 2, 3):
        assert scaled[good, i].max() < 1e-4, NAMES[i]
    assert ang[good].max() < 1e-3
