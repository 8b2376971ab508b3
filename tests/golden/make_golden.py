"""Regenerate the golden fixtures in this folder.

    python tests/golden/make_golden.py

Sources of truth:
* neighbour indices -- scipy.spatial.KDTree, the comparator the reference's own
  tests use (tests/test_pgeof.py:8-27: kNN on 1000 points in [0, 200)^3 with
  k=10; radius 0.2 with 10 neighbours on 1000 points in [0, 1)^3, missing = -1).
  The reference seeds nothing; these fixtures fix seeds 11 and 12.
* distances and features -- the oracle (oracle/pgeof_oracle.c, FP32-literal
  restatement of include/pca.hpp and include/pgeof.hpp) and the FP64 numpy
  restatement (oracle/oracle.py), on a 2000-point uniform cloud (seed 0) with
  k=20 neighbours.
"""

from __future__ import annotations

import os
import sys

import numpy as np
from scipy.spatial import KDTree

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import oracle  # noqa: E402


def main():
    # --- reference test shapes (tests/test_pgeof.py:8-27), seeded
    rng = np.random.default_rng(11)
    xyz = rng.uniform(0.0, 200.0, size=(1000, 3)).astype(np.float32)
    _, knn_idx = KDTree(xyz).query(xyz, k=10)
    np.savez_compressed(os.path.join(HERE, "knn_1000_k10.npz"), xyz=xyz, scipy_idx=knn_idx.astype(np.int64))

    rng = np.random.default_rng(12)
    xyz = rng.random(size=(1000, 3), dtype=np.float32)
    _, r_idx = KDTree(xyz).query(xyz, k=10, distance_upper_bound=0.2)
    r_idx[r_idx == xyz.shape[0]] = -1
    np.savez_compressed(os.path.join(HERE, "radius_1000_r02_k10.npz"), xyz=xyz, scipy_idx=r_idx.astype(np.int64))

    # --- features on a small uniform cloud
    rng = np.random.default_rng(0)
    xyz = rng.random((2000, 3), dtype=np.float32)
    k = 20
    idx, d2 = oracle.knn_search(xyz, xyz, k)
    nn = idx.reshape(-1).astype(np.uint32)
    nn_ptr = (np.arange(xyz.shape[0] + 1) * k).astype(np.uint32)
    feats = oracle.compute_features(xyz, nn, nn_ptr, 1)
    multi = oracle.compute_features_multiscale(xyz, nn, nn_ptr, [5, 10, 20])
    opt = oracle.compute_features_optimal(xyz, nn, nn_ptr, 1, 1, 5)
    ids = [12, 10, 1, 6, 13, 3]  # Verticality, Curvature, Planarity, Normal_z, Eigentropy, VerticalityPGEOF
    sel32 = oracle.compute_features_selected(xyz, 0.1, 20, ids)
    sel64 = oracle.compute_features_selected(xyz.astype(np.float64), 0.1, 20, ids)
    f64 = oracle.fp64_compute_features(xyz, nn, nn_ptr, 1)
    np.savez_compressed(
        os.path.join(HERE, "features_2000_k20.npz"),
        xyz=xyz, idx=idx, d2=d2, features=feats, multiscale=multi, optimal=opt,
        selected_ids=np.array(ids, np.int32), selected_f32=sel32, selected_f64=sel64, features_fp64=f64,
    )
    print("fixtures written to", HERE)


if __name__ == "__main__":
    main()
