"""Child process of tests/test_gpu_features.py::test_row_order_is_invisible:
computes features with the row-order threshold taken from the environment
(read once per process) and saves them for the parent to compare."""
import os
import sys

import numpy as np
import torch

sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
import point_geometric_features_gb300 as pgeof  # noqa: E402
from point_geometric_features_gb300.synthetic import outdoor_scene  # noqa: E402

out_path = sys.argv[1]
t = torch.from_numpy(outdoor_scene(120_000, seed=51)).cuda()
idx, _ = pgeof.knn_search(t, t, 20)
nn = idx.reshape(-1)
ptr = torch.arange(0, 20 * (t.shape[0] + 1), 20, dtype=torch.int32, device="cuda")
f1 = pgeof.compute_features(t, nn, ptr).cpu().numpy()
f3 = pgeof.compute_features_multiscale(t, nn, ptr, [5, 10, 20]).cpu().numpy()
# a CSR that is not a kNN table: variable rows, some empty, reversed order
rng = np.random.default_rng(5)
cnt = rng.integers(0, 30, t.shape[0])
ptr2 = np.zeros(t.shape[0] + 1, np.int64)
ptr2[1:] = np.cumsum(cnt)
nn2 = rng.integers(0, t.shape[0], int(ptr2[-1])).astype(np.int32)
g = pgeof.compute_features(t, torch.from_numpy(nn2).cuda(), torch.from_numpy(ptr2.astype(np.int32)).cuda()).cpu().numpy()
np.savez(out_path, f1=f1, f3=f3, g=g)
