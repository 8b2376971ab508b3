"""Multi-cloud batches (the 256-cloud workload's shape, scaled down): one device pipeline
over many clouds of uneven size must equal per-cloud knn_search +
compute_features calls exactly, also when replayed from a CUDA graph on new
data."""

import numpy as np
import pytest

from point_geometric_features_gb300.synthetic import log_uniform_sizes, scaled_scene, uniform_cube

pytestmark = pytest.mark.gpu


def _clouds(torch, n_clouds, lo, hi, seed):
    sizes = log_uniform_sizes(n_clouds, lo, hi, seed)
    rng = np.random.default_rng(seed)
    out = []
    for i, n in enumerate(sizes):
        side = float(rng.uniform(5.0, 50.0))
        out.append(torch.from_numpy(scaled_scene(int(n), seed=seed * 1000 + i, side=side)).cuda())
    return out


def _per_cloud(pgeof, torch, clouds, k):
    idx, d2, feats = [], [], []
    for c in clouds:
        i, d = pgeof.knn_search(c, c, k)
        ptr = torch.arange(0, k * (c.shape[0] + 1), k, dtype=torch.int32, device="cuda")
        f = pgeof.compute_features(c, i.reshape(-1), ptr)
        idx.append(i.cpu().numpy().astype(np.uint32))
        d2.append(d.cpu().numpy())
        feats.append(f.cpu().numpy())
    return np.concatenate(idx), np.concatenate(d2), np.concatenate(feats)


@pytest.mark.parametrize("k", [8, 32])
def test_batch_equals_per_cloud(cuda, pgeof, k):
    torch = cuda
    clouds = _clouds(torch, 24, 300, 30_000, seed=3)
    ri, rd, rf = _per_cloud(pgeof, torch, clouds, k)
    bi, bd, bf = pgeof.batch_knn_features(clouds, k)
    np.testing.assert_array_equal(bi.cpu().numpy().astype(np.uint32), ri)
    np.testing.assert_array_equal(bd.cpu().numpy(), rd)
    np.testing.assert_array_equal(bf.cpu().numpy(), rf)


def test_batch_plan_replay_on_new_data(cuda, pgeof):
    torch = cuda
    clouds = _clouds(torch, 16, 200, 20_000, seed=4)
    plan = pgeof.BatchPlan(clouds, 16)
    for rep in range(2):
        if rep == 1:
            # same shapes, new points: refill the plan's input in place and replay
            clouds = [torch.from_numpy(uniform_cube(int(c.shape[0]), seed=77 + j, side=7.0)).cuda()
                      for j, c in enumerate(clouds)]
            plan.xyz.copy_(torch.cat(clouds, 0))
        bi, bd, bf = plan()
        torch.cuda.synchronize()
        ri, rd, rf = _per_cloud(pgeof, torch, clouds, 16)
        np.testing.assert_array_equal(bi.cpu().numpy().astype(np.uint32), ri)
        np.testing.assert_array_equal(bd.cpu().numpy(), rd)
        np.testing.assert_array_equal(bf.cpu().numpy(), rf)
    plan.close()


def test_full_256_cloud_batch_equals_per_cloud(cuda, pgeof):
    """The batch workload as stated: 256 clouds with sizes log-uniform in
    [2,000, 200,000] (seed 3), each the outdoor-scene generator scaled to a
    cube side U(5, 50) m, knn k=32 + compute_features. Every cloud's indices,
    distances and features from the graph-captured batch plan equal its
    per-cloud knn_search + compute_features results."""
    torch = cuda
    k = 32
    sizes = log_uniform_sizes(256, 2_000, 200_000, seed=3)
    rng = np.random.default_rng(3)
    clouds = [torch.from_numpy(scaled_scene(int(n), seed=3000 + i, side=float(rng.uniform(5.0, 50.0)))).cuda()
              for i, n in enumerate(sizes)]
    assert len(clouds) == 256
    plan = pgeof.BatchPlan(clouds, k)
    bi, bd, bf = plan()
    torch.cuda.synchronize()
    off = 0
    for j, c in enumerate(clouds):
        n = int(c.shape[0])
        i, d = pgeof.knn_search(c, c, k)
        ptr = torch.arange(0, k * (n + 1), k, dtype=torch.int32, device="cuda")
        f = pgeof.compute_features(c, i.reshape(-1), ptr)
        assert torch.equal(bi[off:off + n].view(torch.int32), i.view(torch.int32)), f"cloud {j}: indices"
        assert torch.equal(bd[off:off + n], d), f"cloud {j}: distances"
        assert torch.equal(bf[off:off + n], f), f"cloud {j}: features"
        off += n
    assert off == plan.xyz.shape[0]
    plan.close()


def test_batch_errors_and_tiny_clouds(cuda, pgeof):
    torch = cuda
    a = torch.from_numpy(uniform_cube(5, seed=1)).cuda()
    b = torch.from_numpy(uniform_cube(3000, seed=2)).cuda()
    with pytest.raises(ValueError):
        pgeof.batch_knn_features([a, b], 6)  # k larger than the first cloud
    bi, bd, bf = pgeof.batch_knn_features([a, b], 5)  # a cloud of exactly k points
    ri, rd, rf = _per_cloud(pgeof, torch, [a, b], 5)
    np.testing.assert_array_equal(bi.cpu().numpy().astype(np.uint32), ri)
    np.testing.assert_array_equal(bf.cpu().numpy(), rf)
