"""Resident grid index (pgeof_index_*, GridIndex): one build, many searches.

Every search on the index must return exactly what the per-call entry points
(include/nn_search.hpp:31-132) return -- and the oracle -- for any k, radius
or query set, whatever k_hint / radius_hint the index was built with; the
fused feature pipeline on the index must equal knn_features on the cloud."""

import numpy as np
import pytest

from oracle import oracle
from point_geometric_features_gb300.synthetic import outdoor_scene, uniform_cube

pytestmark = pytest.mark.gpu

_CACHE = {}


def _oracle(kind, xyz, *args):
    """Oracle results shared by the parametrized cases (same cloud, same args)."""
    key = (kind, xyz.shape[0], float(xyz[0, 0]), args)
    if key not in _CACHE:
        _CACHE[key] = getattr(oracle, kind)(xyz, xyz, *args)
    return _CACHE[key]


@pytest.mark.parametrize("k_hint", [4, 16, 64])
def test_index_knn_self_many_k_matches_oracle(cuda, pgeof, k_hint):
    xyz = outdoor_scene(20_000, seed=11)
    with pgeof.GridIndex(xyz, k_hint=k_hint) as ix:
        assert len(ix) == xyz.shape[0]
        for k in (1, 9, 50, 130):  # 130: the general kernel (k > 128)
            idx, d2 = ix.knn_search(None, k)
            assert idx.dtype == np.uint32 and d2.dtype == np.float32 and idx.shape == (xyz.shape[0], k)
            ri, rd = _oracle("knn_search", xyz, k)
            np.testing.assert_array_equal(d2, rd)
            np.testing.assert_array_equal(idx, ri)


def test_index_knn_external_queries_equal_per_call(cuda, pgeof):
    rng = np.random.default_rng(12)
    data = uniform_cube(30_000, seed=12)
    query = (rng.random((5_000, 3), dtype=np.float32) * 1.4 - 0.2).astype(np.float32)  # some outside the box
    with pgeof.GridIndex(data, k_hint=32) as ix:
        for k in (5, 32, 77):
            idx, d2 = ix.knn_search(query, k)
            pi, pd = pgeof.knn_search(data, query, k)
            np.testing.assert_array_equal(idx, pi)
            np.testing.assert_array_equal(d2, pd)
        ri, rd = oracle.knn_search(data, query, 77)
        np.testing.assert_array_equal(idx, ri)
        np.testing.assert_array_equal(d2, rd)


@pytest.mark.parametrize("radius_hint", [0.0, 0.02, 0.3])
def test_index_radius_many_radii_matches_oracle(cuda, pgeof, radius_hint):
    xyz = uniform_cube(15_000, seed=13)
    with pgeof.GridIndex(xyz, k_hint=20, radius_hint=radius_hint) as ix:
        for r, max_knn in ((0.01, 8), (0.05, 30), (0.2, 64)):
            idx, d2 = ix.radius_search(None, r, max_knn)
            assert idx.dtype == np.int32 and idx.shape == (xyz.shape[0], max_knn)
            ri, rd = _oracle("radius_search", xyz, r, max_knn)
            np.testing.assert_array_equal(idx, ri)
            np.testing.assert_array_equal(d2, rd)
        q = xyz[::7].copy()
        idx, d2 = ix.radius_search(q, 0.05, 30)
        pi, pd = pgeof.radius_search(xyz, q, 0.05, 30)
        np.testing.assert_array_equal(idx, pi)
        np.testing.assert_array_equal(d2, pd)


def test_index_knn_features_equal_fused_per_call(cuda, pgeof):
    torch = cuda
    xyz = torch.from_numpy(outdoor_scene(50_000, seed=14)).cuda()
    ix = pgeof.GridIndex(xyz, k_hint=50)
    for k, scales in ((50, [10, 20, 50]), (20, None), (32, [8, 8, 32])):
        got = ix.knn_features(k, scales)
        want = pgeof.knn_features(xyz, k, scales)
        assert got.is_cuda and got.shape == want.shape
        assert torch.equal(got, want)
    ix.close()


def test_index_device_tensors_and_streams(cuda, pgeof):
    """Two torch streams search one index concurrently; close() while the
    second stream's search is still queued waits for it."""
    torch = cuda
    data = torch.from_numpy(uniform_cube(200_000, seed=15)).cuda()
    ix = pgeof.GridIndex(data, k_hint=16)
    ref_i, ref_d = pgeof.knn_search(data, data, 16)
    s1, s2 = torch.cuda.Stream(), torch.cuda.Stream()
    s1.wait_stream(torch.cuda.current_stream())
    s2.wait_stream(torch.cuda.current_stream())
    with torch.cuda.stream(s1):
        a_i, a_d = ix.knn_search(None, 16)
    with torch.cuda.stream(s2):
        b_i, b_d = ix.knn_search(data, 16)
    ix.close()
    torch.cuda.synchronize()
    for i, d in ((a_i, a_d), (b_i, b_d)):
        assert i.is_cuda and torch.equal(i.view(torch.int32), ref_i.view(torch.int32)) and torch.equal(d, ref_d)


def test_index_errors(cuda, pgeof):
    xyz = uniform_cube(100, seed=16)
    ix = pgeof.GridIndex(xyz)
    with pytest.raises(ValueError, match="knn size is greater"):
        ix.knn_search(None, 101)
    with pytest.raises(ValueError, match="max knn size is greater"):
        ix.radius_search(None, 0.1, 101)
    with pytest.raises(ValueError, match="k_scales"):
        ix.knn_features(10, [5, 3])
    with pytest.raises(TypeError):
        ix.knn_search(xyz.astype(np.float64), 3)
    idx, d2 = ix.knn_search(np.zeros((0, 3), np.float32), 5)
    assert idx.shape == (0, 5) and idx.dtype == np.uint32 and d2.shape == (0, 5)
    idx, d2 = ix.radius_search(np.zeros((0, 3), np.float32), 0.1, 5)
    assert idx.shape == (0, 5) and idx.dtype == np.int32
    with pytest.raises(ValueError, match="knn size is greater"):
        ix.knn_search(np.zeros((0, 3), np.float32), 101)
    ix.close()
    with pytest.raises(ValueError, match="closed"):
        ix.knn_search(None, 3)
    with pytest.raises(ValueError, match="at least one point"):
        pgeof.GridIndex(np.zeros((0, 3), np.float32))
