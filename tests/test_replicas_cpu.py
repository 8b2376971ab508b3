"""Multi-process host logic of the replica path (no GPU): query-row ranges,
cloud partitions and the max-over-ranks timing reduction, run as two gloo
ranks on CPU. The oracle stands in for each rank's device pass, so the test
checks that sharded rows concatenate to the one-process result exactly."""

import os
import socket

import numpy as np
import pytest

from point_geometric_features_gb300.replicas import partition_clouds, query_range


@pytest.mark.parametrize("m", [0, 1, 7, 1000, 1_000_003])
@pytest.mark.parametrize("world", [1, 2, 3, 8])
def test_query_range_partitions_rows(m, world):
    ranges = [query_range(m, r, world) for r in range(world)]
    assert ranges[0][0] == 0 and ranges[-1][1] == m
    for (a0, a1), (b0, b1) in zip(ranges, ranges[1:]):
        assert a1 == b0
    sizes = [hi - lo for lo, hi in ranges]
    assert max(sizes) - min(sizes) <= 1 and min(sizes) >= 0


def test_query_range_rejects_bad_arguments():
    for args in ((10, 2, 2), (10, -1, 2), (10, 0, 0), (-1, 0, 1)):
        with pytest.raises(ValueError):
            query_range(*args)


def test_partition_clouds_balanced_and_complete():
    rng = np.random.default_rng(3)
    sizes = np.exp(rng.uniform(np.log(2000), np.log(200_000), 256)).astype(int)
    for world in (1, 2, 4, 8):
        parts = partition_clouds(sizes, world)
        flat = sorted(i for p in parts for i in p)
        assert flat == list(range(len(sizes)))
        loads = [int(sizes[p].sum()) if p else 0 for p in parts]
        assert max(loads) - min(loads) <= int(sizes.max())
        assert all(p == sorted(p) for p in parts)
        assert parts == partition_clouds(sizes, world)  # deterministic
    with pytest.raises(ValueError):
        partition_clouds([1, 2], 0)


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out_dir):
    import torch.distributed as dist

    from oracle import oracle
    from point_geometric_features_gb300.replicas import max_over_ranks, partition_clouds, query_range
    from point_geometric_features_gb300.synthetic import scaled_scene, uniform_cube

    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        # one cloud, query rows split over the ranks on a replicated cloud
        xyz = uniform_cube(3000, seed=5)
        lo, hi = query_range(xyz.shape[0], rank, world)
        idx, d2 = oracle.knn_search(xyz, xyz[lo:hi], 10, threads=1)
        rows = [None] * world
        dist.all_gather_object(rows, (lo, idx, d2))
        # independent clouds split over the ranks
        sizes = [300, 1200, 450, 900, 60, 2000, 700]
        clouds = [scaled_scene(n, seed=40 + i, side=10.0) for i, n in enumerate(sizes)]
        mine = partition_clouds(sizes, world)[rank]
        feats = {}
        for i in mine:
            ci, _ = oracle.knn_search(clouds[i], clouds[i], 8, threads=1)
            ptr = (np.arange(sizes[i] + 1) * 8).astype(np.uint32)
            feats[i] = oracle.compute_features(clouds[i], ci.reshape(-1), ptr, threads=1)
        parts = [None] * world
        dist.all_gather_object(parts, feats)
        t_max = max_over_ranks(0.5 + rank)
        if rank == 0:
            full_idx, full_d2 = oracle.knn_search(xyz, xyz, 10, threads=1)
            rows.sort(key=lambda r: r[0])
            np.testing.assert_array_equal(np.concatenate([r[1] for r in rows]), full_idx)
            np.testing.assert_array_equal(np.concatenate([r[2] for r in rows]), full_d2)
            merged = {}
            for p in parts:
                assert not set(p) & set(merged)
                merged.update(p)
            assert sorted(merged) == list(range(len(sizes)))
            for i, n in enumerate(sizes):
                ci, _ = oracle.knn_search(clouds[i], clouds[i], 8, threads=1)
                ptr = (np.arange(n + 1) * 8).astype(np.uint32)
                np.testing.assert_array_equal(merged[i], oracle.compute_features(clouds[i], ci.reshape(-1), ptr,
                                                                                 threads=1))
            assert t_max == 0.5 + (world - 1)
            open(os.path.join(out_dir, "ok"), "w").write("ok")
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks_shard_rows_and_clouds(tmp_path):
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp

    from oracle import oracle

    oracle.build()
    mp.spawn(_rank_main, args=(2, _free_port(), str(tmp_path)), nprocs=2, join=True)
    assert (tmp_path / "ok").exists()
    del torch
