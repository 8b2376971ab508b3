"""Serving (the Poisson request stream): requests admitted while others run
overlap on the GPU, and every result equals the same request run alone."""

import numpy as np
import pytest

from point_geometric_features_gb300.synthetic import log_uniform_sizes, scaled_scene

pytestmark = pytest.mark.gpu


def _pool(n, lo, hi, seed):
    rng = np.random.default_rng(seed)
    sizes = log_uniform_sizes(n, lo, hi, seed)
    return [scaled_scene(int(s), seed=seed * 100 + i, side=float(rng.uniform(5.0, 50.0))) for i, s in enumerate(sizes)]


def test_results_same_alone_and_in_the_mix(cuda, pgeof):
    from point_geometric_features_gb300.serving import Request, Server, radius_for_count

    pool = _pool(10, 1_000, 60_000, seed=5)
    rng = np.random.default_rng(6)
    feats = [pgeof.Verticality, pgeof.Curvature, pgeof.Planarity, pgeof.Normal_z]
    reqs = []
    for i in range(30):
        xyz = pool[int(rng.integers(len(pool)))]
        k = int(rng.choice([16, 32, 64]))
        reqs.append(Request(i, xyz, k, radius_for_count(xyz, 1.5 * k), feats))
    alone = {r.rid: pgeof.compute_features_selected(r.xyz, r.radius, r.max_knn, feats) for r in reqs}
    server = Server(slots=4, budget_bytes=2 << 30)
    try:
        for r in reqs:  # a burst: many in flight at once
            server.submit(r)
        results = server.drain(len(reqs), timeout=300)
    finally:
        server.close()
    assert server.adm.peak_in_flight > 1  # work really overlapped
    assert len({r.slot for r in results}) > 1
    for res in results:
        np.testing.assert_array_equal(res.features, alone[res.rid])


def test_poisson_stream_summary(cuda, pgeof):
    from point_geometric_features_gb300.serving import Server, run_stream

    pool = _pool(8, 1_000, 50_000, seed=7)
    server = Server(slots=4, budget_bytes=4 << 30)
    try:
        out = run_stream(server, pool, rate=60.0, duration=2.0, seed=8)
    finally:
        server.close()
    assert out["requests"] > 60
    assert 0 < out["p50_ms"] <= out["p99_ms"] < 5_000
    assert out["points_per_s"] > 0


def test_native_server_results_same_alone_and_in_the_mix(cuda, pgeof):
    """The library's own server (pgeof_server_*): float32 and float64 requests
    in one burst overlap on the GPU and each equals the call made alone."""
    from point_geometric_features_gb300.serving import NativeServer, Request, radius_for_count

    pool = _pool(10, 1_000, 60_000, seed=9)
    rng = np.random.default_rng(10)
    feats = [pgeof.Verticality, pgeof.Curvature, pgeof.Planarity, pgeof.Normal_z, pgeof.Eigentropy]
    reqs = []
    for i in range(40):
        xyz = pool[int(rng.integers(len(pool)))]
        if i % 4 == 3:
            xyz = xyz.astype(np.float64)
        k = int(rng.choice([16, 32, 64]))
        reqs.append(Request(i, xyz, k, radius_for_count(xyz, 1.5 * k), feats))
    alone = {r.rid: pgeof.compute_features_selected(r.xyz, r.radius, r.max_knn, feats) for r in reqs}
    server = NativeServer(slots=4, budget_bytes=2 << 30)
    try:
        for r in reqs:
            server.submit(r)
        results = server.drain(len(reqs))
        assert server.adm.peak_in_flight > 1
        assert 0 < server.adm.peak_bytes <= 2 << 30
    finally:
        server.close()
    assert len(results) == len(reqs) and len({r.slot for r in results}) > 1
    for res in results:
        assert res.features.dtype == alone[res.rid].dtype
        np.testing.assert_array_equal(res.features, alone[res.rid])
        assert res.done >= res.admitted >= res.arrival


def test_native_server_reports_request_errors(cuda, pgeof):
    from point_geometric_features_gb300.serving import NativeServer, Request

    pool = _pool(2, 1_000, 2_000, seed=11)
    server = NativeServer(slots=2, budget_bytes=1 << 30)
    try:
        server.submit(Request(0, pool[0], 16, 1.0, [pgeof.Linearity]))
        bad = pool[1].copy()
        bad[0, 0] = np.inf  # rejected after the bounding box, before any cell is indexed
        server.submit(Request(1, bad, 16, 1.0, [pgeof.Linearity]))
        server.submit(Request(2, pool[1], 16, 1.0, [pgeof.Linearity]))
        with pytest.raises(ValueError, match="coordinates must be finite"):
            server.drain(3)
        res = server.drain(3)  # the other requests still complete
    finally:
        server.close()
    assert sorted(r.rid for r in res) == [0, 2]
    np.testing.assert_array_equal(res[-1].features, pgeof.compute_features_selected(pool[1], 1.0, 16,
                                                                                   [pgeof.Linearity]))


def test_native_poisson_stream_summary(cuda, pgeof):
    from point_geometric_features_gb300.serving import NativeServer, run_stream

    pool = _pool(8, 1_000, 50_000, seed=7)
    server = NativeServer(slots=4, budget_bytes=4 << 30)
    try:
        out = run_stream(server, pool, rate=60.0, duration=2.0, seed=8)
    finally:
        server.close()
    assert out["requests"] > 60
    assert 0 < out["p50_ms"] <= out["p99_ms"] < 5_000
    assert out["peak_in_flight_requests"] >= 1


def test_native_server_resident_clouds(cuda, pgeof):
    """Clouds kept on the device with their grid (add_cloud): repeated requests
    with other radii, k and feature lists, mixed with plain requests, each
    equal to compute_features_selected on the same xyz alone."""
    from point_geometric_features_gb300.serving import NativeServer, Request, radius_for_count

    pool = _pool(6, 2_000, 80_000, seed=12)
    rng = np.random.default_rng(13)
    lists = [[pgeof.Verticality, pgeof.Curvature, pgeof.Planarity, pgeof.Normal_z],
             [pgeof.Linearity, pgeof.Eigentropy], [pgeof.Normal_x, pgeof.Normal_y, pgeof.Normal_z, pgeof.Volume]]
    server = NativeServer(slots=4, budget_bytes=2 << 30)
    try:
        cids = [server.add_cloud(pool[i], radius_hint=radius_for_count(pool[i], 48), k_hint=32) for i in range(3)]
        reqs, expect = [], {}
        for i in range(36):
            j = int(rng.integers(len(pool)))
            k = int(rng.choice([16, 32, 64]))
            feats = lists[int(rng.integers(len(lists)))]
            r = radius_for_count(pool[j], float(rng.uniform(0.5, 3.0)) * k)
            req = Request(i, pool[j], k, r, feats, cloud=cids[j] if j < 3 and i % 3 else 0)
            reqs.append(req)
            expect[i] = pgeof.compute_features_selected(pool[j], r, k, feats)
        for req in reqs:
            server.submit(req)
        results = server.drain(len(reqs))
        assert server.adm.peak_in_flight > 1
        server.remove_cloud(cids[0])
        with pytest.raises(ValueError, match="unknown resident cloud"):
            server.submit(Request(99, None, 16, 1.0, lists[0], cloud=cids[0]))
    finally:
        server.close()
    assert sum(1 for r in reqs if r.cloud) >= 10
    for res in results:
        np.testing.assert_array_equal(res.features, expect[res.rid])


def test_native_stream_at_the_serving_rate(cuda, pgeof):
    """The serving workload's shape at its full rate for 4 s: Poisson arrivals
    at 200 req/s, clouds log-uniform in [1,000, 500,000] points, k in
    {16, 32, 64}, the four selected features, 8 slots and a 40 GB budget. Every
    request completes, requests overlap on the GPU, and a sample of 40 results
    equals the same requests run alone."""
    import time

    from point_geometric_features_gb300.serving import NativeServer, Request, poisson_arrivals, radius_for_count

    pool = _pool(24, 1_000, 500_000, seed=13)
    feats = [pgeof.Verticality, pgeof.Curvature, pgeof.Planarity, pgeof.Normal_z]
    rng = np.random.default_rng(14)
    times = poisson_arrivals(200.0, 4.0, 15)
    reqs = []
    for i, _ in enumerate(times):
        xyz = pool[int(rng.integers(len(pool)))]
        k = int(rng.choice([16, 32, 64]))
        reqs.append(Request(i, xyz, k, radius_for_count(xyz, 1.5 * k), feats))
    server = NativeServer(slots=8, budget_bytes=40 << 30)
    try:
        t0 = time.perf_counter()
        for req, t in zip(reqs, times):
            now = time.perf_counter() - t0
            if t > now:
                time.sleep(t - now)
            req.arrival = t0 + t
            server.submit(req)
        results = server.drain(len(reqs))
        peak = server.adm.peak_in_flight
    finally:
        server.close()
    assert len(reqs) > 600 and len(results) == len(reqs)
    assert peak > 1
    lat = np.array([r.latency_ms for r in results])
    print(f"[serving] {len(reqs)} requests, p50 {np.percentile(lat, 50):.3f} ms, p99 {np.percentile(lat, 99):.3f} ms, "
          f"peak in flight {peak}")
    by_rid = {r.rid: r for r in results}
    for rid in np.random.default_rng(16).choice(len(reqs), 40, replace=False):
        r = reqs[int(rid)]
        np.testing.assert_array_equal(by_rid[int(rid)].features,
                                      pgeof.compute_features_selected(r.xyz, r.radius, r.max_knn, feats))
