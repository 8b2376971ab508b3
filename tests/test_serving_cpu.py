"""Admission control of the serving loop, on the host (no GPU): the byte
budget and the slot count are never exceeded, every request is admitted, and
a request larger than the whole budget still runs (alone)."""

import random
import threading
import time

from point_geometric_features_gb300.serving import AdmissionControl, poisson_arrivals, request_footprint


def test_budget_and_slots_hold_under_contention():
    adm = AdmissionControl(slots=3, budget_bytes=1000)
    seen = {"bytes": 0, "slots": 0, "max_bytes": 0, "max_slots": 0}
    lock = threading.Lock()
    done = []

    def client(i):
        rng = random.Random(i)
        for _ in range(20):
            nb = rng.randint(50, 700)
            slot = adm.admit(nb)
            with lock:
                seen["bytes"] += min(nb, 1000)
                seen["slots"] += 1
                seen["max_bytes"] = max(seen["max_bytes"], seen["bytes"])
                seen["max_slots"] = max(seen["max_slots"], seen["slots"])
            time.sleep(rng.random() * 0.002)
            with lock:
                seen["bytes"] -= min(nb, 1000)
                seen["slots"] -= 1
            adm.release(slot, nb)
        done.append(i)

    threads = [threading.Thread(target=client, args=(i,)) for i in range(8)]
    for t in threads:
        t.start()
    for t in threads:
        t.join(timeout=30)
    assert len(done) == 8
    assert seen["max_bytes"] <= 1000 and seen["max_slots"] <= 3
    assert adm.in_use == 0 and adm.in_flight == 0 and len(adm.free_slots) == 3
    assert adm.peak_in_flight <= 3


def test_oversized_request_runs_alone():
    adm = AdmissionControl(slots=2, budget_bytes=100)
    s = adm.admit(10_000)
    assert adm.in_use == 100
    got = []
    t = threading.Thread(target=lambda: got.append(adm.admit(10)))
    t.start()
    time.sleep(0.05)
    assert not got  # waits while the oversized request holds the whole budget
    adm.release(s, 10_000)
    t.join(timeout=5)
    assert got and adm.in_use == 10


def test_footprint_and_arrivals():
    assert request_footprint(100_000, 64, 4) > request_footprint(100_000, 16, 4) > 100_000 * 12
    t = poisson_arrivals(200.0, 10.0, seed=4)
    assert 1700 < len(t) < 2300 and (t >= 0).all() and (t < 10.0).all()


class _FakeServerExt:
    """The pgeof_server_* bindings as NativeServer calls them, run on the CPU
    with the oracle: raw host pointers in, results written through them, a
    request's error raised by its wait. Checks NativeServer's own bookkeeping
    (in-flight table, results, resident-cloud ids, error propagation)."""

    def __init__(self):
        import itertools

        self.ids = itertools.count(1)
        self.pending, self.clouds, self.peak = {}, {}, 0

    @staticmethod
    def _view(ptr, shape, dtype):
        import ctypes

        import numpy as np

        n = int(np.prod(shape))
        ctype = ctypes.c_double if dtype == np.float64 else ctypes.c_float
        return np.ctypeslib.as_array((ctype * n).from_address(ptr)).reshape(shape)

    def _server_create(self, slots, budget):
        return 7

    def _server_submit(self, h, xyz_ptr, n, r, max_knn, ids, out_ptr, f64):
        import numpy as np

        dt = np.float64 if f64 else np.float32
        rid = next(self.ids)
        self.pending[rid] = (self._view(xyz_ptr, (n, 3), dt).copy(), r, max_knn, list(ids),
                             self._view(out_ptr, (n, len(ids)), dt))
        self.peak = max(self.peak, len(self.pending))
        return rid

    def _server_add_cloud(self, h, xyz_ptr, n, radius_hint, k_hint):
        import numpy as np

        cid = next(self.ids)
        self.clouds[cid] = self._view(xyz_ptr, (n, 3), np.float32).copy()
        return cid

    def _server_remove_cloud(self, h, cid):
        del self.clouds[cid]

    def _server_submit_resident(self, h, cid, r, max_knn, ids, out_ptr):
        import numpy as np

        xyz = self.clouds[cid]
        rid = next(self.ids)
        self.pending[rid] = (xyz, r, max_knn, list(ids), self._view(out_ptr, (xyz.shape[0], len(ids)), np.float32))
        self.peak = max(self.peak, len(self.pending))
        return rid

    def _server_wait(self, h, rid):
        import numpy as np

        from oracle import oracle

        xyz, r, max_knn, ids, out = self.pending.pop(rid)
        if not np.isfinite(xyz).all():
            raise ValueError("point coordinates must be finite")
        out[...] = oracle.compute_features_selected(xyz, r, max_knn, ids)
        return 0.5, 0.1, rid % 3

    def _server_stats(self, h):
        return 1 << 20, self.peak, 0

    def _server_destroy(self, h):
        assert not self.pending


def test_native_server_bookkeeping_on_host():
    import numpy as np
    import pytest

    from oracle import oracle
    from point_geometric_features_gb300.serving import NativeServer, Request
    from point_geometric_features_gb300.synthetic import uniform_cube

    clouds = [uniform_cube(n, seed=60 + n) for n in (300, 500, 800)]
    ext = _FakeServerExt()
    server = NativeServer(slots=3, budget_bytes=1 << 30, _ext=ext)
    feats = [0, 3, 10, 13]
    reqs = [Request(0, clouds[0], 16, 0.2, feats), Request(1, clouds[1].astype(np.float64), 32, 0.25, feats)]
    bad = clouds[2].copy()
    bad[5, 1] = np.inf
    reqs.append(Request(2, bad, 16, 0.2, feats))
    cid = server.add_cloud(clouds[2], radius_hint=0.2)
    reqs.append(Request(3, None, 8, 0.15, [1, 2], cloud=cid))
    for r in reqs:
        server.submit(r)
    with pytest.raises(ValueError, match="finite"):
        server.drain(len(reqs))
    res = {r.rid: r for r in server.drain(len(reqs))}
    assert sorted(res) == [0, 1, 3]
    np.testing.assert_array_equal(res[0].features, oracle.compute_features_selected(clouds[0], 0.2, 16, feats))
    assert res[1].features.dtype == np.float64
    np.testing.assert_array_equal(res[1].features,
                                  oracle.compute_features_selected(clouds[1].astype(np.float64), 0.25, 32, feats))
    np.testing.assert_array_equal(res[3].features, oracle.compute_features_selected(clouds[2], 0.15, 8, [1, 2]))
    assert res[3].n_points == clouds[2].shape[0]
    for r in res.values():
        assert r.done >= r.admitted >= r.arrival and r.latency_ms == pytest.approx(0.5)
    assert server.adm.peak_in_flight == 4 and server.adm.peak_bytes == 1 << 20
    server.remove_cloud(cid)
    with pytest.raises(ValueError, match="unknown resident cloud"):
        server.submit(Request(9, None, 8, 0.1, [1], cloud=cid))
    server.close()
