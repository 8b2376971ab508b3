"""Request serving for compute_features_selected (include/pgeof.hpp:325-375).

Continuous batching: a request is admitted as soon as a slot (a CUDA stream
with its own host worker) and enough of the device-memory budget are free, so
requests that arrive while others run on the GPU start right away and their
kernels overlap on the device. Each admitted request is copied in, processed
by the GB300 path (radius grid, fused radius search, PCA, selected features)
and copied back on its slot's stream; its latency is measured from arrival to
result. Results do not depend on what else is in flight (every kernel is
deterministic and requests share nothing but the memory pool).

The reference has no serving layer; this module is the host-side scheduler
around the library's device entry points.
"""

from __future__ import annotations

import collections
import queue
import threading
import time
from dataclasses import dataclass

import numpy as np

__all__ = ["Request", "Result", "AdmissionControl", "Server", "NativeServer", "request_footprint",
           "radius_for_count"]


@dataclass
class Request:
    rid: int
    xyz: np.ndarray  # float32 (n, 3), host
    max_knn: int
    radius: float
    features: list
    arrival: float = 0.0  # time.perf_counter() at arrival
    cloud: int = 0  # NativeServer: id of a resident cloud (add_cloud) to run on instead of xyz


@dataclass
class Result:
    rid: int
    features: np.ndarray
    arrival: float
    admitted: float
    done: float
    n_points: int
    slot: int

    @property
    def latency_ms(self) -> float:
        return (self.done - self.arrival) * 1e3


def request_footprint(n_points: int, max_knn: int, n_features: int) -> int:
    """Upper bound of the device bytes one request holds while in flight:
    input (12 B/pt), cell-sorted copy (16), grid build (4 x 4 + cells 4 x 5),
    neighbour table (4 * max_knn), counts (4), output (4 * n_features)."""
    per_point = 12 + 16 + 16 + 20 + 4 * max(int(max_knn), 1) + 4 + 4 * int(n_features)
    return int(n_points) * per_point + (1 << 20)


def radius_for_count(xyz: np.ndarray, count: float) -> float:
    """Radius whose disc holds ~`count` points at the cloud's mean surface
    density (LiDAR-like clouds are dominated by 2D surfaces)."""
    ext = np.ptp(xyz, axis=0).astype(np.float64)
    area = max(float(np.sort(ext)[-1] * np.sort(ext)[-2]), 1e-12)
    density = xyz.shape[0] / area
    return float(np.sqrt(count / (np.pi * density)))


class AdmissionControl:
    """Slots plus a device-memory byte budget; admit() blocks until a slot is
    free and the request's footprint fits next to what is in flight."""

    def __init__(self, slots: int, budget_bytes: int):
        self.budget = int(budget_bytes)
        self.in_use = 0
        self.in_flight = 0
        self.free_slots = collections.deque(range(slots))
        self.cv = threading.Condition()
        self.peak_bytes = 0
        self.peak_in_flight = 0

    def admit(self, nbytes: int, stop: threading.Event | None = None) -> int:
        nbytes = min(int(nbytes), self.budget)  # a request larger than the budget runs alone
        with self.cv:
            while not (self.free_slots and self.in_use + nbytes <= self.budget):
                if stop is not None and stop.is_set():
                    return -1
                self.cv.wait(timeout=0.05)
            self.in_use += nbytes
            self.in_flight += 1
            self.peak_bytes = max(self.peak_bytes, self.in_use)
            self.peak_in_flight = max(self.peak_in_flight, self.in_flight)
            return self.free_slots.popleft()

    def release(self, slot: int, nbytes: int) -> None:
        nbytes = min(int(nbytes), self.budget)
        with self.cv:
            self.in_use -= nbytes
            self.in_flight -= 1
            self.free_slots.append(slot)
            self.cv.notify_all()


class Server:
    """Admits requests from submit() into `slots` concurrent GPU slots within
    `budget_bytes` of device memory and runs each through
    compute_features_selected on its slot's stream."""

    def __init__(self, slots: int = 8, budget_bytes: int = 40 << 30, device: int = 0):
        import torch

        import point_geometric_features_gb300 as pgeof

        self.torch = torch
        self.pgeof = pgeof
        self.device = torch.device("cuda", device)
        self.adm = AdmissionControl(slots, budget_bytes)
        self.streams = [torch.cuda.Stream(device=self.device) for _ in range(slots)]
        self.pending: queue.Queue = queue.Queue()
        self.results: list[Result] = []
        self.lock = threading.Lock()
        self.stop = threading.Event()
        self.workers = [threading.Thread(target=self._worker, daemon=True) for _ in range(slots)]
        self.dispatcher = threading.Thread(target=self._dispatch, daemon=True)
        self.slot_queues = [queue.Queue() for _ in range(slots)]
        for i, w in enumerate(self.workers):
            w._slot = i  # noqa: SLF001
        self.dispatcher.start()
        for w in self.workers:
            w.start()

    # ---------------------------------------------------------------- public
    def submit(self, req: Request) -> None:
        if not req.arrival:
            req.arrival = time.perf_counter()
        self.pending.put(req)

    def drain(self, n_expected: int, timeout: float = 600.0) -> list[Result]:
        t0 = time.perf_counter()
        while True:
            with self.lock:
                if len(self.results) >= n_expected:
                    return list(self.results)
            if time.perf_counter() - t0 > timeout:
                raise TimeoutError(f"only {len(self.results)} of {n_expected} requests finished")
            time.sleep(0.002)

    def close(self) -> None:
        """Stop admitting, let in-flight requests finish, join every thread."""
        self.stop.set()
        for q in self.slot_queues:
            q.put(None)
        self.pending.put(None)
        for t in [self.dispatcher, *self.workers]:
            t.join(timeout=60)
        for s in self.streams:
            s.synchronize()

    # ---------------------------------------------------------------- internals
    def _dispatch(self) -> None:
        while not self.stop.is_set():
            req = self.pending.get()
            if req is None:
                return
            nbytes = request_footprint(req.xyz.shape[0], req.max_knn, len(req.features))
            slot = self.adm.admit(nbytes, self.stop)
            if slot < 0:
                return
            self.slot_queues[slot].put((req, nbytes, time.perf_counter()))

    def _worker(self) -> None:
        torch = self.torch
        slot = threading.current_thread()._slot  # noqa: SLF001
        stream = self.streams[slot]
        q = self.slot_queues[slot]
        torch.cuda.set_device(self.device)
        while True:
            item = q.get()
            if item is None:
                return
            req, nbytes, admitted = item
            try:
                with torch.cuda.stream(stream):
                    host = torch.from_numpy(req.xyz).pin_memory()
                    xyz = host.to(self.device, non_blocking=True)
                    out = self.pgeof.compute_features_selected(xyz, req.radius, req.max_knn, req.features)
                    res = torch.empty(out.shape, dtype=out.dtype, pin_memory=True)
                    res.copy_(out, non_blocking=True)
                stream.synchronize()
                feats = res.numpy()
            finally:
                self.adm.release(slot, nbytes)
            with self.lock:
                self.results.append(Result(req.rid, feats, req.arrival, admitted, time.perf_counter(),
                                           req.xyz.shape[0], slot))


class _NativePeaks:
    """peak_bytes / peak_in_flight of a NativeServer, read from the library."""

    def __init__(self, server):
        self._server = server

    @property
    def peak_bytes(self) -> int:
        return int(self._server._stats()[0])

    @property
    def peak_in_flight(self) -> int:
        return int(self._server._stats()[1])


class NativeServer:
    """The same continuous-batching server as ``Server``, run by the library
    itself (pgeof_server_*: C++ worker threads, one CUDA stream each, FIFO
    admission within the device-memory budget): no Python on the request path.
    submit() enqueues the request with its host arrays; drain() waits for the
    results, whose latencies the library timestamps."""

    def __init__(self, slots: int = 8, budget_bytes: int = 40 << 30, device: int = 0, _ext=None):
        if _ext is not None:  # a stand-in for the library's bindings (host-logic tests)
            self._ext = _ext
            self._h = _ext._server_create(int(slots), int(budget_bytes))
        else:
            import torch

            from . import pgeof_ext

            self._ext = pgeof_ext
            with torch.cuda.device(device):
                self._h = pgeof_ext._server_create(int(slots), int(budget_bytes))
        self._inflight: dict = {}  # request id -> (Request, xyz, output array), kept alive until waited on
        self._clouds: dict = {}  # resident cloud id -> point count
        self.results: list[Result] = []
        self.adm = _NativePeaks(self)

    def _stats(self):
        return self._ext._server_stats(self._h)

    def add_cloud(self, xyz: np.ndarray, radius_hint: float = 0.0, k_hint: int = 16) -> int:
        """Keep a float32 cloud and its grid on the device for repeated
        requests (Request(cloud=id)); returns its id. Its bytes are reserved
        from the budget until remove_cloud()."""
        xyz = np.ascontiguousarray(xyz, dtype=np.float32)
        if xyz.ndim != 2 or xyz.shape[1] != 3:
            raise TypeError("xyz must be a (n, 3) array")
        cid = self._ext._server_add_cloud(self._h, xyz.ctypes.data, xyz.shape[0], float(radius_hint), int(k_hint))
        self._clouds[cid] = xyz.shape[0]
        return cid

    def remove_cloud(self, cid: int) -> None:
        """Refuse new requests on the cloud, wait for its queued ones, free it."""
        self._ext._server_remove_cloud(self._h, int(cid))
        self._clouds.pop(int(cid), None)

    def submit(self, req: Request) -> None:
        if not req.arrival:
            req.arrival = time.perf_counter()
        if req.cloud:
            ids = [int(v) for v in req.features]
            n = self._clouds.get(int(req.cloud))
            if n is None:
                raise ValueError("unknown resident cloud id")
            out = np.zeros((n, len(ids)), np.float32)
            rid = self._ext._server_submit_resident(self._h, int(req.cloud), float(req.radius), int(req.max_knn),
                                                    ids, out.ctypes.data)
            self._inflight[rid] = (req, np.empty((n, 0), np.float32), out)
            return
        xyz = np.ascontiguousarray(req.xyz)
        f64 = xyz.dtype == np.float64
        if not f64 and xyz.dtype != np.float32:
            raise TypeError("xyz must be float32 or float64")
        ids = [int(v) for v in req.features]
        out = np.zeros((xyz.shape[0], len(ids)), xyz.dtype)
        rid = self._ext._server_submit(self._h, xyz.ctypes.data, xyz.shape[0], float(req.radius), int(req.max_knn),
                                       ids, out.ctypes.data, f64)
        self._inflight[rid] = (req, xyz, out)

    def drain(self, n_expected: int | None = None, timeout: float = 600.0) -> list[Result]:
        for rid in sorted(self._inflight):
            req, xyz, out = self._inflight.pop(rid)
            lat, qms, slot = self._ext._server_wait(self._h, rid)
            self.results.append(Result(req.rid, out, req.arrival, req.arrival + qms / 1e3,
                                       req.arrival + lat / 1e3, xyz.shape[0], slot))
        return list(self.results)

    def close(self) -> None:
        if getattr(self, "_h", 0):
            self._ext._server_destroy(self._h)
            self._h = 0

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def summarize(results: list[Result], wall_s: float) -> dict:
    lat = np.array([r.latency_ms for r in results])
    pts = sum(r.n_points for r in results)
    wait = np.array([(r.admitted - r.arrival) * 1e3 for r in results])
    return {
        "requests": len(results),
        "p50_ms": float(np.percentile(lat, 50)) if len(lat) else None,
        "p99_ms": float(np.percentile(lat, 99)) if len(lat) else None,
        "mean_ms": float(lat.mean()) if len(lat) else None,
        "admission_wait_p99_ms": float(np.percentile(wait, 99)) if len(wait) else None,
        "points": int(pts),
        "points_per_s": pts / wall_s if wall_s > 0 else None,
        "wall_s": wall_s,
    }


def poisson_arrivals(rate: float, duration: float, seed: int) -> np.ndarray:
    rng = np.random.default_rng(seed)
    t, out = 0.0, []
    while True:
        t += rng.exponential(1.0 / rate)
        if t >= duration:
            return np.array(out)
        out.append(t)


def run_stream(server: Server, pool: list, rate: float, duration: float, seed: int, ks=(16, 32, 64),
               features=None, clouds=None) -> dict:
    """Replay a Poisson stream of requests drawn from `pool` (list of float32
    clouds) against `server`; returns the latency / throughput summary.
    `clouds` (NativeServer): resident cloud ids parallel to `pool`, so that the
    requests run on the resident copies."""
    import point_geometric_features_gb300 as pgeof

    features = features or [pgeof.Verticality, pgeof.Curvature, pgeof.Planarity, pgeof.Normal_z]
    rng = np.random.default_rng(seed + 1)
    times = poisson_arrivals(rate, duration, seed)
    reqs = []
    for i, _t in enumerate(times):
        j = int(rng.integers(len(pool)))
        xyz = pool[j]
        k = int(rng.choice(ks))
        reqs.append(Request(i, xyz, k, radius_for_count(xyz, 1.5 * k), features,
                            cloud=int(clouds[j]) if clouds is not None else 0))
    t0 = time.perf_counter()
    for req, t in zip(reqs, times):
        now = time.perf_counter() - t0
        if t > now:
            time.sleep(t - now)
        req.arrival = t0 + t
        server.submit(req)
    results = server.drain(len(reqs))
    wall = max(r.done for r in results) - t0
    out = summarize(results, wall)
    out["peak_in_flight_bytes"] = server.adm.peak_bytes
    out["peak_in_flight_requests"] = server.adm.peak_in_flight
    return out
