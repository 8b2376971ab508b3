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
