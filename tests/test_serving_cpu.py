"""Serving configuration, host side: the seeded request stream, the footprint model and the
continuous-batching scheduler (with a host-only stand-in for the device work)."""
import threading
import time

import numpy as np

from voxhenry_gb300 import serving, structure


def test_request_stream_is_seeded_and_valid():
    a = serving.request_stream(40)
    b = serving.request_stream(40)
    assert [r.workload.sigma_e.shape for r in a] == [r.workload.sigma_e.shape for r in b]
    kinds = {r.kind for r in a}
    assert kinds == {"bar", "cylinder", "spiral"}
    for r in a[:12]:
        w = r.workload
        assert 1 <= len(w.freqs) <= 64 and 1 <= len(w.pnt_lft) <= 4
        assert 0.5e-6 <= w.dx <= 2e-6 and 3.5e7 <= w.sigma_e.max() <= 5.8e7
        if w.sigma_e.size < 4e5:
            prob = structure.build_problem(w.sigma_e, w.lambdaL, w.dx, w.pnt_lft, w.pnt_rght,
                                           tensor=(np.zeros(1), np.zeros(3)))
            assert prob.rhs.shape[1] == len(w.pnt_lft)
            assert np.all(np.abs(prob.rhs).sum(axis=0) > 0)          # every port excites the structure
            exact = serving.footprint_bytes(prob, len(w.freqs))
            est = serving.footprint_estimate(w, len(w.freqs))
            assert 0.5 * exact < est < 3 * exact     # the admission estimate, before the exact one is known


def test_fifo_latencies_match_an_event_simulation():
    rng = np.random.default_rng(2)
    s = rng.uniform(0.1, 2.0, 200)
    arr = serving.poisson_arrivals(200, 0.8 / s.mean())
    lat = serving.fifo_latencies(s, arr)
    t, sim = 0.0, []
    for a, d in zip(arr, s):
        t = max(t, a) + d
        sim.append(t - a)
    np.testing.assert_allclose(lat, sim, rtol=0, atol=1e-12)
    assert np.all(lat >= s - 1e-12)


class FakeSlot:
    def __init__(self, index):
        self.index = index
        self.key = None

    def drop(self):
        self.key = None

    def close(self):
        pass


class FakeDevice:
    """Stands in for the GPU work: sleeps in proportion to the frequency points and records how many
    requests and how many footprint bytes were in flight."""

    def __init__(self, sec_per_point=0.004):
        self.lock = threading.Lock()
        self.running = 0
        self.bytes = 0
        self.peak = 0
        self.peak_bytes = 0
        self.sec = sec_per_point

    def solve(self, slot, req, rec, budget, reserve):
        w = req.workload
        need = min(budget, serving.footprint_estimate(w, len(w.freqs)))
        reserve(need)
        key = serving.geometry_key(w)
        rec.reused_geometry = slot.key == key
        slot.key = key
        with self.lock:
            self.running += 1
            self.bytes += need
            self.peak = max(self.peak, self.running)
            self.peak_bytes = max(self.peak_bytes, self.bytes)
        time.sleep(self.sec * len(w.freqs))
        with self.lock:
            self.running -= 1
            self.bytes -= need
        rec.R = rec.L = np.zeros((len(w.freqs), 1, 1))
        rec.flags = np.zeros(len(w.freqs), dtype=np.int32)
        rec.freq_points = len(w.freqs)


def small_requests(n):
    return [r for r in serving.request_stream(4 * n) if r.workload.sigma_e.size < 1.5e5][:n]


def test_scheduler_overlaps_requests_and_keeps_arrival_order():
    reqs = small_requests(12)
    dev = FakeDevice()
    srv = serving.Server(slots=3, budget_bytes=1 << 50, solve=dev.solve, slot_factory=FakeSlot)
    recs = srv.run(reqs)                        # all arrive at once
    assert len(recs) == 12 and all(r.error is None for r in recs)
    assert dev.peak == 3 and srv.max_in_flight == 3
    starts = [r.start for r in recs]
    assert starts == sorted(starts)             # admitted first come, first served
    assert all(r.latency >= r.finish - r.start for r in recs)
    s = serving.summarize_run(recs)
    assert s["all_converged"] and s["p99_latency_s"] >= s["p50_latency_s"] > 0


def test_scheduler_admits_by_memory_footprint():
    """With a budget that holds only the largest request alone, the bytes in flight never exceed it."""
    reqs = small_requests(10)
    needs = [serving.footprint_estimate(r.workload, len(r.workload.freqs)) for r in reqs]
    budget = max(needs)
    dev = FakeDevice()
    srv = serving.Server(slots=4, budget_bytes=budget, solve=dev.solve, slot_factory=FakeSlot)
    recs = srv.run(reqs)
    assert len(recs) == 10
    assert dev.peak_bytes <= budget
    assert dev.peak >= 2 if sorted(needs)[0] + sorted(needs)[1] <= budget else dev.peak == 1


def test_scheduler_replays_arrivals_and_reuses_geometries():
    reqs = small_requests(4)
    rep = serving.Request(99, reqs[0].kind, reqs[0].workload)   # the same geometry again, later
    reqs = reqs + [rep]
    arr = np.array([0.0, 0.01, 0.02, 0.03, 0.5])
    dev = FakeDevice(sec_per_point=0.001)
    srv = serving.Server(slots=4, budget_bytes=1 << 50, solve=dev.solve, slot_factory=FakeSlot)
    t0 = time.perf_counter()
    recs = srv.run(reqs, arr)
    assert time.perf_counter() - t0 >= 0.5
    assert all(r.start >= r.arrival - 1e-6 for r in recs)
    assert recs[-1].reused_geometry and recs[-1].slot == recs[0].slot
