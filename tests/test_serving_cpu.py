"""Serving configuration, host side: the seeded request stream, the FIFO latency recursion and the
footprint model (vh_schur_analyze needs no GPU)."""
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
            assert serving.footprint_bytes(prob, len(w.freqs)) > 0


def test_fifo_latencies_match_an_event_simulation():
    rng = np.random.default_rng(2)
    s = rng.uniform(0.1, 2.0, 200)
    arr = serving.poisson_arrivals(200, 0.8 / s.mean())
    lat = serving.fifo_latencies(s, arr)
    # event simulation: the server takes requests in arrival order when it is free
    t, sim = 0.0, []
    for a, d in zip(arr, s):
        t = max(t, a) + d
        sim.append(t - a)
    np.testing.assert_allclose(lat, sim, rtol=0, atol=1e-12)
    assert np.all(lat >= s - 1e-12)
    summ = serving.summarize({"service_s": s, "freq_points": np.full(200, 8), "converged": np.ones(200, bool)})
    assert summ["p99_latency_s"] >= summ["p50_latency_s"] > 0
