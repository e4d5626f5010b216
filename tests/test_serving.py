"""Serving loop: admission by device-memory footprint and FIFO order (host
logic, with a fake runner), and the CUDA runner against direct calls."""
import threading
import time

import numpy as np
import pytest

from variantdbscan_gb300 import serving as sv


def _reqs(k=12, seed=0):
    rng = np.random.default_rng(seed)
    out = []
    t = 0.0
    for i in range(k):
        t += rng.exponential(1.0)
        n = int(rng.integers(100, 2000))
        out.append(sv.Request(t, rng.uniform(0, 10, n), rng.uniform(0, 10, n),
                              np.array([0.5, 1.0]), np.array([4, 8], np.uint32)))
    return out


class FakeRunner:
    """Sleeps in proportion to the request size and records overlaps."""
    active = 0
    peak = 0
    lock = threading.Lock()
    log = []

    def __init__(self, table_budget):
        self.table_budget = table_budget

    def __call__(self, req):
        with FakeRunner.lock:
            FakeRunner.active += 1
            FakeRunner.peak = max(FakeRunner.peak, FakeRunner.active)
            FakeRunner.log.append(req.arrival)
        time.sleep(1e-6 * req.n)
        with FakeRunner.lock:
            FakeRunner.active -= 1
        return np.zeros((len(req.eps), req.n), np.uint32)


def _reset():
    FakeRunner.active = FakeRunner.peak = 0
    FakeRunner.log = []


def test_all_requests_served_in_arrival_order():
    _reset()
    reqs = _reqs()
    srv = sv.Server(FakeRunner, workers=3, hbm_budget=1 << 40, table_budget=1 << 20)
    res = srv.serve(reqs, rate=2000.0)
    assert not res.errors and len(res.latencies) == len(reqs)
    assert np.all(res.latencies >= 0)
    adm = [r.admitted for r in sorted(reqs, key=lambda r: r.arrival)]
    assert adm == sorted(adm)
    assert res.throughput > 0 and res.percentile_ms(99) >= res.percentile_ms(50)


def test_budget_admits_one_request_at_a_time():
    _reset()
    reqs = _reqs()
    tb = 1 << 20
    biggest = max(sv.footprint(r, tb) for r in reqs)
    srv = sv.Server(FakeRunner, workers=4, hbm_budget=biggest, table_budget=tb)
    res = srv.serve(reqs, rate=float("inf"))
    assert res.peak_footprint <= biggest
    assert FakeRunner.peak == 1  # the footprints never allow two in flight


def test_budget_bounds_the_footprint_in_flight():
    _reset()
    reqs = _reqs(20, seed=3)
    tb = 1 << 20
    budget = 3 * max(sv.footprint(r, tb) for r in reqs)
    srv = sv.Server(FakeRunner, workers=8, hbm_budget=budget, table_budget=tb)
    res = srv.serve(reqs, rate=float("inf"))
    assert res.peak_footprint <= budget
    assert 1 <= FakeRunner.peak <= 3


def test_request_larger_than_the_budget_is_rejected():
    reqs = _reqs(2)
    srv = sv.Server(FakeRunner, workers=1, hbm_budget=1000, table_budget=0)
    with pytest.raises(ValueError):
        srv.serve(reqs, rate=1.0)


@pytest.mark.gpu
def test_served_labels_match_direct_calls():
    import variantdbscan_gb300 as v
    from variantdbscan_gb300 import synthetic as syn
    stream = syn.request_stream(count=6, seed=4, n_lo=5000, n_hi=40000)
    reqs = sv.requests_from(stream)
    srv = sv.Server(sv.library_runner_factory(), workers=3, hbm_budget=8 << 30)
    bpp, base = srv.calibrate(reqs)
    assert 0 <= bpp < 2000 and 0 < base < (1 << 30)  # measured index bytes
    res = srv.serve(reqs, rate=float("inf"))
    assert not res.errors
    # every request's measured footprint within its admission estimate
    assert 0 < res.footprint_ratio <= 1.0
    ctx = v.Context()
    for r in reqs:
        want, _ = ctx.run([v.BatchItem(r.x, r.y, r.eps, r.minpts)])
        np.testing.assert_array_equal(r.labels, want[0])
    ctx.close()


def test_calibration_sets_the_per_point_footprint():
    class Measuring:
        def __init__(self, table_budget):
            pass

        def __call__(self, r):
            # 120 bytes per point of index, a table of 1 MB, the labels
            r.device_bytes = 120 * r.n + (1 << 20) + 4 * r.variant_points
            r.table_bytes = 1 << 20
            return np.zeros((len(r.eps), r.n), np.uint32)

    reqs = _reqs(4)
    srv = sv.Server(Measuring, workers=2, hbm_budget=1 << 40, table_budget=1 << 20)
    bpp, base = srv.calibrate(reqs)
    assert bpp == pytest.approx(120.0) and base <= 1
    assert abs(srv.footprint(reqs[0]) - (120 * reqs[0].n + 4 * reqs[0].variant_points
                                         + (1 << 20))) <= 2
    res = srv.serve(reqs, rate=float("inf"))
    assert res.footprint_ratio == pytest.approx(1.0)
