"""Serving loop host logic: the request stream, arrival-order service with
queueing, admission by footprint, warm starts and the latency report, with a
fake solver and a fake clock."""
import numpy

from kelvin_gb300 import serve


def test_request_stream_is_seeded_and_in_range():
    a = serve.request_stream(200, rate=20.0, seed=3)
    b = serve.request_stream(200, rate=20.0, seed=3)
    assert [(r.arrival, r.kind, r.params, r.theta, r.ng) for r in a] == \
        [(r.arrival, r.kind, r.params, r.theta, r.ng) for r in b]
    t = numpy.array([r.arrival for r in a])
    assert (numpy.diff(t) > 0).all()
    assert 5.0 < t[-1] < 15.0                       # ~200 / 20 s
    for r in a:
        assert 0.1 <= r.theta <= 4.0 and r.ng in (10, 20, 40)
        if r.kind == 'ueg':
            assert (r.params[0], r.params[1]) in serve.UEG_SHAPES and 1 <= r.params[2] <= 4
        else:
            assert 8 <= r.params[0] <= 16 and 1 <= r.params[1] <= 8
    kinds = {r.kind for r in a}
    assert kinds == {'ueg', 'hubbard'}


class FakeClock(object):
    def __init__(self):
        self.t = 0.0

    def __call__(self):
        return self.t

    def sleep(self, dt):
        self.t += dt


def test_service_order_latency_admission_and_warm_starts():
    clock = FakeClock()
    R = serve.Request
    reqs = [R(0, 0.0, 'ueg', (14, 19, 4.0), 0.5, 10),
            R(1, 0.1, 'ueg', (14, 19, 4.0), 1.0, 10),      # same system and grid: warm
            R(2, 0.2, 'hubbard', (16, 4.0), 0.3, 40),      # too big: rejected
            R(3, 5.0, 'ueg', (38, 33, 2.0), 0.2, 20)]      # arrives after the queue drains
    calls = []

    def solve(r, warm):
        calls.append((r.rid, warm is not None))
        clock.t += 1.0                                     # every solve takes 1 s
        return -0.01 * r.rid, (numpy.zeros(4), numpy.zeros(8))

    def footprint(r):
        return 10 if r.kind == 'ueg' else 1000

    srv = serve.Server(solve=solve, footprint=footprint, budget=100, clock=clock,
                       sleep=clock.sleep)
    rep = srv.serve(reqs)
    assert calls == [(0, False), (1, True), (3, False)]
    assert rep["solves"] == 3 and rep["rejected"] == 1 and rep["warm_started"] == 1
    by = {d["rid"]: d for d in rep["requests"]}
    assert by[0]["end"] == 1.0 and by[1]["start"] == 1.0 and by[1]["end"] == 2.0
    assert by[3]["start"] == 5.0 and by[3]["end"] == 6.0   # waited for its arrival
    lat = numpy.array([1.0, 1.9, 1.0]) * 1e3
    assert abs(rep["p50_ms"] - numpy.percentile(lat, 50)) < 1e-9
    assert abs(rep["p99_ms"] - numpy.percentile(lat, 99)) < 1e-9
    assert abs(rep["solves_per_s"] - 3 / 6.0) < 1e-12


def test_default_footprint_is_the_solver_footprint():
    """Admission uses kvft_solver_footprint (host arithmetic, no device): it
    grows with the spin orbitals and the grid, and a budget below every
    request's footprint rejects the whole stream without solving."""
    reqs = serve.request_stream(12, rate=20.0, seed=1)
    srv = serve.Server(budget=1 << 20, solve=lambda r, w: (_ for _ in ()).throw(AssertionError),
                       clock=FakeClock(), sleep=lambda dt: None)
    small = serve.Request(0, 0.0, 'ueg', (14, 19, 1.0), 1.0, 10)
    big = serve.Request(1, 0.0, 'ueg', (38, 57, 1.0), 1.0, 10)
    wide = serve.Request(2, 0.0, 'ueg', (38, 57, 1.0), 1.0, 40)
    assert srv.footprint(small) < srv.footprint(big) < srv.footprint(wide)
    assert srv.footprint(big) > 8 * 114 ** 4 * 10
    rep = srv.serve(reqs)
    assert rep["solves"] == 0 and rep["rejected"] == 12 and rep["p50_ms"] is None
