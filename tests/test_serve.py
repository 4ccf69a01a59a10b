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


class FakeBackend(object):
    """Solves whose energy after k sweeps of a phase is known: a request
    converges after `sweeps[rid]` sweeps of its last phase (earlier phases
    stall at once); a round of sweeps takes 1 s of the fake clock whatever
    the number of active solves (their work overlaps)."""

    def __init__(self, clock, footprints, sweeps):
        self.clock = clock
        self.fp = footprints
        self.sweeps = sweeps
        self.opened, self.open_now, self.max_open = [], 0, 0
        self.begun = set()

    def mem_total(self):
        return 1000

    def footprint(self, req, precision):
        return self.fp[req.rid]

    def open(self, sv, warm):
        self.opened.append((sv.req.rid, None if warm is None else float(warm[0][0])))
        self.open_now += 1
        self.max_open = max(self.max_open, self.open_now)
        sv.handle = {"k": 0}

    def begin(self, sv, damp):
        if not self.begun:
            self.clock.t += 1.0
        self.begun.add(sv.req.rid)

    def end(self, sv):
        self.begun.discard(sv.req.rid)
        h = sv.handle
        h["k"] += 1
        last = sv.phase == len(sv.levels) - 1
        if not last:
            return -1.0, 1.0                        # no progress: stalls after 3 sweeps
        left = self.sweeps[sv.req.rid] - sv.it_phase
        return -0.01 * sv.req.rid - (1e-3 if left > 1 else 0.0), 1e-9

    def close(self, sv, keep):
        self.open_now -= 1
        amps = (numpy.array([sv.req.theta]), numpy.array([float(sv.req.rid)]))
        return sv.omega_cc, amps if keep else None


def test_continuous_batching_admission_overlap_and_warm_starts():
    clock = FakeClock()
    R = serve.Request
    reqs = [R(0, 0.0, 'ueg', (14, 19, 4.0), 0.5, 10),
            R(1, 0.5, 'ueg', (14, 19, 4.0), 2.0, 10),      # admitted while 0 runs
            R(2, 0.6, 'hubbard', (16, 4.0), 0.3, 40),      # too big for the device
            R(3, 0.7, 'ueg', (38, 33, 2.0), 0.2, 20),      # waits for memory
            R(4, 40.0, 'ueg', (14, 19, 4.0), 0.6, 10)]     # warm: nearest of 0.5, 2.0
    fp = {0: 300, 1: 300, 2: 2000, 3: 500, 4: 300}
    be = FakeBackend(clock, fp, {0: 4, 1: 6, 3: 2, 4: 2})
    srv = serve.Server(precision='mixed', slots=3, budget=900, backend=be, clock=clock,
                       sleep=clock.sleep)
    rep = srv.serve(reqs)
    by = {d["rid"]: d for d in rep["requests"]}
    assert not by[2]["ok"] and "budget" in by[2]["reason"]
    assert rep["solves"] == 4 and rep["rejected"] == 1
    # 0 and 1 run together; 3 needs 500 more than the 600 they hold, so it
    # starts only when 0 has finished
    assert be.max_open == 2 and rep["max_active"] == 2
    assert by[1]["start"] < by[0]["end"]
    assert by[3]["start"] >= by[0]["end"]
    # few-digit phases stall after 3 sweeps each (3 and 5 levels), then the
    # last phase needs the request's sweeps plus Kelvin's second energy
    assert by[0]["iterations"] == 3 + 3 + 4 and by[0]["converged"]
    # warm start of 4 from the kept solve at the nearest temperature (0.5)
    assert be.opened[-1] == (4, 0.5) and by[4]["warm"]
    assert abs(by[4]["omega_cc"] - (-0.04)) < 1e-15
    lat = [by[r]["end"] - by[r]["arrival"] for r in (0, 1, 3, 4)]
    assert abs(rep["p50_ms"] - numpy.percentile(numpy.array(lat) * 1e3, 50)) < 1e-9


def test_default_footprint_is_the_solver_footprint():
    """Admission uses kvft_solver_footprint (host arithmetic, no device) plus
    the slot's workspace cap: it grows with the spin orbitals and the grid,
    and a budget below every request's footprint rejects the whole stream
    without solving."""
    from kelvin_gb300 import _lib
    be = serve.DeviceBackend.__new__(serve.DeviceBackend)
    be.workspace_bytes = 1 << 30
    be.accel = 0
    small = serve.Request(0, 0.0, 'ueg', (14, 19, 1.0), 1.0, 10)
    big = serve.Request(1, 0.0, 'ueg', (38, 57, 1.0), 1.0, 10)
    wide = serve.Request(2, 0.0, 'ueg', (38, 57, 1.0), 1.0, 40)
    f = lambda r: be.footprint(r, 'mixed')
    assert f(small) < f(big) < f(wide)
    assert f(big) > 8 * 114 ** 4 * 10 + (1 << 30)
    assert f(small) == _lib.lib().kvft_solver_footprint(38, 10, _lib.PREC_MIXED) + (1 << 30)
    # with Anderson mixing of depth 3: seven FP32 arrays over T1 and the
    # spin-conserving elements of T2
    be.accel = 3
    assert f(small) == _lib.lib().kvft_solver_footprint(38, 10, _lib.PREC_MIXED) + (1 << 30) \
        + 4 * 7 * 10 * (38 * 38 + 6 * 19 ** 4)
    be.accel = 0

    class NoSolve(FakeBackend):
        def footprint(self, req, precision):
            return f(req)

        def open(self, sv, warm):
            raise AssertionError("nothing fits")
    reqs = serve.request_stream(12, rate=20.0, seed=1)
    clock = FakeClock()
    srv = serve.Server(budget=1 << 20, backend=NoSolve(clock, {}, {}), clock=clock,
                       sleep=clock.sleep)
    rep = srv.serve(reqs)
    assert rep["solves"] == 0 and rep["rejected"] == 12 and rep["p50_ms"] is None


class CutBackend(FakeBackend):
    """The few-digit phase's residual falls by 10x a sweep from 1 (so a cut at
    1e-2 ends it after three sweeps); records the mixing factor it is given."""

    def begin(self, sv, damp):
        self.damps = getattr(self, "damps", set()) | {damp}
        FakeBackend.begin(self, sv, damp)

    def end(self, sv):
        if sv.phase < len(sv.levels) - 1:
            self.begun.discard(sv.req.rid)
            return -1.0, 10.0 ** -(sv.it_phase + 1)
        return FakeBackend.end(self, sv)


def test_accelerated_scheme_phases():
    """With accel the mixed form goes from 3 digit levels straight to the
    6-level refinement (as ccsd.ccsd), the few-digit phase ends at the
    residual cut, and the solves step with the mixing factor's damp = 1 - mix."""
    clock = FakeClock()
    R = serve.Request
    reqs = [R(0, 0.0, 'ueg', (14, 19, 4.0), 0.5, 10)]
    be = CutBackend(clock, {0: 100}, {0: 4})
    srv = serve.Server(precision='mixed', slots=2, budget=900, backend=be, clock=clock,
                       sleep=clock.sleep, accel=3, mix=0.7, low_tconv=1e-2)
    assert srv.levels == (3, 6)
    rep = srv.serve(reqs)
    d = rep["requests"][0]
    # the cut ends the few-digit phase at its third sweep (1e-3 < 1e-2; a
    # stall would take four); the fake's last phase meets Kelvin's test at
    # its second sweep (an unchanged energy)
    assert d["ok"] and d["converged"] and d["iterations"] == 3 + 2
    assert be.damps == {1.0 - 0.7}
    assert serve.Server(precision='mixed', accel=3, refine_digits=7).levels == (3, 7)
    # without accel: Kelvin's damping and the 3, 5, 7 ladder
    srv = serve.Server(precision='mixed', slots=2, budget=900, backend=FakeBackend(
        FakeClock(), {0: 100}, {0: 4}), clock=clock, sleep=clock.sleep)
    assert srv.levels == (3, 5, 7) and srv.damp == 0.5 and srv.low_tconv is None
