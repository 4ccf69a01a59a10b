"""Serving loop for streams of FT-CCSD requests on one GPU.

Requests arrive as a Poisson stream; each names a model system (a UEG recipe
or a Hubbard ring), a reduced temperature and a tau grid.  One worker solves
them in arrival order on the device, admitting a request only when its device
footprint (kvft_solver_footprint) fits the memory budget, and warm-starting a
system already solved at another temperature on the same grid from that
solve's converged amplitudes.  A request's latency is its completion time
minus its arrival time (queueing included); the report gives solves/s and the
p50/p99 latencies.

    from kelvin_gb300 import serve
    reqs = serve.request_stream(64, rate=20.0, seed=0)
    print(serve.Server(precision='mixed').serve(reqs))
"""
import time

import numpy

from . import _lib, systems
from .ccsd import PRECISIONS, ccsd

# (electrons, plane waves) of the UEG requests; Hubbard rings take 8-16 sites
UEG_SHAPES = ((14, 19), (14, 27), (38, 33), (38, 57))
NGRIDS = (10, 20, 40)


class Request(object):
    """One solve: kind 'ueg' with params (N, plane waves, rs) or 'hubbard'
    with (sites, U/t); theta = T / T_F (UEG) or T / t (Hubbard)."""

    def __init__(self, rid, arrival, kind, params, theta, ng):
        self.rid, self.arrival = rid, arrival
        self.kind, self.params, self.theta, self.ng = kind, params, theta, ng

    def key(self):
        """Requests with one key share a system and a grid (warm starts)."""
        return (self.kind, self.params, self.ng)

    def n_spin_orbitals(self):
        return 2 * (self.params[1] if self.kind == 'ueg' else self.params[0])

    def system(self):
        if self.kind == 'ueg':
            N, norb, rs = self.params
            return systems.ueg_recipe(N, rs, norb, self.theta, device_build=True)
        sites, u = self.params
        return systems.hubbard_recipe(sites, 1.0, u, 1.0 / self.theta, device_build=True)


def request_stream(count, rate=20.0, seed=0):
    """`count` requests with exponential inter-arrival times (mean 1/rate s),
    drawn uniformly from the four UEG shapes (rs uniform in [1, 4]) and
    Hubbard rings (8-16 sites, U/t uniform in [1, 8]), theta log-uniform in
    [0.1, 4] and ng from {10, 20, 40}; seeded, so a stream is reproducible."""
    rng = numpy.random.default_rng(seed)
    out, t = [], 0.0
    for rid in range(count):
        t += rng.exponential(1.0 / rate)
        pick = int(rng.integers(0, len(UEG_SHAPES) + 1))
        if pick < len(UEG_SHAPES):
            N, norb = UEG_SHAPES[pick]
            params = (N, norb, round(float(rng.uniform(1.0, 4.0)), 3))
            kind = 'ueg'
        else:
            params = (int(rng.integers(8, 17)), round(float(rng.uniform(1.0, 8.0)), 3))
            kind = 'hubbard'
        theta = float(numpy.exp(rng.uniform(numpy.log(0.1), numpy.log(4.0))))
        ng = int(NGRIDS[int(rng.integers(0, len(NGRIDS)))])
        out.append(Request(rid, t, kind, params, theta, ng))
    return out


class Server(object):
    """Solves requests in arrival order on one device.

    ``solve(req, warm)`` -> (Omega, amplitudes) and ``footprint(req)`` ->
    bytes default to the device solver; ``clock``/``sleep`` to real time.
    ``budget`` is the device memory a request may use (default: 90 % of the
    device).  Warm-start amplitudes are kept per key while they take at most
    ``warm_bytes`` on the host."""

    def __init__(self, precision='mixed', ctx=None, budget=None, solve=None, footprint=None,
                 clock=time.perf_counter, sleep=time.sleep, warm_bytes=2 << 30):
        self.precision = precision
        self.ctx = ctx
        self.budget = budget
        self.solve = solve or self._solve_on_device
        self.footprint = footprint or self._footprint
        self.clock, self.sleep = clock, sleep
        self.warm_bytes = warm_bytes
        self.cache = {}

    def _device(self):
        if self.ctx is None:
            self.ctx = _lib.context(0)
        return self.ctx

    def _footprint(self, req):
        prec = PRECISIONS[self.precision][0]
        return int(_lib.lib().kvft_solver_footprint(req.n_spin_orbitals(), req.ng, prec))

    def _budget(self):
        if self.budget is None:
            import torch
            free, total = torch.cuda.mem_get_info(0)
            self.budget = int(0.9 * total)
        return self.budget

    def _solve_on_device(self, req, warm):
        s = req.system()
        cc = ccsd(s, T=s.T, mu=s.mu, ngrid=req.ng, damp=0.5, econv=1e-8, max_iter=200,
                  precision=self.precision, ctx=self._device())
        try:
            omega = cc.run(*warm)[0] if warm is not None else cc.run()[0]
            # in the form run() takes them back (per spin case for unrestricted systems)
            return omega, (cc.T1, cc.T2)
        finally:
            cc.release()

    def serve(self, requests):
        """Run the stream; returns the report (see `report`)."""
        reqs = sorted(requests, key=lambda r: r.arrival)
        t0 = self.clock()
        done = []
        for r in reqs:
            now = self.clock() - t0
            if now < r.arrival:
                self.sleep(r.arrival - now)
            start = self.clock() - t0
            if self.footprint(r) > self._budget():
                done.append({"rid": r.rid, "ok": False, "arrival": r.arrival, "start": start,
                             "end": start, "reason": "footprint above the memory budget"})
                continue
            warm = self.cache.get(r.key())
            omega, amps = self.solve(r, warm)
            end = self.clock() - t0
            if amps is not None and _nbytes(amps) <= self.warm_bytes:
                self.cache[r.key()] = amps
            done.append({"rid": r.rid, "ok": True, "arrival": r.arrival, "start": start,
                         "end": end, "warm": warm is not None, "omega": omega})
        return report(done, self.clock() - t0)


def _nbytes(x):
    if isinstance(x, (tuple, list)):
        return sum(_nbytes(y) for y in x)
    return x.nbytes


def report(done, wall):
    """solves, rejected, solves/s over the wall time, p50/p99 latency (ms,
    completion - arrival) and warm-started count."""
    ok = [d for d in done if d["ok"]]
    lat = numpy.array([d["end"] - d["arrival"] for d in ok]) * 1e3
    return {"solves": len(ok), "rejected": len(done) - len(ok),
            "solves_per_s": len(ok) / wall if wall > 0 else 0.0,
            "p50_ms": float(numpy.percentile(lat, 50)) if len(lat) else None,
            "p99_ms": float(numpy.percentile(lat, 99)) if len(lat) else None,
            "warm_started": sum(1 for d in ok if d.get("warm")), "wall_s": wall,
            "requests": done}
