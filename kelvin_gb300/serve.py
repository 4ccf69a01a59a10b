"""Serving loop for streams of FT-CCSD requests on one GPU: continuous
batching.

Requests arrive as a Poisson stream; each names a model system (a UEG recipe
or a Hubbard ring), a reduced temperature and a tau grid.  Up to `slots`
requests are on the device at once, each with its own resident solver
(integrals, grid and amplitudes in HBM) on its own context and CUDA stream.
A request is admitted as soon as it has arrived, a slot is free and its
device footprint (kvft_solver_footprint plus the slot's capped tau-chunk
workspace) fits the memory the active slots leave; requests that arrive
while others run wait only for that.  The loop runs in rounds: it queues one
amplitude iteration of every active solve (kvft_solver_step_begin, no host
wait), so their kernels overlap on the device, then collects each result
(kvft_solver_step_end) and advances that solve's own convergence state --
the same phases as ccsd.converge: few-digit sweeps to their noise floor, then
FP64-accurate sweeps to Kelvin's test.  A finished solve frees its slot at
once.  Each solve starts from the converged amplitudes of the finished solve
of the same system and grid whose temperature is nearest (in log Theta), when
one is kept.  A request's latency is its completion time minus its arrival
time; the report gives solves/s and the p50/p99 latencies.

    from kelvin_gb300 import serve
    reqs = serve.request_stream(64, rate=20.0, seed=0)
    print(serve.Server(precision='mixed').serve(reqs))
"""
import time

import numpy

from . import _lib, systems
from .ccsd import PRECISIONS
from .systems import grand_potential0

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
        return systems.hubbard_mf_recipe(sites, 1.0, u, 1.0 / self.theta, device_build=True)


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


class Solve(object):
    """One request on the device: its solver and convergence state (the
    phases of ccsd.converge, advanced one sweep at a time)."""

    def __init__(self, req, levels, refine, conv, start, warm, low_tconv=None):
        self.req = req
        self.low_tconv = low_tconv        # few-digit phases also end below it
        self.levels = list(levels)        # digit levels of the phases, last = refine
        self.refine = refine
        self.conv = conv
        self.start = start
        self.warm = warm
        self.phase = 0
        self.Eold = 888888888.888888888
        self.best, self.since = float("inf"), 0
        self.it_phase = 0
        self.iterations = 0
        self.omega_cc = None
        self.done = False
        self.converged = False
        self.handle = None                # backend state (solver, context, ...)

    def level(self):
        return self.levels[self.phase]

    def advance(self, E, res):
        """Kelvin's test (and, in the few-digit phases, the noise-floor stop)
        after one sweep; True when the solve is finished."""
        self.iterations += 1
        self.it_phase += 1
        conv = abs(E - self.Eold) < self.conv["econv"] and res < self.conv["tconv"]
        last = self.phase == len(self.levels) - 1
        stalled = False
        if not last:
            if res < 0.9 * self.best:
                self.best, self.since = res, 0
            else:
                self.since += 1
                stalled = self.since >= 3
            if self.low_tconv is not None:
                conv = res < self.low_tconv
        self.Eold = E
        if last and (conv or self.it_phase >= self.conv["max_iter"]):
            self.omega_cc, self.converged, self.done = E, conv, True
        elif not last and (conv or stalled or self.it_phase >= self.conv["max_iter"]):
            self.phase += 1
            self.it_phase = 0
            self.Eold = 888888888.888888888
            self.best, self.since = float("inf"), 0
        return self.done


class DeviceBackend(object):
    """Solves on the GPU: one context (CUDA stream) per slot, each with its
    tau-chunk workspace capped so that the slots share the device, and each
    solve's iterations captured once and replayed as a CUDA graph."""

    def __init__(self, slots, workspace_bytes, device=0, graphs=True, accel=0):
        self.graphs = graphs
        self.accel = accel
        self.free_ctx = [_lib.Context(device) for _ in range(slots)]
        for c in self.free_ctx:
            c.set_workspace_limit(workspace_bytes)
        self.workspace_bytes = workspace_bytes

    def mem_total(self):
        return self.free_ctx[0].mem_info()[1] if self.free_ctx else 0

    def footprint(self, req, precision):
        prec = PRECISIONS[precision][0]
        fp = int(_lib.lib().kvft_solver_footprint(req.n_spin_orbitals(), req.ng, prec)) + \
            self.workspace_bytes
        if self.accel:
            # the FP32 Anderson history (1 + 2 depth arrays) over T1 and the
            # spin-conserving elements of T2 (the model systems are spin-blocked)
            n = req.n_spin_orbitals()
            h = n // 2
            fp += 4 * (1 + 2 * self.accel) * req.ng * (n * n + 6 * h ** 4)
        return fp

    def open(self, sv, warm):
        from .cc_utils import DeviceSolver
        from .quadrature import ft_quad
        ctx = self.free_ctx.pop()
        s = sv.req.system()
        beta = 1.0 / s.T
        ti, g, G = ft_quad(sv.req.ng, beta, 'lin')
        en = s.g_energies_tot()
        ctx.set_precision(*_level_precision(sv.level()))
        eri = s.device_aint_tot(ctx)
        try:
            solver = DeviceSolver.from_system(ctx, en, s.g_fock_tot(), eri, beta, s.mu, ti, g, G)
        finally:
            eri.free()
        if warm is not None:
            solver.set_amplitudes(*warm)
            solver.guess(2)
        else:
            solver.guess(1)
        if self.accel:
            solver.set_acceleration(self.accel)
        elif self.graphs:
            solver.set_graph(True)        # iterations replayed as CUDA graphs
        sv.handle = (ctx, solver, s)
        sv.level_set = sv.level()

    def begin(self, sv, damp):
        ctx, solver, _ = sv.handle
        if sv.level_set != sv.level():
            ctx.set_precision(*_level_precision(sv.level()))
            sv.level_set = sv.level()
        solver.step_begin(damp)

    def end(self, sv):
        return sv.handle[1].step_end()

    def close(self, sv, keep):
        """Release the slot; (Omega, the converged amplitudes on the host when
        `keep`)."""
        ctx, solver, s = sv.handle
        amps = solver.amplitudes() if keep else None
        omega = None
        if sv.omega_cc is not None:
            E0 = grand_potential0(1.0 / s.T, s.g_energies_tot(), s.mu) + s.const_energy()
            omega = E0 + s.get_mp1() + sv.omega_cc
        solver.close()
        self.free_ctx.append(ctx)
        sv.handle = None
        return omega, amps


def _level_precision(levels):
    return (_lib.PREC_MIXED, levels) if levels <= 3 else (_lib.PREC_FP64_TC, levels)


class Server(object):
    """Continuous batching of a request stream on one device.

    ``backend`` runs the solves (default: DeviceBackend on the GPU);
    ``clock``/``sleep`` default to real time.  ``budget``: device bytes the
    active solves may hold (default 90 % of the device).  Converged
    amplitudes are kept on the host per (system, grid) and temperature while
    they take at most ``warm_bytes``; ``warm=False`` turns warm starts off.
    ``accel`` > 0: Anderson mixing of that depth with mixing factor ``mix``
    (None: 1 - damp), the few-digit phase going straight to the
    FP64-accurate one and ending once Kelvin's residual is below
    ``low_tconv`` (as ccsd.converge), and the refinement at
    ``refine_digits`` levels (None: 6 with accel, else 7, as ccsd.ccsd); the
    split step keeps the solves overlapped on the device."""

    def __init__(self, precision='mixed', slots=4, budget=None, backend=None,
                 clock=time.perf_counter, sleep=time.sleep, warm_bytes=8 << 30, warm=True,
                 damp=0.5, econv=1e-8, max_iter=200, workspace_bytes=24 << 30, graphs=True,
                 accel=0, mix=None, low_tconv=None, refine_digits=None):
        self.precision = precision
        self.slots = slots
        self.budget = budget
        self._backend = backend
        self.workspace_bytes = workspace_bytes
        self.graphs = graphs
        self.clock, self.sleep = clock, sleep
        self.warm_bytes = warm_bytes
        self.use_warm = warm
        self.accel = accel
        self.low_tconv = low_tconv if accel else None
        self.damp = 1.0 - mix if accel and mix is not None else damp
        self.conv = {"econv": econv, "tconv": 1000.0 * econv, "max_iter": max_iter}
        self.cache = {}                   # key -> {theta: amplitudes}
        digits = PRECISIONS[precision][1]
        refine = refine_digits if refine_digits is not None else (6 if accel else 7)
        self.levels = ((digits, refine) if accel else (digits, 5, refine)) \
            if precision == 'mixed' else (digits,)

    def backend(self):
        if self._backend is None:
            self._backend = DeviceBackend(self.slots, self.workspace_bytes, graphs=self.graphs,
                                          accel=self.accel)
        return self._backend

    def _budget(self):
        if self.budget is None:
            self.budget = int(0.9 * self.backend().mem_total())
        return self.budget

    def _warm(self, req):
        """Amplitudes of the finished solve of the same system and grid at the
        temperature nearest to the request's (log Theta), or None."""
        if not self.use_warm:
            return None
        kept = self.cache.get(req.key())
        if not kept:
            return None
        th = min(kept, key=lambda t: abs(numpy.log(t) - numpy.log(req.theta)))
        return kept[th]

    def _keep(self, req, amps):
        if amps is None:
            return
        self.cache.setdefault(req.key(), {})[req.theta] = amps
        total = sum(_nbytes(a) for k in self.cache.values() for a in k.values())
        while total > self.warm_bytes and self.cache:
            # drop the oldest kept solve
            k = next(iter(self.cache))
            th = next(iter(self.cache[k]))
            total -= _nbytes(self.cache[k].pop(th))
            if not self.cache[k]:
                del self.cache[k]

    def serve(self, requests):
        """Run the stream; returns the report (see `report`)."""
        be = self.backend()
        pending = sorted(requests, key=lambda r: r.arrival)
        budget = self._budget()
        t0 = self.clock()
        active, done, used = [], [], 0
        fps = {}
        rounds = 0
        max_active = 0
        while pending or active:
            now = self.clock() - t0
            # admit: arrived, a free slot, and room in the memory budget
            while pending and pending[0].arrival <= now and len(active) < self.slots:
                r = pending[0]
                fp = be.footprint(r, self.precision)
                if fp > budget:
                    pending.pop(0)
                    done.append({"rid": r.rid, "ok": False, "arrival": r.arrival,
                                 "start": now, "end": now,
                                 "reason": "footprint above the memory budget"})
                    continue
                if used + fp > budget:
                    break                 # waits for memory to free up
                pending.pop(0)
                warm = self._warm(r)
                sv = Solve(r, self.levels, self.levels[-1], self.conv, now, warm is not None,
                           self.low_tconv)
                be.open(sv, warm)
                fps[r.rid] = fp
                used += fp
                active.append(sv)
            max_active = max(max_active, len(active))
            if not active:
                if pending:
                    self.sleep(max(0.0, pending[0].arrival - (self.clock() - t0)))
                continue
            # one round: a sweep of every active solve, overlapped on the device
            failed = {}
            for sv in active:
                try:
                    be.begin(sv, self.damp)
                except Exception as e:
                    failed[sv.req.rid] = str(e)
            finished = []
            for sv in active:
                if sv.req.rid in failed:
                    finished.append(sv)
                    continue
                try:
                    E, res = be.end(sv)
                except Exception as e:            # e.g. a diverging solve
                    failed[sv.req.rid] = str(e)
                    finished.append(sv)
                    continue
                if sv.advance(E, res):
                    finished.append(sv)
            rounds += 1
            for sv in finished:
                active.remove(sv)
                bad = failed.get(sv.req.rid)
                omega, amps = be.close(sv, keep=self.use_warm and bad is None)
                end = self.clock() - t0
                used -= fps.pop(sv.req.rid)
                if bad is not None:
                    done.append({"rid": sv.req.rid, "ok": False, "arrival": sv.req.arrival,
                                 "start": sv.start, "end": end, "reason": bad})
                    continue
                if amps is not None and _nbytes(amps) <= self.warm_bytes:
                    self._keep(sv.req, amps)
                done.append({"rid": sv.req.rid, "ok": True, "arrival": sv.req.arrival,
                             "start": sv.start, "end": end, "warm": sv.warm,
                             "omega": omega, "omega_cc": sv.omega_cc,
                             "iterations": sv.iterations, "converged": sv.converged})
        rep = report(done, self.clock() - t0)
        rep.update({"slots": self.slots, "rounds": rounds, "max_active": max_active})
        return rep


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
            "converged": sum(1 for d in ok if d.get("converged", True)),
            "solves_per_s": len(ok) / wall if wall > 0 else 0.0,
            "p50_ms": float(numpy.percentile(lat, 50)) if len(lat) else None,
            "p99_ms": float(numpy.percentile(lat, 99)) if len(lat) else None,
            "warm_started": sum(1 for d in ok if d.get("warm")), "wall_s": wall,
            "requests": done}
