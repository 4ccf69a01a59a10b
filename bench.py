#!/usr/bin/env python
"""FT-CCSD solves/s on GB300 (libkvft) or on the host cores (reference arm).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl kvft|reference]
                    [--workload ueg114|ueg38] [--precision mixed|fp64_tc|fp64]
                    [--quad gl|lin]
    python bench.py --gemm M,N,K,batch [--precision ...]      # one contraction shape
    python bench.py --system-build [--workload ...]
        # time building the model system's integrals: dense n^4 on the host
        # against kvft_ueg_eri on the device (closed-form Fock and E1)
    python bench.py --profile-step [--workload ...] [--precision ...]
        # one warm-up iteration, then one iteration; prints the library's
        # kernel-launch counts so that a profiler's launch list can be cut to
        # exactly the second iteration
    python bench.py --accuracy
        # mixed against FP64-accurate on the smaller configurations: the
        # 38-spin-orbital UEG (Simpson and Gauss-Legendre grids), the 16-site
        # Hubbard ring at beta 1, 4, 10 and the 66-spin-orbital UEG:
        # |dOmega|, |dE|, |dS|

Workloads are seeded synthetic uniform electron gases (the benchmark configs):

* ueg114 (default): 38 electrons, rs = 1, the 57 lowest plane waves (114 spin
  orbitals), Theta = 0.25, ng = 20 Gauss-Legendre points, damping 0.5, econv
  1e-10.  A solve takes seconds, so a timed step is ONE amplitude iteration
  (CCSD update of all tau points + integration + damping + norms + energy)
  and solves/s = 1 / sum over the solve's phases of (iterations x seconds per
  iteration at that phase's digit levels), the iteration counts taken from a
  complete solve in the same run.
* ueg38: 14 electrons, rs = 4, 19 plane waves (38 spin orbitals), Theta = 0.5,
  ng = 10: a step is a complete solve (first-order guess to convergence).

``value`` times the steps with the integrals and buffers already resident in
HBM; ``e2e`` times complete solves through the public drop-in API
(``kelvin_gb300.ccsd.ccsd(sys, ...).run()``) from host arrays, including the
host->device upload of the integrals and the read-back of the amplitudes.
The headline precision is 'mixed': three BF16 digit levels on tensor cores
until the iteration's noise floor, five levels to theirs, then FP64-accurate
(seven-level) sweeps until Kelvin's convergence test passes; quadrature,
damping and energy are FP64 throughout.  Beside it the same run measures the
FP64-accurate solve (|dOmega| of the mixed solve against it) and one
iteration of the plain FP64 path (FP64 FMA contractions).  With N > 1
(torchrun) every rank runs an independent replica: only the timings are
reduced (gloo).  One JSON line is printed by rank 0.

The reference arm (--impl reference) runs the oracle -- the numpy FP64
restatement of Kelvin's iteration (ccsd_stanton at every tau point,
int_tbar, damping, ft_cc_energy) -- on the host cores: a complete solve of the
38-spin-orbital configuration, its iterations timed one by one.  A solve of
the 114-spin-orbital configuration needs tens of minutes per iteration on the
host, so its rate appears only as a labelled estimate.
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "FT-CCSD solves/s"
UNIT = "solves/s"

WORKLOADS = {
    "ueg114": dict(N=38, rs=1.0, norb=57, theta=0.25, ng=20, damp=0.5, econv=1e-10,
                   max_iter=100, step="iteration",
                   label="UEG 38 e-, rs=1, 57 plane waves (114 spin orbitals), Theta=0.25, "
                         "ng=20, damping 0.5, econv 1e-10"),
    "ueg66": dict(N=14, rs=2.0, norb=33, theta=0.5, ng=16, damp=0.5, econv=1e-10,
                  max_iter=100, step="iteration",
                  label="UEG 14 e-, rs=2, 33 plane waves (66 spin orbitals), Theta=0.5, "
                        "ng=16, damping 0.5, econv 1e-10"),
    "ueg38": dict(N=14, rs=4.0, norb=19, theta=0.5, ng=10, damp=0.5, econv=1e-10,
                  max_iter=100, step="solve",
                  label="UEG 14 e-, rs=4, 19 plane waves (38 spin orbitals), Theta=0.5, "
                        "ng=10, damping 0.5, econv 1e-10"),
}
# DRAM / algorithmic byte ratios per kernel category, measured by ncu on a
# small case (read at run time from the committed summary, so that a re-taken
# capture updates them); roofline.traffic = ratio x live algorithmic bytes
TRAFFIC_FILE = os.path.join(ROOT, "profiles", "traffic.json")
STEP_EVENTS = 8     # first event slot of the per-step timings (at most 50 steps)


def load_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        return json.load(open(p)), "measured"
    return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0, "bf16_tflops_sustained": 1700.0}, \
        "fallback"


class ClockSampler(object):
    """nvidia-smi clocks / throttle reasons sampled during the timed region."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device = device
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device), "--query-gpu=" + self.FIELDS,
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            threading.Thread(target=self._read, daemon=True).start()
        except Exception:
            self.proc = None

    def _read(self):
        for ln in self.proc.stdout:
            self.lines.append(ln.strip())

    def stop(self):
        if not self.proc:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        sm, smax, reasons = [], [], set()
        names = ("hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap")
        for ln in self.lines:
            p = [x.strip() for x in ln.split(",")]
            if len(p) < 8:
                continue
            try:
                sm.append(float(p[0]))
                smax.append(float(p[1]))
            except ValueError:
                continue
            for nm, v in zip(names, p[4:8]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(smax),
                "samples": len(sm), "reasons": sorted(reasons)}


def build_system(w):
    from kelvin_gb300 import systems
    return systems.ueg_recipe(w["N"], w["rs"], w["norb"], w["theta"])


def dist_setup():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("gloo")
    return ws, rank, local


def barrier(ws):
    if ws > 1:
        import torch.distributed as dist
        dist.barrier()


def max_over_ranks(ws, x):
    if ws == 1:
        return x
    import torch
    import torch.distributed as dist
    t = torch.tensor([float(x)], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


# ---------------------------------------------------------------------------
# CPU reference: the oracle (numpy FP64 restatement of Kelvin's path) on the
# host cores
# ---------------------------------------------------------------------------
def oracle_c1_iterations(quad, max_iters, until_converged):
    """The oracle's FT-CCSD loop (Kelvin's ccsd_stanton over all tau points,
    int_tbar, damping, residual norms, ft_cc_energy; cc_utils.py:111-173)
    on the 38-spin-orbital configuration, each iteration timed.  Stops after
    `max_iters` iterations or, with until_converged, at Kelvin's test if that
    comes later.  Returns (seconds of the first-order guess, per-iteration
    seconds, the iteration at which Kelvin's test passed or None, Omega_cc)."""
    import numpy
    from oracle import ft_ccsd, ft_utils, quadrature
    w = WORKLOADS["ueg38"]
    sysobj = build_system(w)
    beta = 1.0 / sysobj.T
    en = sysobj.g_energies_tot()
    ng, alpha = w["ng"], w["damp"]
    full = quad == "gl"
    ti, g, G = quadrature.ft_quad(ng, beta, quad)
    F, I = ft_ccsd.ft_integrals(sysobj.g_fock_tot(), sysobj.g_aint_tot(), en, beta, sysobj.mu)
    D1, D2 = ft_utils.D1(en, en), ft_utils.D2(en, en)
    t0 = time.perf_counter()
    T1 = quadrature.int_tbar1(ng, numpy.repeat(-F.vo[None], ng, 0), ti, D1, G, full=full)
    T2 = quadrature.int_tbar2(ng, numpy.repeat(-I.vvoo[None], ng, 0), ti, D2, G, full=full)
    t_guess = time.perf_counter() - t0
    nl1, nl2 = numpy.linalg.norm(T1) + 0.1, numpy.linalg.norm(T2) + 0.1
    Eold, times, conv_at, i = 888888888.888888888, [], None, 0
    while True:
        t0 = time.perf_counter()
        T1n, T2n = ft_ccsd.ccsd_stanton(F, I, T1, T2, D1, D2, ti, ng, G, full=full)
        res = (numpy.linalg.norm(T1n - T1) / nl1 + numpy.linalg.norm(T2n - T2) / nl2)
        T1 = alpha * T1 + (1.0 - alpha) * T1n
        T2 = alpha * T2 + (1.0 - alpha) * T2n
        nl1, nl2 = numpy.linalg.norm(T1) + 0.1, numpy.linalg.norm(T2) + 0.1
        E = ft_ccsd.ft_cc_energy(T1, T2, F.ov, I.oovv, g, beta)
        times.append(time.perf_counter() - t0)
        i += 1
        if conv_at is None and abs(E - Eold) < w["econv"] and res < 1e3 * w["econv"]:
            conv_at = i
        Eold = E
        if i >= max_iters and (conv_at is not None or not until_converged):
            break
        if i >= 200:
            break
    return t_guess, times, conv_at, E


def c2_estimate(t_iter_c1, iters):
    """solves/s of the 114-spin-orbital configuration ESTIMATED from a
    38-spin-orbital iteration: contraction work scales as n^6 ng, so
    t_114 = t_38 (114/38)^6 (20/10)."""
    t = t_iter_c1 * (114.0 / 38.0) ** 6 * 2.0
    return {"value": 1.0 / (t * iters), "unit": UNIT, "seconds_per_iteration": t,
            "iterations": iters,
            "how": "ESTIMATE, not measured: the measured 38-spin-orbital oracle iteration "
                   "scaled by the contraction work n^6 ng to 114 spin orbitals, ng = 20, "
                   "times the iteration count of Kelvin's damped FP64 solve"}


def run_reference(args, w):
    ws, rank, _ = dist_setup()
    if rank != 0:
        return 0
    threads = os.cpu_count()
    t_guess, times, conv_at, E = oracle_c1_iterations(args.quad, args.warmup + args.steps,
                                                      until_converged=True)
    timed = times[args.warmup:args.warmup + args.steps]
    t_iter = statistics.median(timed)
    iters = conv_at or len(times)
    t_solve = t_guess + sum(times[:iters])
    value = 1.0 / t_solve
    wl = WORKLOADS["ueg38"]
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": UNIT,
            "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": t_iter * 1e3, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": wl["label"] + " (%s tau grid)" % args.quad,
                       "step": "one amplitude iteration of the oracle's complete solve",
                       "iterations_per_solve": iters, "converged": conv_at is not None,
                       "omega_cc": E, "guess_s": t_guess, "solve_s": t_solve,
                       "impl": "oracle: numpy FP64 restatement of Kelvin's FT-CCSD iteration "
                               "(Kelvin is pure Python with an un-vendored dependency and "
                               "cannot run on the GPU host); BLAS threads = all host cores",
                       "note": "value = 1 / measured wall time of the complete 38-spin-"
                               "orbital solve; the 114-spin-orbital rate is only estimated"},
            "estimate_ueg114": c2_estimate(t_iter, iters),
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port",
                             "sample": "complete oracle solve of the 38-spin-orbital UEG "
                                       "(%d iterations, %.1f s)" % (iters, t_solve)},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}
    print(json.dumps(line))
    return 0


def load_traffic(precision, category, algorithmic_per_launch):
    """Per-launch DRAM bytes of a kernel category: the DRAM / algorithmic
    ratio measured by ncu on a small case (profiles/traffic.json) times this
    run's algorithmic bytes per launch of the category; (bytes, how) or
    (None, None) where no ratio was measured."""
    try:
        t = json.load(open(TRAFFIC_FILE))
    except (OSError, ValueError):
        return None, None
    e = t.get(precision, {}).get(category)
    if not e or not algorithmic_per_launch:
        return None, None
    r = e["dram_per_algorithmic"]
    return r * algorithmic_per_launch, (
        "%.3f x the live algorithmic bytes per launch; the ratio is ncu's on %s"
        % (r, t.get("measured_on", "a small case")))


# ---------------------------------------------------------------------------
# GPU arm
# ---------------------------------------------------------------------------
def run_gpu(args, w):
    ws, rank, local = dist_setup()
    from kelvin_gb300 import _lib, ccsd
    from kelvin_gb300.cc_utils import DeviceSolver
    from kelvin_gb300.quadrature import ft_quad

    ctx = _lib.context(local)
    prec, digits = ccsd.PRECISIONS[args.precision]
    if args.digits:
        digits = args.digits
    sysobj = build_system(w)
    beta = 1.0 / sysobj.T
    en = sysobj.g_energies_tot()
    fock, eri = sysobj.g_fock_tot(), sysobj.g_aint_tot()
    full = args.quad == "gl"
    ti, g, G = ft_quad(w["ng"], beta, args.quad)
    conv = {"econv": w["econv"], "tconv": 1000.0 * w["econv"], "max_iter": w["max_iter"],
            "damp": w["damp"]}
    n, ng = en.shape[0], w["ng"]
    per_solve = w["step"] == "solve"
    mixed = args.precision == "mixed"

    ctx.set_precision(prec, digits)
    solver = DeviceSolver.from_system(ctx, en, fock, eri, beta, sysobj.mu, ti, g, G)
    solver.full = full
    if args.accel:
        solver.set_acceleration(args.accel)
    solver.guess(1)
    ladder = (5,) if not args.accel else ()
    low_tconv = args.low_tconv if args.accel else None
    # the mixed form's refinement levels (the driver's default for the update)
    refine = 6 if args.accel else 7

    def one_step():
        if per_solve:
            solver.guess(1)
            E, info = ccsd.converge(solver, ctx, dict(conv, damp=1.0 - args.mix)
                                    if args.accel else conv, args.precision, digits,
                                    ladder=ladder, low_tconv=low_tconv,
                                    refine_digits=refine)
            return E, info["iterations"] + info["iterations_refine"]
        return solver.step(w["damp"])[0], 1

    for _ in range(args.warmup):
        one_step()
    ctx.sync()
    barrier(ws)
    clocks = ClockSampler(local)
    clocks.start()
    l0 = ctx.launches()
    ctx.profile_begin()
    ctx.record(0)
    results = []
    for k in range(args.steps):
        if k < 50:
            ctx.record(STEP_EVENTS + k)
        results.append(one_step())
    if args.steps <= 50:
        ctx.record(STEP_EVENTS + args.steps)
    ctx.record(1)
    ctx.sync()
    prof = ctx.profile_end()
    launches = ctx.launches() - l0
    ms = max_over_ranks(ws, ctx.elapsed_ms(0, 1))
    lat = sorted(ctx.elapsed_ms(STEP_EVENTS + k, STEP_EVENTS + k + 1)
                 for k in range(min(args.steps, 50))) if args.steps <= 50 else []
    clk = clocks.stop()
    step_ms = ms / args.steps

    def timed_steps(precision, levels, count, warm=1):
        """Device milliseconds of one iteration at a precision (mean of
        `count` after `warm` untimed ones), on the resident solver."""
        ctx.set_precision(precision, levels)
        for _ in range(warm):
            solver.step(w["damp"])
        ctx.sync()
        ctx.record(4)
        for _ in range(count):
            solver.step(w["damp"])
        ctx.record(5)
        ctx.sync()
        return ctx.elapsed_ms(4, 5) / count

    level_ms = {}
    dfma_ms = None
    if not per_solve:
        level_ms[digits if args.precision != "fp64" else 0] = step_ms
        if mixed:
            for lv in sorted(set(ladder + (refine, 7))):
                level_ms[lv] = timed_steps(_lib.PREC_FP64_TC, lv, 2)
        elif args.precision == "fp64_tc":
            level_ms[7] = step_ms
        # the plain FP64 path: FP64 FMA contractions on the FP64 pipe (one
        # iteration; tens of seconds at 114 spin orbitals)
        dfma_ms = step_ms if args.precision == "fp64" else \
            timed_steps(_lib.PREC_FP64, 7, 1, warm=0)
        ctx.set_precision(prec, digits)
    solver.close()

    # ---- complete solves through the public drop-in API (e2e) -------------
    # from host arrays: integral upload, guess, all phases of the iteration,
    # and the read-back of the amplitudes
    def solve(precision, lv, accel):
        cc = ccsd.ccsd(sysobj, T=sysobj.T, mu=sysobj.mu, max_iter=w["max_iter"],
                       damp=w["damp"], ngrid=ng, econv=w["econv"], quad=args.quad,
                       precision=precision, digits=lv, accel=accel,
                       mix=args.mix if accel else None,
                       low_tconv=low_tconv if accel else None, ctx=ctx)
        ctx.sync()
        ctx.record(2)
        t0 = time.perf_counter()
        cc.run()
        ctx.record(3)
        ctx.sync()
        wall = max(ctx.elapsed_ms(2, 3), (time.perf_counter() - t0) * 1e3)
        out = {"omega_cc": cc.Gcc, "iterations": cc.iterations + cc.iterations_refine,
               "phases": cc.phases, "converged": bool(cc.converged), "ms": wall}
        cc.release()
        return out

    barrier(ws)
    n_e2e = args.steps if per_solve else 1
    e2e_runs = [solve(args.precision, digits, args.accel) for _ in range(n_e2e)]
    e2e_ms = max_over_ranks(ws, sum(r["ms"] for r in e2e_runs))
    e2e_value = ws * n_e2e / (e2e_ms / 1e3)
    sol = e2e_runs[-1]
    # FP64-accurate solves: with the headline's iteration scheme (its rate), and
    # Kelvin's damped loop (the parity path: the accuracy reference)
    acc64 = solve("fp64_tc", 7, args.accel) if args.precision != "fp64_tc" else sol
    ref64 = solve("fp64_tc", 7, 0) if args.accel else acc64
    h2d = 8 * (n + n * n + n ** 4 + 2 * ng + ng * ng)
    # the amplitudes Kelvin's solve leaves on the instance: T1 and the
    # spin-conserving elements of T2 cross the link (the host array's other
    # blocks are zero pages); plus the scalars each iteration reads back
    h = n // 2
    d2h = 8 * ng * (n * n + 6 * h ** 4) + 8 * 7 * (sol["iterations"] + 2)

    # solves/s with everything resident: per-phase iterations of the measured
    # solve times that phase's measured seconds per iteration
    if per_solve:
        value = ws / (step_ms / 1e3)
        t_solve_ms = step_ms
    else:
        t_solve_ms = 0.0
        for lv, it, _ in sol["phases"]:
            t_solve_ms += it * level_ms.get(lv if args.precision != "fp64" else 0, step_ms)
        value = ws / (t_solve_ms / 1e3)

    if rank != 0:
        return 0
    peaks, peak_src = load_peaks()
    kernels = {"gemm6": "tc_gemm_kernel, n^6-class contractions",
               "gemm": "tc_gemm_kernel, n^5-class contractions", "quad": "quad_kernel",
               "energy": "energy2_kernel", "elem": "element-wise passes",
               "pack": "digit packing (pack_rows/pack_exp/pack_digits)"}
    if args.precision == "fp64":
        kernels["gemm6"] = "gemm_f64_kernel, n^6-class contractions"
        kernels["gemm"] = "gemm_f64_kernel, n^5-class contractions"

    def roof(c):
        """Achieved rate of one category against its bound: tensor flops for
        the n^6 contractions (GB300's FP64 pipe for the FP64 form), bytes per
        second against HBM for everything else."""
        nl, dms, work = prof[c]
        if nl == 0 or dms <= 0:
            return None
        if c == "gemm6":
            achieved, unit, bound = work / (dms / 1e3) / 1e12, "TFLOP/s", "tensor"
            if args.precision == "fp64":
                peak = 1.25
                psrc = "nominal GB300 FP64 1.25 TFLOP/s (no measured FP64 figure)"
            else:
                pairs = sum(l - 1 for l in range(2, digits + 1))
                achieved *= pairs      # BF16 tensor flops issued per FP64-equivalent flop
                peak = peaks["bf16_tflops_sustained"]
                psrc = "bf16_tflops_sustained of %s peaks; achieved = the spin-blocked " \
                       "algorithmic 2MNK flops x %d digit-pair products" % (peak_src, pairs)
        else:
            achieved, unit, bound = work / (dms / 1e3) / 1e9, "GB/s", "hbm"
            peak = peaks["hbm_gbs"]
            psrc = "hbm_gbs of %s peaks; achieved = algorithmic bytes" % peak_src
        return {"bound": bound, "kernel": kernels[c], "achieved": achieved, "peak": peak,
                "unit": unit, "frac": achieved / peak, "launches": nl,
                "avg_launch_ms": dms / nl, "peak_source": psrc}

    cats = {c: roof(c) for c in prof}
    dom = max(prof, key=lambda c: prof[c][1])
    roofline = dict(cats[dom])
    nl_dom = prof[dom][0]
    traffic, thow = load_traffic(args.precision, dom,
                                 prof[dom][2] / nl_dom if nl_dom and dom != "gemm6" else None)
    roofline.update({
        "category": dom, "traffic": traffic,
        "traffic_unit": "bytes per launch (ncu dram__bytes_read.sum + dram__bytes_write.sum)"
                        if traffic else None, "traffic_how": thow,
        "categories": {c: {k: cats[c][k] for k in ("bound", "achieved", "unit", "frac",
                                                   "avg_launch_ms", "launches")}
                       for c in cats if cats[c]},
        "breakdown_ms_per_step": {c: round(prof[c][1] / args.steps, 3) for c in prof}})

    # CPU baseline: a bounded sample of the oracle's iteration (guess and three
    # iterations of the 38-spin-orbital solve) on the host cores
    t_guess, times, _, _ = oracle_c1_iterations(args.quad, 3, until_converged=False)
    t_iter_c1 = statistics.median(times)
    cfg = {"workload": w["label"].replace("ng=%d" % ng, "ng=%d %s" % (
               ng, "Gauss-Legendre" if full else "Simpson ('lin')")),
           "step": w["step"], "precision": args.precision,
           "update": ("Anderson mixing, depth %d, mixing factor %g (the damped update's "
                      "fixed point; Kelvin's test)%s" % (
                          args.accel, args.mix,
                          "; few-digit phase until Kelvin's residual < %g or its noise floor"
                          % low_tconv if mixed and low_tconv else "")
                      if args.accel else "Kelvin's damped update"),
           "digits": digits if args.precision != "fp64" else None,
           "solve": {k: sol[k] for k in ("iterations", "phases", "converged", "omega_cc")},
           "l2": "per-step working set > 129 MB L2 (no flush)",
           "parallelism": "replicas" if ws > 1 else "single GPU"}
    if not per_solve:
        cfg["ms_per_iteration"] = {("fp64_fma" if k == 0 else "%d_levels" % k): v
                                   for k, v in sorted(level_ms.items())}
        cfg["ms_per_solve_resident"] = t_solve_ms
    if lat:
        q = lambda f: lat[min(len(lat) - 1, int(f * len(lat)))]
        cfg["step_latency_ms"] = {"p50": q(0.5), "p99": q(0.99), "n": len(lat)}
    # mixed against FP64-accurate on the 38-spin-orbital configuration as well,
    # with E and S from the Lambda equations (Kelvin's Simpson grid, on which
    # they are built): a few seconds
    if mixed and not per_solve:
        cfg["accuracy_38_spin_orbitals"] = small_accuracy(ctx, args)
    # the reference arm's workload (the 38-spin-orbital configuration on this
    # run's grid), end to end through the same driver: the like-for-like
    # rate beside the reference's (median of three solves each)
    if not per_solve and ws == 1:
        w38 = WORKLOADS["ueg38"]
        s38 = build_system(w38)

        def solve38(precision, accel):
            runs = []
            for _ in range(3):
                cc = ccsd.ccsd(s38, T=s38.T, mu=s38.mu, max_iter=w38["max_iter"],
                               damp=w38["damp"], ngrid=w38["ng"], econv=w38["econv"],
                               quad=args.quad, precision=precision, accel=accel,
                               mix=args.mix if accel else None,
                               low_tconv=low_tconv if accel else None, ctx=ctx)
                ctx.sync()
                t0 = time.perf_counter()
                cc.run()
                ctx.sync()
                runs.append((time.perf_counter() - t0,
                             cc.iterations + cc.iterations_refine, cc.Gcc))
                cc.release()
            t, it, E = sorted(runs)[1]
            return {"solves_per_s": 1.0 / t, "iterations": it, "omega_cc": E}
        cfg["reference_workload_e2e"] = {
            "workload": w38["label"] + " (%s tau grid)" % args.quad,
            "mixed": solve38(args.precision, args.accel),
            "fp64_tc_damped": solve38("fp64_tc", 0),
            "how": "ccsd(...).run() from host arrays, wall clock, median of three; the "
                   "reference arm times the oracle's complete solve of this workload"}
    if ref64 is not sol:
        d = abs(sol["omega_cc"] - ref64["omega_cc"])
        cfg["fp64_tc_solve"] = {k: ref64[k] for k in ("iterations", "converged", "omega_cc",
                                                     "ms")}
        cfg["accuracy"] = {"abs_dOmega": d, "abs_dOmega_per_electron": d / w["N"],
                           "bar_per_electron": 1e-6,
                           "against": "FP64-accurate solve with Kelvin's damped loop, same run"}
        if acc64 is not ref64:
            cfg["fp64_tc_accelerated_solve"] = {k: acc64[k] for k in ("iterations", "converged",
                                                                      "omega_cc", "ms")}
        if not per_solve and 7 in level_ms:
            fp64tc = 1.0 / (acc64["iterations"] * level_ms[7] / 1e3)
            cfg["fp64_tc_solves_per_s"] = fp64tc
            cfg["mixed_over_fp64_tc"] = value / fp64tc
            cfg["fp64_tc_damped_solves_per_s"] = 1.0 / (ref64["iterations"] * level_ms[7] / 1e3)
    if dfma_ms is not None:
        it64 = acc64["iterations"]
        plain = 1.0 / (it64 * dfma_ms / 1e3)
        cfg["plain_fp64_solves_per_s"] = plain
        cfg["plain_fp64_how"] = ("one measured iteration of the FP64 FMA path x the "
                                 "iteration count of the FP64-accurate solve with the same "
                                 "update (%d)" % it64)
        cfg["over_plain_fp64"] = value / plain
        cfg["plain_fp64_damped_solves_per_s"] = 1.0 / (ref64["iterations"] * dfma_ms / 1e3)
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": step_ms,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": {"fp64": "f64", "fp64_tc": "f64 (7 BF16 digit levels, tensor cores)",
                      "mixed": "bf16 digits/f32 acc (%s levels) + %d-level refinement "
                               "(FP64-accurate: 7); f64 quadrature, update, energy"
                               % (", ".join(str(x) for x in (digits,) + ladder), refine)}[
                          args.precision],
            "data": "synthetic", "config": cfg, "roofline": roofline,
            "cpu_baseline": {"value": None, "unit": UNIT, "cores": os.cpu_count(),
                             "kind": "port"},
            "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": h2d,
                    "d2h_bytes_per_step": d2h,
                    "how": "ccsd(...).run() from host arrays: integral upload, solve, "
                           "amplitudes read back into ccsd.T1 / ccsd.T2 (numpy)"},
            "gpu_launches": launches, "clocks": clk}
    est = c2_estimate(t_iter_c1, ref64["iterations"])     # the reference's damped loop
    if per_solve:
        line["cpu_baseline"].update({
            "value": 1.0 / (t_guess + t_iter_c1 * ref64["iterations"]),
            "sample": "oracle guess + 3 iterations of the same solve on the host (median "
                      "%.2f s/iteration) x the %d iterations of Kelvin's damped FP64 solve"
                      % (t_iter_c1, ref64["iterations"])})
    else:
        line["cpu_baseline"].update({
            "value": est["value"],
            "sample": "oracle guess + 3 iterations of the 38-spin-orbital solve on the host "
                      "(median %.2f s/iteration), SCALED by the contraction work n^6 ng to "
                      "this workload (an estimate; a measured 114-spin-orbital iteration takes "
                      "tens of minutes)" % t_iter_c1})
    print(json.dumps(line))
    return 0


def run_profile_step(args, w):
    """One warm-up iteration and one profiled iteration of the solver."""
    from kelvin_gb300 import _lib, ccsd
    from kelvin_gb300.cc_utils import DeviceSolver
    from kelvin_gb300.quadrature import ft_quad
    ctx = _lib.context(0)
    prec, digits = ccsd.PRECISIONS[args.precision]
    ctx.set_precision(prec, args.digits or digits)
    s = build_system(w)
    beta = 1.0 / s.T
    ti, g, G = ft_quad(w["ng"], beta, args.quad)
    solver = DeviceSolver.from_system(ctx, s.g_energies_tot(), s.g_fock_tot(), s.g_aint_tot(),
                                      beta, s.mu, ti, g, G)
    solver.full = args.quad == "gl"
    solver.guess(1)
    if args.accel:
        solver.set_acceleration(args.accel)
    # enough warm-up iterations for a full Anderson history
    for _ in range(1 + (args.accel if args.accel else 0)):
        solver.step(w["damp"])
    ctx.sync()
    l0 = ctx.launches()
    ctx.profile_begin()
    E, res = solver.step(w["damp"])
    ctx.sync()
    recs = ctx.profile_records()
    shapes = ctx.profile_shapes()
    ctx.profile_end()
    if args.records:
        # every timed scope of the iteration: category, ms, work, GEMM shape
        with open(args.records, "w") as f:
            for (c, ms, wk), sh in zip(recs, shapes):
                f.write("%s %.4f %.4e %d %d %d %d\n" % ((c, ms, wk) + tuple(sh)))
    # the category of each contraction of the step, in launch order: one
    # GEMM kernel (tc_gemm_kernel or gemm_f64_kernel) per contraction
    gemm_cats = [c for c, _, _ in recs if c in ("gemm6", "gemm")]
    print(json.dumps({"profile_step": args.workload, "precision": args.precision,
                      "accel": args.accel, "launches_before": l0, "launches_in_step": ctx.launches() - l0,
                      "omega_cc": E, "res": res, "gemm_categories": gemm_cats}))
    solver.close()
    return 0


def run_system_build(args, w):
    """Seconds to build the workload's integrals on the host and on the device."""
    from kelvin_gb300 import _lib, systems
    ctx = _lib.context(0)
    t0 = time.perf_counter()
    s = systems.ueg_recipe(w["N"], w["rs"], w["norb"], w["theta"])
    eri = s.g_aint_tot()
    fock, e1 = s.g_fock_tot(), s.get_mp1()
    t_host = time.perf_counter() - t0
    n = eri.shape[0]
    del eri
    out = []
    for _ in range(2):                 # the first also loads the module's kernels
        ctx.sync()
        t0 = time.perf_counter()
        d = systems.ueg_recipe(w["N"], w["rs"], w["norb"], w["theta"], device_build=True)
        deri = d.device_aint_tot(ctx)
        fock_d, e1_d = d.g_fock_tot(), d.get_mp1()
        ctx.sync()
        out.append(time.perf_counter() - t0)
        deri.free()
    print(json.dumps({"system_build": args.workload, "n_spin_orbitals": n,
                      "host_dense_s": t_host, "device_s": out[-1],
                      "fock_max_diff": float(abs(fock - fock_d).max()),
                      "e1_diff": float(abs(e1 - e1_d))}))
    return 0


def run_gemm(args):
    """Time one contraction shape through kvft_gemm (device-resident operands)."""
    import numpy
    from kelvin_gb300 import _lib, ccsd
    M, N, K, B = (int(x) for x in args.gemm.split(","))
    ctx = _lib.context(0)
    prec, digits = ccsd.PRECISIONS[args.precision]
    digits = args.digits or digits
    rng = numpy.random.default_rng(0)
    A = _lib.DeviceArray.from_host(ctx, rng.standard_normal((B, M, K)))
    Bm = _lib.DeviceArray.from_host(ctx, rng.standard_normal((B, K, N)))
    C = _lib.DeviceArray(ctx, (B, M, N))

    def once():
        ctx.check(ctx.L.kvft_gemm(ctx.h, M, N, K, B, prec, digits, A.ptr, Bm.ptr, C.ptr),
                  "kvft_gemm")

    for _ in range(max(args.warmup, 1)):
        once()
    ctx.sync()
    ctx.profile_begin()
    ctx.record(0)
    for _ in range(args.steps):
        once()
    ctx.record(1)
    ctx.sync()
    prof = ctx.profile_end()
    ms = ctx.elapsed_ms(0, 1) / args.steps
    flops = 2.0 * M * N * K * B
    pairs = sum(l - 1 for l in range(2, digits + 1)) if args.precision != "fp64" else 1
    print(json.dumps({"gemm": [M, N, K, B], "precision": args.precision, "digits": digits,
                      "ms": ms, "fp64_equiv_tflops": flops / ms / 1e9,
                      "bf16_tflops_issued": flops * pairs / ms / 1e9 if pairs > 1 else None,
                      "breakdown_ms": {c: round(v[1] / args.steps, 4) for c, v in prof.items()}}))
    return 0


def run_esn(args):
    """The differentiation workload (UEG, 14 electrons, rs = 2, 33 plane waves
    = 66 spin orbitals, Theta = 0.5, ng = 16): E, S, N from the Lambda
    equations (one adjoint solve) and from central differences of Omega
    (four further solves), each timed end to end after the same FP64-grade
    solve, with their differences."""
    from kelvin_gb300 import _lib, ccsd as kccsd, systems
    ctx = _lib.context(0)
    s = systems.ueg_recipe(14, 2.0, 33, 0.5, device_build=True)
    out = {"workload": "ueg66_esn", "n_spin_orbitals": 66, "ngrid": 16}

    def solve():
        cc = kccsd.ccsd(s, T=s.T, mu=s.mu, ngrid=16, damp=0.5, econv=1e-10, max_iter=200,
                        precision="fp64_tc", ctx=ctx)
        cc.run()
        return cc
    for method in ("lambda", "fd"):
        cc = solve()
        t0 = time.perf_counter()
        E, S, N = cc.compute_ESN(method=method)
        out[method] = {"E": E, "S": S, "N": N, "seconds": time.perf_counter() - t0}
        cc.release()
    out["dE"] = out["lambda"]["E"] - out["fd"]["E"]
    out["dS"] = out["lambda"]["S"] - out["fd"]["S"]
    out["dN"] = out["lambda"]["N"] - out["fd"]["N"]
    print(json.dumps(out))
    return 0


def small_accuracy(ctx, args):
    """|dOmega|, |dE|, |dS| of the mixed form (as benchmarked) against Kelvin's
    damped FP64-accurate solve: UEG 14 electrons, rs = 4, 19 plane waves,
    Theta = 0.5, ng = 10 (Simpson), E and S from the Lambda equations."""
    from kelvin_gb300 import _lib, ccsd as kccsd, systems
    s = systems.ueg_recipe(14, 4.0, 19, 0.5, device_build=True)
    out = {}
    for prec, acc in (("fp64_tc", 0), ("mixed", args.accel)):
        cc = kccsd.ccsd(s, T=s.T, mu=s.mu, max_iter=200, damp=0.5, ngrid=10, econv=1e-10,
                        precision=prec, accel=acc, mix=args.mix if acc else None,
                        low_tconv=args.low_tconv if acc else None, ctx=ctx)
        try:
            Om = cc.run()[0]
            E, S, N = cc.compute_ESN(method="lambda")
            out[prec] = (Om, E, S)
        finally:
            cc.release()
            ctx.set_precision(_lib.PREC_FP64, 7)
    (o0, e0, s0), (o1, e1, s1) = out["fp64_tc"], out["mixed"]
    return {"abs_dOmega": abs(o1 - o0), "abs_dE": abs(e1 - e0), "abs_dS": abs(s1 - s0),
            "electrons": 14, "grid": "Simpson, ng = 10"}


def run_accuracy(args):
    """|dOmega|, |dE|, |dS| of the mixed form against the FP64-accurate form
    on the configurations small enough to differentiate in seconds: E, S from
    the Lambda equations on Kelvin's Simpson grid, from central differences
    of Omega on a Gauss-Legendre grid (both evaluate the derivative with
    FP64-accurate contractions, so the differences measure the mixed solve's
    amplitudes).  Also |dOmega| where the few-digit phases ended."""
    from kelvin_gb300 import _lib, ccsd as kccsd, systems
    ctx = _lib.context(0)
    cases = [
        ("ueg38 Simpson", systems.ueg_recipe(14, 4.0, 19, 0.5, device_build=True), 10, "lin",
         0.5),
        ("ueg38 Gauss-Legendre", systems.ueg_recipe(14, 4.0, 19, 0.5, device_build=True), 10,
         "gl", 0.5),
        ("ueg66 (differentiation config)", systems.ueg_recipe(14, 2.0, 33, 0.5,
                                                               device_build=True), 16, "lin",
         0.5),
    ]
    for beta in (1.0, 4.0, 10.0):
        cases.append(("hubbard16 beta=%g" % beta,
                      systems.hubbard_mf_recipe(16, 1.0, 4.0, beta, device_build=True), 40,
                      "lin", 0.5))
    out = []
    for name, s, ng, quad, damp in cases:
        res = {}
        for prec in ("fp64_tc", "mixed"):
            # the reference: Kelvin's damped loop; the mixed form: as benchmarked
            cc = kccsd.ccsd(s, T=s.T, mu=s.mu, max_iter=300, damp=damp, ngrid=ng,
                            econv=1e-10, quad=quad, precision=prec,
                            accel=args.accel if prec == "mixed" else 0,
                            mix=args.mix if prec == "mixed" and args.accel else None,
                            low_tconv=args.low_tconv if prec == "mixed" and args.accel
                            else None, ctx=ctx)
            t0 = time.perf_counter()
            try:
                cc.run()
                E, S, N = cc.compute_ESN(method="lambda" if quad == "lin" else "fd")
                res[prec] = {"omega": cc.Gtot, "omega_cc": cc.Gcc, "omega_low": cc.omega_low,
                             "E": E, "S": S,
                             "N": N, "iterations": cc.iterations + cc.iterations_refine,
                             "phases": getattr(cc, "phases", None),
                             "converged": bool(cc.converged),
                             "seconds": time.perf_counter() - t0}
            except Exception as e:          # a solve that diverges is reported as such
                res[prec] = {"error": str(e)}
            finally:
                cc.release()
                ctx.set_precision(_lib.PREC_FP64, 7)
        a, b = res["fp64_tc"], res["mixed"]
        row = {"config": name, "electrons": float(getattr(s, "N", 0.0)), "fp64_tc": a,
               "mixed": b}
        if "error" not in a and "error" not in b:
            row.update({"abs_dOmega": abs(b["omega"] - a["omega"]),
                        "abs_dOmega_low_phases": abs(b["omega_low"] - a["omega_cc"]),
                        "abs_dE": abs(b["E"] - a["E"]), "abs_dS": abs(b["S"] - a["S"])})
        out.append(row)
        print(json.dumps(row), flush=True)
    return 0


def run_serve(args):
    """A seeded Poisson stream of mixed requests (kelvin_gb300.serve): solves/s
    and p50/p99 latency, completion minus arrival."""
    from kelvin_gb300 import serve
    reqs = serve.request_stream(args.serve, rate=args.rate, seed=0)
    rep = serve.Server(precision=args.precision, slots=args.slots, accel=args.accel,
                       mix=args.mix if args.accel else None,
                       low_tconv=args.low_tconv if args.accel else None).serve(reqs)
    done = rep.pop("requests")
    fails = {}
    for d in done:
        if not d["ok"]:
            k = d.get("reason", "")[:60]
            fails[k] = fails.get(k, 0) + 1
    print(json.dumps(dict({"serve": args.serve, "rate_per_s": args.rate,
                           "precision": args.precision, "accel": args.accel,
                           "not_solved": fails}, **rep)))
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gemm", default="", help="M,N,K,batch: time one contraction shape")
    ap.add_argument("--system-build", action="store_true",
                    help="time the integrals' build on the host and on the device")
    ap.add_argument("--profile-step", action="store_true",
                    help="one warm-up and one profiled solver iteration")
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="kvft", choices=["kvft", "reference"])
    ap.add_argument("--workload", default="ueg114", choices=sorted(WORKLOADS))
    ap.add_argument("--precision", default="mixed", choices=["fp64", "fp64_tc", "mixed"])
    ap.add_argument("--digits", type=int, default=0)
    ap.add_argument("--serve", type=int, default=0,
                    help="serve this many requests of a seeded Poisson stream")
    ap.add_argument("--rate", type=float, default=20.0, help="request rate of --serve (1/s)")
    ap.add_argument("--slots", type=int, default=4, help="--serve: solves on the device at once")
    ap.add_argument("--esn", action="store_true",
                    help="E, S, N of the 66-spin-orbital UEG: Lambda route against differences")
    ap.add_argument("--accel", type=int, default=3,
                    help="Anderson depth of the iteration (0: Kelvin's damped update)")
    ap.add_argument("--mix", type=float, default=0.7,
                    help="Anderson mixing factor (with --accel)")
    ap.add_argument("--low-tconv", type=float, default=3e-4,
                    help="mixed form with --accel: end the few-digit phase once Kelvin's "
                         "residual measure is below this")
    ap.add_argument("--quad", default="gl", choices=["gl", "lin"],
                    help="tau grid: Gauss-Legendre (the configurations') or Kelvin's Simpson")
    ap.add_argument("--accuracy", action="store_true",
                    help="mixed against FP64-accurate on the smaller configurations")
    ap.add_argument("--records", default="",
                    help="--profile-step: write every timed scope (with GEMM shapes) here")
    args = ap.parse_args()
    w = WORKLOADS[args.workload]
    if args.accuracy:
        return run_accuracy(args)
    if args.serve:
        return run_serve(args)
    if args.esn:
        return run_esn(args)
    if args.gemm:
        return run_gemm(args)
    if args.profile_step:
        return run_profile_step(args, w)
    if args.system_build:
        return run_system_build(args, w)
    if args.impl == "reference":
        return run_reference(args, w)
    return run_gpu(args, w)


if __name__ == "__main__":
    sys.exit(main())
