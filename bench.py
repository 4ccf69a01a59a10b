#!/usr/bin/env python
"""FT-CCSD solves/s on GB300 (libkvft) or on the host cores (reference arm).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl kvft|reference]
                    [--workload ueg114|ueg38] [--precision mixed|fp64_tc|fp64]
    python bench.py --gemm M,N,K,batch [--precision ...]      # one contraction shape
    python bench.py --system-build [--workload ...]
        # time building the model system's integrals: dense n^4 on the host
        # against kvft_ueg_eri on the device (closed-form Fock and E1)
    python bench.py --profile-step [--workload ...] [--precision ...]
        # one warm-up iteration, then one iteration; prints the library's
        # kernel-launch counts so that a profiler's launch list can be cut to
        # exactly the second iteration

Workloads are seeded synthetic uniform electron gases (the benchmark configs):

* ueg114 (default): 38 electrons, rs = 1, the 57 lowest plane waves (114 spin
  orbitals), Theta = 0.25, ng = 20, damping 0.5, econv 1e-10.  A full solve
  takes minutes, so a step is ONE amplitude iteration (CCSD update of all tau
  points + integration + damping + norms + energy) and
  solves/s = iterations/s / iterations_per_solve.
* ueg38: 14 electrons, rs = 4, 19 plane waves (38 spin orbitals), Theta = 0.5,
  ng = 10: a step is a complete solve (first-order guess to convergence).

``value`` times K steps with the integrals and buffers already resident in HBM;
``e2e`` times the same through the public drop-in API
(``kelvin_gb300.ccsd.ccsd(sys, ...).run()``) from host arrays, including the
host->device upload of the integrals and the read-back of the amplitudes.
The headline precision is 'mixed' (three BF16 digit levels on tensor cores;
FP64 quadrature, damping and energy); one FP64-accurate step is timed beside
it.  With N > 1 (torchrun) every rank runs an independent replica: only the
timings are reduced (gloo).  One JSON line is printed by rank 0.
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

# iters: amplitude iterations of the converged solve (guess 1), by precision;
# for 'mixed' the few-digit iterations before the REFINE refinement sweeps.
# ueg114 was measured by full solves on a GB300 (kelvin_gb300.ccsd.ccsd(...).run()):
# mixed 27 + 2 sweeps, Omega_cc -0.9542852803 (12.8 s); 7 levels 30, -0.9542857194.
WORKLOADS = {
    "ueg114": dict(N=38, rs=1.0, norb=57, theta=0.25, ng=20, damp=0.5, econv=1e-10,
                   max_iter=100, iters={"mixed": 27, "fp64_tc": 30, "fp64": 30},
                   step="iteration",
                   label="UEG 38 e-, rs=1, 57 plane waves (114 spin orbitals), Theta=0.25, "
                         "ng=20, damping 0.5, econv 1e-10"),
    "ueg38": dict(N=14, rs=4.0, norb=19, theta=0.5, ng=10, damp=0.5, econv=1e-10,
                  max_iter=100, iters=30, step="solve",
                  label="UEG 14 e-, rs=4, 19 plane waves (38 spin orbitals), Theta=0.5, "
                        "ng=10, damping 0.5, econv 1e-10"),
}
ITERS_FALLBACK = 30
# DRAM bytes per launch (dram__bytes_read.sum + dram__bytes_write.sum) of
# the contraction classes, mean over those launches of one ueg114 iteration,
# from the ncu launch lists of `python bench.py --profile-step [--precision
# fp64_tc]` (one replay pass per launch, so the full-size workload was
# captured).  A measured input of the roofline, not computed here: re-take
# it when the kernels change.
NCU_TRAFFIC = {
    ("ueg114", "mixed", "gemm6"): 2.4163e9, ("ueg114", "mixed", "gemm"): 1.5885e9,
    ("ueg114", "mixed", "elem"): 4.0275e9,
    ("ueg114", "fp64_tc", "gemm6"): 5.0731e9, ("ueg114", "fp64_tc", "gemm"): 1.8195e9,
    ("ueg114", "fp64_tc", "elem"): 3.1879e9,
}
REFINE = 2          # refinement sweeps that end a mixed solve
REFINE_DIGITS = 5   # their digit levels
STEP_EVENTS = 8     # first event slot of the per-step timings (at most 50 steps)


def iters_of(w, precision):
    it = w["iters"]
    if isinstance(it, dict):
        return it.get(precision, ITERS_FALLBACK)
    return it or ITERS_FALLBACK


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
# CPU reference: the oracle (numpy FP64 port of Kelvin's path) on host cores
# ---------------------------------------------------------------------------
def cpu_iteration_seconds(w, sysobj):
    """(seconds per amplitude iteration of the numpy FP64 path, sample text).

    n <= 40: one full iteration (ccsd_stanton over all tau points, int_tbar,
    damping, ft_cc_energy).  Larger n (a numpy iteration is many minutes):
    the W_abef ladder contraction of one tau point (2 n^6 flops, Kelvin's
    einsum 'efij,abef->abij'), scaled by the iteration's 10 n^6 ng flops."""
    import numpy
    from oracle import ft_ccsd, ft_utils, quadrature
    beta = 1.0 / sysobj.T
    en = sysobj.g_energies_tot()
    n, ng = en.shape[0], w["ng"]
    threads = os.cpu_count()
    if n <= 40:
        ti, g, G = quadrature.ft_quad(ng, beta, "lin")
        F, I = ft_ccsd.ft_integrals(sysobj.g_fock_tot(), sysobj.g_aint_tot(), en, beta,
                                    sysobj.mu)
        D1, D2 = ft_utils.D1(en, en), ft_utils.D2(en, en)
        T1 = numpy.zeros((ng, n, n))
        T2 = numpy.zeros((ng, n, n, n, n))
        t0 = time.perf_counter()
        T1n, T2n = ft_ccsd.ccsd_stanton(F, I, T1, T2, D1, D2, ti, ng, G)
        T1 = w["damp"] * T1 + (1 - w["damp"]) * T1n
        T2 = w["damp"] * T2 + (1 - w["damp"]) * T2n
        ft_ccsd.ft_cc_energy(T1, T2, F.ov, I.oovv, g, beta)
        dt = time.perf_counter() - t0
        return dt, "1 full amplitude iteration (numpy FP64 oracle port, %d threads, %.2f s)" % (
            threads, dt)
    rng = numpy.random.default_rng(0)
    W = rng.standard_normal((n * n, n * n))
    tau = rng.standard_normal((n * n, n * n))
    t0 = time.perf_counter()
    W @ tau
    dt = time.perf_counter() - t0
    it = dt * 5.0 * ng
    return it, ("one n^6 contraction of the iteration (W_abef ladder of one tau point, "
                "%d^2 x %d^2 x %d^2 FP64 BLAS via numpy, %d threads, %.2f s) scaled by "
                "10 n^6 ng / 2 n^6 = %d (n^5 terms and quadrature not counted: a lower "
                "bound on the CPU time)" % (n, n, n, threads, dt, 5 * ng))


def run_reference(args, w):
    ws, rank, _ = dist_setup()
    if rank != 0:
        return 0
    sysobj = build_system(w)
    iters = iters_of(w, "fp64")                           # the reference is FP64
    cpu_iteration_seconds(w, sysobj)                      # warm-up sample
    times, sample = [], ""
    for _ in range(args.steps):
        t, sample = cpu_iteration_seconds(w, sysobj)
        times.append(t)
    t_iter = statistics.median(times)
    value = 1.0 / (t_iter * iters)
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": UNIT,
            "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": t_iter * 1e3 * (iters if w["step"] == "solve" else 1),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic",
            "config": {"workload": w["label"], "step": w["step"],
                       "iterations_per_solve": iters,
                       "impl": "oracle numpy FP64 port of Kelvin's path (Kelvin is pure "
                               "Python and cannot run on the GPU host)"},
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": os.cpu_count(),
                             "kind": "port", "sample": "%d x %s; solves/s = 1 / (median "
                             "s/iteration x %d iterations)" % (args.steps, sample, iters)},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}
    print(json.dumps(line))
    return 0


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
    ti, g, G = ft_quad(w["ng"], beta, "lin")
    conv = {"econv": w["econv"], "tconv": 1000.0 * w["econv"], "max_iter": w["max_iter"],
            "damp": w["damp"]}
    n, ng = en.shape[0], w["ng"]
    per_solve = w["step"] == "solve"
    iters = iters_of(w, args.precision)

    ctx.set_precision(prec, digits)
    solver = DeviceSolver.from_system(ctx, en, fock, eri, beta, sysobj.mu, ti, g, G)
    solver.guess(1)

    def one_step():
        if per_solve:
            solver.guess(1)
            E, info = ccsd.converge(solver, ctx, conv, args.precision, digits, REFINE,
                                    REFINE_DIGITS)
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
    value = ws / (step_ms / 1e3) / (1 if per_solve else iters)
    if per_solve:
        iters = results[-1][1]

    # an FP64-accurate (7-level) step beside the headline precision, and for a
    # per-iteration workload the refinement sweep that ends a mixed solve
    fp64_step_ms = refine_step_ms = None
    if args.precision == "mixed":
        def timed_step(levels):
            ctx.set_precision(_lib.PREC_FP64_TC, levels)
            one_step()                                   # warm-up at this precision
            ctx.sync()
            ctx.record(4)
            one_step()
            ctx.record(5)
            ctx.sync()
            return ctx.elapsed_ms(4, 5)
        fp64_step_ms = timed_step(7)
        if not per_solve:
            refine_step_ms = timed_step(REFINE_DIGITS)
            # a mixed solve = iterations at few digits + the refinement sweeps
            value = ws / ((iters * step_ms + REFINE * refine_step_ms) / 1e3)
        ctx.set_precision(prec, digits)
    solver.close()

    # ---- end to end through the public API (e2e) -----------------------------
    barrier(ws)
    ctx.sync()
    t0 = time.perf_counter()
    ctx.record(2)
    # complete solves (one for the per-iteration workload) through the drop-in
    # driver from host arrays: integral upload, guess, iterations, refinement
    # sweeps and the read-back of all amplitudes
    n_e2e = args.steps if per_solve else 1
    for _ in range(n_e2e):
        cc = ccsd.ccsd(sysobj, T=sysobj.T, mu=sysobj.mu, max_iter=w["max_iter"],
                       damp=w["damp"], ngrid=ng, econv=w["econv"], precision=args.precision,
                       digits=digits, refine_sweeps=REFINE, refine_digits=REFINE_DIGITS,
                       ctx=ctx)
        cc.run()
        e2e_iters = cc.iterations + cc.iterations_refine
        cc.release()
    ctx.record(3)
    ctx.sync()
    e2e_ms = max(ctx.elapsed_ms(2, 3), (time.perf_counter() - t0) * 1e3)
    e2e_ms = max_over_ranks(ws, e2e_ms)
    e2e_value = ws * n_e2e / (e2e_ms / 1e3)
    h2d = 8 * (n + n * n + n ** 4 + 2 * ng + ng * ng)
    d2h = 8 * ng * (n * n + n ** 4) + 8 * 7 * (e2e_iters + 2)

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
                psrc = "nominal GB300 FP64 1.25 TFLOP/s (MEASURED_PEAKS.json has no FP64 figure)"
            else:
                pairs = sum(l - 1 for l in range(2, digits + 1))
                achieved *= pairs      # BF16 tensor flops issued per FP64-equivalent flop
                peak = peaks["bf16_tflops_sustained"]
                psrc = "bf16_tflops_sustained of %s peaks; achieved = algorithmic 2MNK flops " \
                       "x %d digit-pair products" % (peak_src, pairs)
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
    traffic = NCU_TRAFFIC.get((args.workload, args.precision, dom))
    roofline.update({
        "category": dom, "traffic": traffic,
        "traffic_unit": "bytes per launch (ncu dram__bytes_read.sum + dram__bytes_write.sum)"
                        if traffic else None,
        "categories": {c: {k: cats[c][k] for k in ("bound", "achieved", "unit", "frac")}
                       for c in cats if cats[c]},
        "breakdown_ms_per_step": {c: round(prof[c][1] / args.steps, 3) for c in prof}})

    t_iter, sample = cpu_iteration_seconds(w, sysobj)
    cpu_iters = iters_of(w, "fp64")                       # the CPU port is FP64
    cpu_val = 1.0 / (t_iter * cpu_iters)
    cfg = {"workload": w["label"], "step": w["step"], "precision": args.precision,
           "digits": digits if args.precision != "fp64" else None,
           "iterations_per_solve": iters, "omega_cc_last_step": results[-1][0],
           "l2": "per-step working set > 129 MB L2 (no flush)",
           "parallelism": "replicas" if ws > 1 else "single GPU"}
    if lat:
        q = lambda f: lat[min(len(lat) - 1, int(f * len(lat)))]
        cfg["step_latency_ms"] = {"p50": q(0.5), "p99": q(0.99), "n": len(lat)}
    if refine_step_ms is not None:
        cfg["refinement"] = {"sweeps": REFINE, "digit_levels": REFINE_DIGITS,
                             "step_ms": refine_step_ms}
    if fp64_step_ms is not None:
        cfg["fp64_tc_step_ms"] = fp64_step_ms
        cfg["fp64_tc_solves_per_s"] = ws / (fp64_step_ms / 1e3) / (1 if per_solve else iters)
        cfg["mixed_over_fp64_tc"] = fp64_step_ms / step_ms
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": step_ms,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f64" if args.precision != "mixed" else "bf16x3-digits/f32acc + f64",
            "data": "synthetic", "config": cfg, "roofline": roofline,
            "cpu_baseline": {"value": cpu_val, "unit": UNIT, "cores": os.cpu_count(),
                             "kind": "port", "sample": sample + "; x %d iterations" % cpu_iters},
            "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": h2d,
                    "d2h_bytes_per_step": d2h},
            "gpu_launches": launches, "clocks": clk}
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
    ti, g, G = ft_quad(w["ng"], beta, "lin")
    solver = DeviceSolver.from_system(ctx, s.g_energies_tot(), s.g_fock_tot(), s.g_aint_tot(),
                                      beta, s.mu, ti, g, G)
    solver.guess(1)
    solver.step(w["damp"])
    ctx.sync()
    l0 = ctx.launches()
    ctx.profile_begin()
    E, res = solver.step(w["damp"])
    ctx.sync()
    recs = ctx.profile_records()
    ctx.profile_end()
    # the category of each contraction of the step, in launch order: one
    # GEMM kernel (tc_gemm_kernel or gemm_f64_kernel) per contraction
    gemm_cats = [c for c, _, _ in recs if c in ("gemm6", "gemm")]
    print(json.dumps({"profile_step": args.workload, "precision": args.precision,
                      "launches_before": l0, "launches_in_step": ctx.launches() - l0,
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


def run_serve(args):
    """A seeded Poisson stream of mixed requests (kelvin_gb300.serve): solves/s
    and p50/p99 latency, completion minus arrival."""
    from kelvin_gb300 import serve
    reqs = serve.request_stream(args.serve, rate=args.rate, seed=0)
    rep = serve.Server(precision=args.precision).serve(reqs)
    rep.pop("requests")
    print(json.dumps(dict({"serve": args.serve, "rate_per_s": args.rate,
                           "precision": args.precision}, **rep)))
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
    ap.add_argument("--esn", action="store_true",
                    help="E, S, N of the 66-spin-orbital UEG: Lambda route against differences")
    args = ap.parse_args()
    w = WORKLOADS[args.workload]
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
