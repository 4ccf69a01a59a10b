"""Iteration and integral plumbing, drop-in for the FT general-spin parts of
kelvin/cc_utils.py.

* ``ft_integrals(sys, en, beta, mu)`` -- Fermi-scaled blocks, computed on the
  GPU (cc_utils.py:569-602);
* ``form_new_ampl`` -- method dispatch (cc_utils.py:17-49; CCSD only);
* ``ft_cc_iter`` -- the damped fixed-point loop (cc_utils.py:111-173) with
  every array resident on the device: each iteration is one libkvft call
  (update + integration + damping + norms + energy) and a 5-double read back.
"""
import ctypes
import logging
import time

import numpy

from . import _lib
from .ft_cc_equations import (F_ORDER, I_ORDER, _SpinBlocks, ccsd_stanton, device_blocks,
                              energies_from_d1, spin_half_of)


class one_e_blocks(object):
    """Attribute container .oo .ov .vo .vv."""

    def __init__(self, oo, ov, vo, vv):
        self.oo, self.ov, self.vo, self.vv = oo, ov, vo, vv


class two_e_blocks(object):
    """Attribute container for the nine antisymmetrised ERI blocks."""

    def __init__(self, vvvv=None, vvvo=None, vovv=None, vvoo=None, vovo=None,
                 oovv=None, vooo=None, ooov=None, oooo=None):
        self.vvvv, self.vvvo, self.vovv = vvvv, vvvo, vovv
        self.vvoo, self.vovo, self.oovv = vvoo, vovo, oovv
        self.vooo, self.ooov, self.oooo = vooo, ooov, oooo


def ft_integrals(sys, en, beta, mu, ctx=None):
    """One- and two-electron integrals scaled by sqrt(f) / sqrt(1-f)."""
    ctx = ctx or _lib.context()
    en = numpy.ascontiguousarray(en, dtype=float)
    n = en.shape[0]
    deps = _lib.DeviceArray.from_host(ctx, en)
    dfock = _lib.DeviceArray.from_host(ctx, sys.g_fock_tot())
    deri = _lib.DeviceArray.from_host(ctx, sys.g_aint_tot())
    F = [_lib.DeviceArray(ctx, (n, n)) for _ in range(4)]
    I = [_lib.DeviceArray(ctx, (n, n, n, n)) for _ in range(9)]
    ctx.check(ctx.L.kvft_ft_integrals(ctx.h, n, deps.ptr, dfock.ptr, deri.ptr, float(beta),
                                      float(mu), _lib.ptr_array(F), _lib.ptr_array(I)),
              "ft_integrals")
    return (one_e_blocks(**{b: a.to_host() for b, a in zip(F_ORDER, F)}),
            two_e_blocks(**{b: a.to_host() for b, a in zip(I_ORDER, I)}))


def form_new_ampl(method, F, I, T1old, T2old, D1, D2, ti, ng, G):
    """New amplitudes for ``method`` (only "CCSD" is on this path)."""
    if method == "CCSD":
        return ccsd_stanton(F, I, T1old, T2old, D1, D2, ti, ng, G)
    raise Exception("Unrecognized method keyword")


class DeviceSolver(object):
    """A kvft_solver: integrals, grid and amplitudes resident in HBM."""

    def __init__(self, ctx, handle, ng, nv, no):
        self.ctx = ctx
        self.h = handle
        self.ng, self.nv, self.no = ng, nv, no
        # tau-integral convention: False, Kelvin's (exp factor for x < y);
        # True, the dense-G convention of Gauss-Legendre grids (every x)
        self.full = False

    @classmethod
    def from_system(cls, ctx, en, fock, eri, beta, mu, ti, g, G):
        """``eri`` is a host array or a DeviceArray (n, n, n, n) already on the GPU."""
        en, fock, ti, g, G = (numpy.ascontiguousarray(a, dtype=float)
                              for a in (en, fock, ti, g, G))
        if isinstance(eri, _lib.DeviceArray):
            eri_ptr = eri.ptr
        else:
            eri = numpy.ascontiguousarray(eri, dtype=float)
            eri_ptr = eri.ctypes.data_as(_lib.vp)
        n, ng = en.shape[0], ti.shape[0]
        h = _lib.vp()
        ctx.check(ctx.L.kvft_solver_create(
            ctx.h, n, ng, en.ctypes.data_as(_lib.vp), fock.ctypes.data_as(_lib.vp),
            eri_ptr, float(beta), float(mu), ti.ctypes.data_as(_lib.vp),
            g.ctypes.data_as(_lib.vp), G.ctypes.data_as(_lib.vp), ctypes.byref(h)),
            "kvft_solver_create")
        return cls(ctx, h, ng, n, n)

    @classmethod
    def from_blocks(cls, ctx, F, I, D1, D2, beta, ti, g, G):
        Fa = [numpy.ascontiguousarray(getattr(F, b), dtype=float) for b in F_ORDER]
        Ia = [numpy.ascontiguousarray(getattr(I, b), dtype=float) for b in I_ORDER]
        D1, D2, ti, g, G = (numpy.ascontiguousarray(a, dtype=float) for a in (D1, D2, ti, g, G))
        nv, no = Fa[2].shape
        ng = ti.shape[0]
        Fp = (_lib.vp * 4)(*[a.ctypes.data_as(_lib.vp) for a in Fa])
        Ip = (_lib.vp * 9)(*[a.ctypes.data_as(_lib.vp) for a in Ia])
        h = _lib.vp()
        ctx.check(ctx.L.kvft_solver_create_blocks(
            ctx.h, nv, no, ng, Fp, Ip, D1.ctypes.data_as(_lib.vp), D2.ctypes.data_as(_lib.vp),
            float(beta), ti.ctypes.data_as(_lib.vp), g.ctypes.data_as(_lib.vp),
            G.ctypes.data_as(_lib.vp), ctypes.byref(h)), "kvft_solver_create_blocks")
        return cls(ctx, h, ng, nv, no)

    def spin_blocks(self, on=None):
        """Alpha-half size of the spin blocks the residual uses (0: none);
        ``on`` = False / True turns them off / back on (they are found at
        creation when the integrals are spin-blocked)."""
        h = ctypes.c_int()
        flag = -1 if on is None else int(bool(on))
        self.ctx.check(self.ctx.L.kvft_solver_set_spin_blocks(self.h, flag, ctypes.byref(h)),
                       "kvft_solver_set_spin_blocks")
        return h.value

    def set_amplitudes(self, T1, T2):
        T1 = numpy.ascontiguousarray(T1, dtype=float)
        T2 = numpy.ascontiguousarray(T2, dtype=float)
        self.ctx.check(self.ctx.L.kvft_solver_set_amplitudes(
            self.h, T1.ctypes.data_as(_lib.vp), T2.ctypes.data_as(_lib.vp)),
            "kvft_solver_set_amplitudes")

    def amplitudes(self, out=None):
        """Host copies (T1, T2).  ``out``: a (T1, T2) pair of C-contiguous
        float64 arrays of these shapes whose T2 holds zeros (e.g. from
        prepare_amplitudes), filled in place."""
        if out is None:
            T1 = numpy.empty((self.ng, self.nv, self.no))
            # zero pages until written: with spin blocks only the
            # spin-conserving elements are copied
            T2 = numpy.zeros((self.ng, self.nv, self.nv, self.no, self.no))
        else:
            T1, T2 = out
        self.ctx.check(self.ctx.L.kvft_solver_read_amplitudes(
            self.h, T1.ctypes.data_as(_lib.vp), T2.ctypes.data_as(_lib.vp), 1),
            "kvft_solver_read_amplitudes")
        return T1, T2

    def prepare_amplitudes(self):
        """Start a host thread that allocates the (T1, T2) arrays for
        amplitudes(out=...) and faults in the pages the read-back will write
        (the spin-conserving blocks of T2, or all of it), so that the first
        touch of tens of GB overlaps the iteration on the device instead of
        following it.  Returns a function that waits and returns the pair."""
        import threading
        shp1 = (self.ng, self.nv, self.no)
        shp2 = (self.ng, self.nv, self.nv, self.no, self.no)
        h = self.spin_blocks() if self.nv == self.no else 0
        box = {}

        def work():
            T1 = numpy.empty(shp1)
            T2 = numpy.zeros(shp2)
            if h:
                lo, hi = slice(0, h), slice(h, 2 * h)
                half = (lo, hi)
                for sa, sb, si, sj in ((0, 0, 0, 0), (1, 1, 1, 1), (0, 1, 0, 1),
                                       (0, 1, 1, 0), (1, 0, 0, 1), (1, 0, 1, 0)):
                    T2[:, half[sa], half[sb], half[si], half[sj]] = 0.0
            else:
                T2[...] = 0.0
            box["out"] = (T1, T2)

        th = threading.Thread(target=work, daemon=True)
        th.start()

        def wait():
            th.join()
            return box["out"]
        return wait

    def lambda_solve(self, conv_options, guess=1, L1=None, L2=None, measure_half=None,
                     history=None):
        """Kelvin's Lambda iteration (cc_utils.py:414-480) on the solver's
        resident integrals and converged amplitudes; guess 1 is Kelvin's
        starting Lambda, 2 its unrestricted driver's, 0 takes L1/L2.  Returns
        host (L1, L2)."""
        ng, nv, no = self.ng, self.nv, self.no
        if guess == 0:
            dL1 = _lib.DeviceArray.from_host(self.ctx, L1)
            dL2 = _lib.DeviceArray.from_host(self.ctx, L2)
        else:
            dL1 = _lib.DeviceArray(self.ctx, (ng, no, nv))
            dL2 = _lib.DeviceArray(self.ctx, (ng, no, no, nv, nv))
        max_iter = int(conv_options["max_iter"])
        hist = numpy.zeros(max(max_iter, 1))
        iters = ctypes.c_int()
        tbeg = time.time()
        self.ctx.check(self.ctx.L.kvft_solver_lambda(
            self.h, int(guess), float(conv_options["damp"]), float(conv_options["tconv"]),
            max_iter, int(measure_half or 0), dL1.ptr, dL2.ptr,
            hist.ctypes.data_as(_lib.vp), ctypes.byref(iters)), "kvft_solver_lambda")
        for i in range(iters.value):
            logging.info(' %2d  %.10f' % (i + 1, hist[i]))
        if history is not None:
            history.extend(float(x) for x in hist[:iters.value])
        if iters.value == 0 or hist[iters.value - 1] >= conv_options["tconv"]:
            logging.warning("CCSD Lambda-equations did not converge!")
        logging.info("Total CCSD Lambda time: %f s" % (time.time() - tbeg))
        return dL1.to_host(), dL2.to_host()

    def lambda_densities(self, L1, L2):
        """Integral gradients (Fg, Ig) of the Lagrangian at the solver's
        amplitudes and the given Lambda (kvft_solver_lambda_densities)."""
        nv, no = self.nv, self.no
        shp1 = {"oo": (no, no), "ov": (no, nv), "vo": (nv, no), "vv": (nv, nv)}
        ext = {"o": no, "v": nv}
        oF = [_lib.DeviceArray(self.ctx, shp1[b]) for b in F_ORDER]
        oI = [_lib.DeviceArray(self.ctx, tuple(ext[c] for c in b)) for b in I_ORDER]
        dL1 = _lib.as_device(self.ctx, L1)
        dL2 = _lib.as_device(self.ctx, L2)
        self.ctx.check(self.ctx.L.kvft_solver_lambda_densities(
            self.h, dL1.ptr, dL2.ptr, _lib.ptr_array(oF), _lib.ptr_array(oI)),
            "kvft_solver_lambda_densities")
        return [a.to_host() for a in oF], [a.to_host() for a in oI]

    def guess(self, kind, damp=0.0):
        """kind 0: zeros, 1: Kelvin's first-order guess, 2: keep.  Runs zero
        iterations and returns the guess energy (Qterm = False)."""
        o = _lib.SolveOpts(econv=0.0, tconv=0.0, damp=damp, max_iter=0, full=int(self.full),
                           guess=int(kind), verbose=0)
        r = _lib.Result()
        st = self.ctx.L.kvft_solver_run(self.h, ctypes.byref(o), ctypes.byref(r))
        if st not in (0, 6):
            self.ctx.check(st, "kvft_solver_run(guess)")
        return r.e_guess

    def run_point(self, conv_options, verbose=False):
        """Kelvin's tau-pointwise schedule on the device; returns the Result."""
        if self.full:
            raise Exception("the pointwise schedule needs a lower-triangular G")
        o = _lib.SolveOpts(econv=float(conv_options["econv"]), tconv=float(conv_options["tconv"]),
                           damp=float(conv_options["damp"]),
                           max_iter=int(conv_options["max_iter"]), full=0, guess=0,
                           verbose=int(bool(verbose)))
        r = _lib.Result()
        st = self.ctx.L.kvft_solver_run_point(self.h, ctypes.byref(o), ctypes.byref(r))
        if st not in (0, 6):
            self.ctx.check(st, "kvft_solver_run_point")
        self.iterations = r.iterations
        self.converged = bool(r.converged)
        if not r.converged:
            logging.warning("CCSD did not converge!")
        return r

    def step(self, damp):
        E = ctypes.c_double()
        res = ctypes.c_double()
        self.ctx.check(self.ctx.L.kvft_solver_step(self.h, float(damp), ctypes.byref(E),
                                                   ctypes.byref(res)), "kvft_solver_step")
        return E.value, res.value

    def set_acceleration(self, depth):
        """Anderson mixing of the given depth (1-3) in place of Kelvin's damped
        update; 0 restores the damped update."""
        self.ctx.check(self.ctx.L.kvft_solver_set_acceleration(self.h, int(depth)),
                       "kvft_solver_set_acceleration")

    def set_graph(self, on=None):
        """CUDA-graph replay of the damped iteration (True / False; None
        leaves it); returns the state: 2 replaying, -1 a capture failed, 0
        otherwise."""
        st = ctypes.c_int()
        flag = -1 if on is None else int(bool(on))
        self.ctx.check(self.ctx.L.kvft_solver_set_graph(self.h, flag, ctypes.byref(st)),
                       "kvft_solver_set_graph")
        return st.value

    def step_begin(self, damp):
        """Queue one iteration on the context's stream and return at once."""
        self.ctx.check(self.ctx.L.kvft_solver_step_begin(self.h, float(damp)),
                       "kvft_solver_step_begin")

    def step_end(self):
        """Wait for the queued iteration; (energy, residual)."""
        E = ctypes.c_double()
        res = ctypes.c_double()
        self.ctx.check(self.ctx.L.kvft_solver_step_end(self.h, ctypes.byref(E),
                                                       ctypes.byref(res)),
                       "kvft_solver_step_end")
        return E.value, res.value

    def close(self):
        if self.h:
            self.ctx.L.kvft_solver_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def iterate(solver, conv_options, method="CCSD", stall=0, quiet=False):
    """The loop of cc_utils.py:131-173 on a DeviceSolver; returns Eold.

    ``stall`` > 0 also stops when the residual has not fallen below 0.9 of
    its best value for that many sweeps (a low-precision noise floor);
    ``quiet`` drops the non-convergence warning (fixed sweep counts)."""
    tbeg = time.time()
    ethresh = conv_options["econv"]
    tthresh = conv_options["tconv"]
    max_iter = conv_options["max_iter"]
    alpha = conv_options["damp"]
    converged = False
    stalled = False
    best, since = float("inf"), 0
    Eold = 888888888.888888888
    i = 0
    while i < max_iter and not converged and not stalled:
        E, res = solver.step(alpha)
        logging.info(' %2d  %.10f   %.4E' % (i + 1, E, res))
        i += 1
        if numpy.abs(E - Eold) < ethresh and res < tthresh:
            converged = True
        if stall:
            if res < 0.9 * best:
                best, since = res, 0
            else:
                since += 1
                stalled = since >= stall
        Eold = E
    if not converged and not stalled and not quiet:
        logging.warning("{} did not converge!".format(method))
    logging.info("Total {} time: {:.4f} s".format(method, time.time() - tbeg))
    solver.iterations = i
    solver.converged = converged
    solver.stalled = stalled
    return Eold


def ft_cc_iter(method, T1old, T2old, F, I, D1, D2, g, G, beta, ng, ti, iprint,
               conv_options, ctx=None):
    """Damped FT-CC iteration (cc_utils.py:111-173); returns (E, T1, T2)."""
    if method != "CCSD":
        raise Exception("Unrecognized method keyword")
    ctx = ctx or _lib.context()
    solver = DeviceSolver.from_blocks(ctx, F, I, D1, D2, beta, ti, g, G)
    try:
        solver.set_amplitudes(T1old, T2old)
        E = iterate(solver, conv_options, method)
        T1, T2 = solver.amplitudes()
    finally:
        solver.close()
    return E, T1, T2


def ft_cc_iter_extrap(method, F, I, D1, D2, g, G, beta, ng, ti, iprint, conv_options,
                      ctx=None):
    """Grid-point-by-grid-point convergence (cc_utils.py:176-242) on the
    device; returns (T1, T2)."""
    if method != "CCSD":
        raise Exception("Unrecognized method keyword")
    ctx = ctx or _lib.context()
    solver = DeviceSolver.from_blocks(ctx, F, I, D1, D2, beta, ti, g, G)
    try:
        solver.run_point(conv_options)
        T1, T2 = solver.amplitudes()
    finally:
        solver.close()
    return T1, T2


def ft_lambda_iter(method, L1old, L2old, T1, T2, F, I, D1, D2, g, G, beta, ng, ti, iprint,
                   conv_options, ctx=None, update=None, history=None, spin_half=None):
    """Damped Lambda iteration (cc_utils.py:414-480); returns (L1, L2).

    The whole loop runs on the GPU (kvft_lambda_solve): each iteration is
    one device update, damping and Kelvin's residual measure,
    res = |L - L_old| / (|L_old| + 0.1) summed over L1 and L2, and the loop
    stops below tconv or at max_iter.  ``spin_half`` (alpha spin orbitals
    first) uses the unrestricted driver's measure over the spin cases
    (cc_utils.py:482-560).  ``update`` runs the same loop on the host around
    a given update (ccsd_lambda_opt's signature without ctx); ``history``
    receives the residual of each iteration."""
    if method != "CCSD":
        raise Exception("Unrecognized method keyword")
    if update is None:
        return _lambda_solve_device(ctx or _lib.context(), L1old, L2old, T1, T2, F, I, D1, g,
                                    G, ng, ti, conv_options, history, spin_half)
    tbeg = time.time()
    thresh = conv_options["tconv"]
    max_iter = conv_options["max_iter"]
    alpha = conv_options["damp"]
    L1old, L2old = numpy.array(L1old, dtype=float), numpy.array(L2old, dtype=float)
    nl1, nl2 = _lambda_norms(L1old, L2old, spin_half)
    converged = False
    i = 0
    while i < max_iter and not converged:
        L1, L2 = update(F, I, T1, T2, L1old, L2old, D1, D2, ti, ng, g, G, beta)
        res = _lambda_res(L1, L2, L1old, L2old, nl1, nl2, spin_half)
        L1old = alpha * L1old + (1.0 - alpha) * L1
        L2old = alpha * L2old + (1.0 - alpha) * L2
        nl1, nl2 = _lambda_norms(L1old, L2old, spin_half)
        logging.info(' %2d  %.10f' % (i + 1, res))
        if history is not None:
            history.append(res)
        i += 1
        if res < thresh:
            converged = True
    if not converged:
        logging.warning("CCSD Lambda-equations did not converge!")
    logging.info("Total CCSD Lambda time: %f s" % (time.time() - tbeg))
    return L1old, L2old


def _spin_cases(L1, L2, na):
    a, b = slice(0, na), slice(na, None)
    return ((L1[:, a, a], L1[:, b, b]),
            (L2[:, a, a, a, a], L2[:, a, b, a, b], L2[:, b, b, b, b]))


def _lambda_norms(L1, L2, na):
    nrm = numpy.linalg.norm
    if na is None:
        return nrm(L1) + 0.1, nrm(L2) + 0.1
    (l1a, l1b), (l2aa, l2ab, l2bb) = _spin_cases(L1, L2, na)
    return nrm(l1a) + nrm(l1b) + 0.1, nrm(l2aa) + nrm(l2bb) + 4 * nrm(l2ab) + 0.1


def _lambda_res(L1, L2, L1old, L2old, nl1, nl2, na):
    nrm = numpy.linalg.norm
    if na is None:
        return nrm(L1 - L1old) / nl1 + nrm(L2 - L2old) / nl2
    d1, d2 = _spin_cases(L1 - L1old, L2 - L2old, na)
    return sum(nrm(x) for x in d1) / nl1 + sum(nrm(x) for x in d2) / nl2


def _lambda_solve_device(ctx, L1, L2, T1, T2, F, I, D1, g, G, ng, ti, conv, history,
                         spin_half):
    """ft_lambda_iter resident on the device (kvft_lambda_solve)."""
    tbeg = time.time()
    blk = device_blocks(ctx, F, I)
    ev, eo = energies_from_d1(D1)
    dT1, dT2 = _lib.as_device(ctx, T1), _lib.as_device(ctx, T2)
    dL1 = _lib.DeviceArray.from_host(ctx, numpy.asarray(L1, dtype=float))
    dL2 = _lib.DeviceArray.from_host(ctx, numpy.asarray(L2, dtype=float))
    dv = [_lib.as_device(ctx, numpy.ascontiguousarray(a, dtype=float))
          for a in (ev, eo, ti, g, G)]
    max_iter = int(conv["max_iter"])
    hist = numpy.zeros(max(max_iter, 1))
    iters = ctypes.c_int()
    blocks = [getattr(F, b) for b in F_ORDER] + [getattr(I, b) for b in I_ORDER]
    h = spin_half_of(blk.nv, blk.no, blocks + [T1, T2, L1, L2])
    with _SpinBlocks(ctx, h):
        ctx.check(ctx.L.kvft_lambda_solve(ctx.h, ng, blk.nv, blk.no, blk.Fp, blk.Ip, dT1.ptr,
                                          dT2.ptr, dv[0].ptr, dv[1].ptr, dv[2].ptr, dv[3].ptr,
                                          dv[4].ptr, float(conv["damp"]), float(conv["tconv"]),
                                          max_iter, int(spin_half or 0), dL1.ptr, dL2.ptr,
                                          hist.ctypes.data_as(ctypes.c_void_p),
                                          ctypes.byref(iters)), "lambda_solve")
    for i in range(iters.value):
        logging.info(' %2d  %.10f' % (i + 1, hist[i]))
    if history is not None:
        history.extend(float(x) for x in hist[:iters.value])
    if iters.value == 0 or hist[iters.value - 1] >= conv["tconv"]:
        logging.warning("CCSD Lambda-equations did not converge!")
    logging.info("Total CCSD Lambda time: %f s" % (time.time() - tbeg))
    return dL1.to_host(), dL2.to_host()
