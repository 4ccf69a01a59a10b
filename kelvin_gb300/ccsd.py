"""Finite-temperature CCSD driver, drop-in for kelvin.ccsd.ccsd (the FT
general-spin path, kelvin/ccsd.py:43-126 and 595-712).

    cc = ccsd(sys, T=T, mu=mu, damp=0.2, ngrid=10)
    Omega, Omega_cc = cc.run()

The system's integrals are uploaded once; integrals, tau grid and amplitudes
stay resident in HBM for the whole solve, and each iteration is one libkvft
call.  ``precision`` selects the contraction arithmetic ('fp64', 'fp64_tc',
'mixed'); quadrature, energy and damping are FP64 in every mode.
"""
import logging

import numpy

from . import _lib
from .cc_utils import DeviceSolver, ft_integrals, ft_lambda_iter, iterate
from .ft_cc_energy import ft_cc_energy
from .ft_cc_equations import (ccsd_lambda_guess, ccsd_stanton, g_to_u_t, kelvin_densities,
                              lambda_densities, normal_ordered_rdms, u_to_g_t1, u_to_g_t2)
from .quadrature import ft_quad
from .systems import fermi, grand_potential0

PRECISIONS = {'fp64': (_lib.PREC_FP64, 7), 'fp64_tc': (_lib.PREC_FP64_TC, 7),
              'mixed': (_lib.PREC_MIXED, 3)}


def converge(solver, ctx, conv, precision, digits, refine_sweeps=None, refine_digits=7,
             ladder=(5,), low_tconv=None):
    """Iterate a DeviceSolver to convergence; returns (Omega_cc, info).

    FP64 forms ('fp64', 'fp64_tc') run Kelvin's loop and test (|dE| < econv
    and res < tconv).  The mixed form runs the same damped update in phases
    of rising digit levels.  A few-digit update is a slightly discontinuous
    map (digit rounding), so each low phase ends at Kelvin's test or when
    the residual has stopped falling for three sweeps (its noise floor): first
    `digits` levels, then each level of `ladder`.  The refinement phase then
    re-evaluates the update with `refine_digits` levels (7: FP64-accurate)
    and iterates until Kelvin's test passes, at most `refine_sweeps` sweeps
    (None: the loop's max_iter).  Only that test counts as convergence: a
    stalled low phase does not.  `low_tconv` also ends each low phase once
    Kelvin's residual measure falls below it (the few-digit map's own fixed
    point is off the FP64 one by about its rounding, so sweeps below that
    level are not needed).  info: iterations (low phases),
    iterations_refine, converged, omega_low (the energy where the low phases
    ended) and phases, a list of (digit levels, sweeps, stalled)."""
    if precision != 'mixed':
        E = iterate(solver, conv, "CCSD")
        return E, {"iterations": solver.iterations, "iterations_refine": 0,
                   "converged": solver.converged, "omega_low": None,
                   "phases": [(digits, solver.iterations, False)]}
    prec = ctx_precision(ctx)
    phases = []
    low_iters = 0
    E_low = None
    converged = False
    try:
        for lv in (digits,) + tuple(l for l in ladder if digits < l < refine_digits):
            ctx.set_precision(_lib.PREC_MIXED if lv <= 3 else _lib.PREC_FP64_TC, lv)
            low = conv if low_tconv is None else dict(conv, econv=float("inf"), tconv=low_tconv)
            E_low = iterate(solver, low, "CCSD (%d digit levels)" % lv, stall=3, quiet=True)
            low_iters += solver.iterations
            phases.append((lv, solver.iterations, bool(solver.stalled)))
            if solver.converged and low_tconv is None:
                break
        ref = dict(conv)
        if refine_sweeps is not None:
            ref["max_iter"] = refine_sweeps
        ctx.set_precision(_lib.PREC_FP64_TC, refine_digits)
        E = iterate(solver, ref, "CCSD refinement")
        phases.append((refine_digits, solver.iterations, False))
        converged = solver.converged
        refine_iters = solver.iterations
    finally:
        ctx.set_precision(*prec)
    return E, {"iterations": low_iters, "iterations_refine": refine_iters,
               "converged": converged, "omega_low": E_low, "phases": phases}


def _d_integrals(h, eri, en, beta, mu, dbeta, dmu):
    """Directional derivatives (dF, dI, dfo) of the Fermi-scaled integrals
    (cc_utils.py:569-602) along (dbeta, dmu) at fixed orbital energies, with
    the mean-field Fock matrix h + sum_r <pr||qr> f_r following the
    occupations (ueg_scf_system.py:398-417, 481-493): closed forms from
    df/dmu = beta f (1-f), df/dbeta = -(e - mu) f (1-f)."""
    fo = fermi(beta, en, mu)
    fv = 1.0 - fo
    so, sv = numpy.sqrt(fo), numpy.sqrt(fv)
    rate = beta * dmu - (en - mu) * dbeta
    dfo = fo * fv * rate
    s = {'o': so, 'v': sv}
    ds = {'o': 0.5 * so * fv * rate, 'v': -0.5 * sv * fo * rate}
    fmo = h + numpy.einsum('prqr,r->pq', eri, fo) - numpy.diag(en)
    dfock = numpy.einsum('prqr,r->pq', eri, dfo)
    one = {}
    for b in ('oo', 'ov', 'vo', 'vv'):
        p, q, dp, dq = s[b[0]], s[b[1]], ds[b[0]], ds[b[1]]
        one[b] = dfock * numpy.outer(p, q) + fmo * (numpy.outer(dp, q) + numpy.outer(p, dq))
    two = {}
    for name in ('vvvv', 'vvvo', 'vovv', 'vvoo', 'vovo', 'oovv', 'vooo', 'ooov', 'oooo'):
        f = [s[c] for c in name]
        d = [ds[c] for c in name]
        acc = 0.0
        for k in range(4):
            v = [d[m] if m == k else f[m] for m in range(4)]
            acc = acc + numpy.einsum('p,q,r,s->pqrs', *v)
        two[name] = eri * acc
    from .cc_utils import one_e_blocks, two_e_blocks
    return one_e_blocks(**one), two_e_blocks(**two), dfo


def _lam_dot(L1, L2, X1, X2, w):
    """sum_y w_y <L_y, X_y> with Kelvin's factor 1/4 on doubles."""
    return (numpy.einsum('y,yia,yai->', w, L1, X1)
            + 0.25 * numpy.einsum('y,yijab,yabij->', w, L2, X2))


def esn_from_lambda(en, h, eri, beta, mu, ngrid, quad, T1, T2, L1, L2, omega, stanton, energy):
    """E, S, N from converged T and Lambda (kelvin/ccsd.py:167-214 with the
    exact grid derivative of 1075-1148).

    dOmega along (dbeta, dmu) is the Lagrangian's explicit derivative.  The
    residual and the energy are linear in the integrals, so the integral part
    is E(T; dF, dI) - (1/beta) sum_y g_y <L_y, Phi_y(dF, dI)>, where Phi is
    the amplitude update ``stanton`` (Kelvin's ccsd_stanton: the integrated
    -F.vo - R) evaluated with the derivative integrals; Kelvin's L is the
    negative adjoint and sum_s g_s <int_L(L)_s, X_s> = sum_y g_y <L_y,
    int_tbar(X)_y>.  The grid scales with beta (g, G, t proportional to it):
    the 1/beta of Omega_cc and the g derivative cancel, and the G and t
    derivatives are Phi with G/beta plus D times Phi with
    G[y,x] (t_x - t_y)/beta.  ``stanton(F, I, T1, T2, D1, D2, ti, ng, G)`` and
    ``energy(T1, T2, f, eri, g, beta)`` are the amplitude update and
    ft_cc_energy; ``omega`` the converged grand potential.
        N = -dOmega/dmu,  E = Omega + beta dOmega/dbeta + mu N,
        S = beta (E - Omega - mu N)"""
    ti, g, G = ft_quad(ngrid, beta, quad)
    ng = ngrid
    fo = fermi(beta, en, mu)
    D1 = en[:, None] - en[None, :]
    D2 = (en[:, None, None, None] + en[None, :, None, None] - en[None, None, :, None]
          - en[None, None, None, :])
    W = numpy.einsum('ijij->ij', eri)
    hd = numpy.diag(h) - en
    x = -beta * (en - mu)
    gp0 = -(numpy.maximum(x, 0.0) + numpy.log1p(numpy.exp(-numpy.abs(x)))) / beta

    def derivative(dbeta, dmu):
        dF, dI, dfo = _d_integrals(h, eri, en, beta, mu, dbeta, dmu)
        d0 = (-fo * dmu + (-gp0 / beta + (en - mu) * fo / beta) * dbeta).sum()
        d1 = hd @ dfo + fo @ W @ dfo
        X1, X2 = stanton(dF, dI, T1, T2, D1, D2, ti, ng, G)
        dcc = energy(T1, T2, dF.ov, dI.oovv, g, beta) - _lam_dot(L1, L2, X1, X2, g) / beta
        if dbeta != 0.0:
            F, I = _scaled(h, eri, en, beta, mu)
            P1, P2 = stanton(F, I, T1, T2, D1, D2, ti, ng, G / beta)
            Gt = G * (ti[None, :] - ti[:, None]) / beta
            Q1, Q2 = stanton(F, I, T1, T2, D1, D2, ti, ng, Gt)
            dcc -= dbeta * _lam_dot(L1, L2, P1 + D1[None] * Q1, P2 + D2[None] * Q2, g) / beta
        return d0 + d1 + dcc

    dO_dmu = derivative(0.0, 1.0)
    dO_dbeta = derivative(1.0, 0.0)
    N = -dO_dmu
    E = omega + beta * dO_dbeta + mu * N
    S = beta * (E - omega - mu * N)
    return E, S, N


def _scaled(h, eri, en, beta, mu):
    """Fermi-scaled blocks of the mean-field Fock matrix and the integrals
    (cc_utils.py:569-602), on the host."""
    from .cc_utils import one_e_blocks, two_e_blocks
    fo = fermi(beta, en, mu)
    s = {'o': numpy.sqrt(fo), 'v': numpy.sqrt(1.0 - fo)}
    fmo = h + numpy.einsum('prqr,r->pq', eri, fo) - numpy.diag(en)
    one = {b: fmo * numpy.outer(s[b[0]], s[b[1]]) for b in ('oo', 'ov', 'vo', 'vv')}
    two = {nm: eri * numpy.einsum('p,q,r,s->pqrs', *[s[c] for c in nm])
           for nm in ('vvvv', 'vvvo', 'vovv', 'vvoo', 'vovo', 'oovv', 'vooo', 'ooov', 'oooo')}
    return one_e_blocks(**one), two_e_blocks(**two)


def ctx_precision(ctx):
    """(precision, digits) last set on a context through set_precision."""
    return getattr(ctx, "_precision", (_lib.PREC_FP64, 7))


class ccsd(object):
    """Coupled cluster singles and doubles (CCSD) driver, T > 0."""

    def __init__(self, sys, T=0.0, mu=0.0, iprint=0, singles=True, econv=1e-8,
                 tconv=None, max_iter=40, damp=0.0, ngrid=10, realtime=False,
                 athresh=0.0, quad='lin', rt_iter="all", precision='fp64',
                 digits=None, refine_sweeps=None, refine_digits=None, ladder=None, accel=0,
                 mix=None, low_tconv=None, device=0, ctx=None):
        self.T = T
        self.mu = mu
        self.finite_T = T != 0
        self.iprint = iprint
        self.singles = singles
        self.econv = econv
        self.tconv = tconv if tconv is not None else 1000.0 * econv
        self.max_iter = max_iter
        self.damp = damp
        self.ngrid = ngrid
        self.realtime = True if self.finite_T else realtime
        self.athresh = athresh
        self.quad = quad
        self.rt_iter = rt_iter
        if precision not in PRECISIONS:
            raise Exception("Unrecognized precision: {}".format(precision))
        self.precision = precision
        self.digits = digits if digits is not None else PRECISIONS[precision][1]
        # mixed form: after the few-digit phases (digits, then each level of
        # `ladder`), sweeps with `refine_digits` levels until Kelvin's test
        # passes, at most refine_sweeps (None: max_iter).  Default 7
        # (FP64-accurate) with Kelvin's damped update; 6 with Anderson mixing,
        # whose refinement sweeps cost 13 % less at 6 levels and land on the
        # same Omega (1.2e-14 Ha apart at 114 spin orbitals; 6-level
        # contractions are within ~1e-11 of FP64 norm-wise)
        self.refine_sweeps = refine_sweeps
        self.refine_digits = refine_digits if refine_digits is not None else (6 if accel else 7)
        # Anderson depth of the amplitude iteration (0: Kelvin's damped update)
        # and its mixing factor (None: 1 - damp, the damped update's); the
        # fixed point does not depend on either
        self.accel = int(accel)
        self.mix = mix
        # mixed form: end each few-digit phase once Kelvin's residual measure
        # is below this (None: at its noise floor only)
        self.low_tconv = low_tconv
        # intermediate digit levels of the mixed form: with Kelvin's damped
        # update a 5-level phase shortens the FP64-accurate one; with Anderson
        # mixing (whose history restarts at every change of precision) going
        # straight from 3 to 7 levels takes fewer sweeps
        self.ladder = tuple(ladder) if ladder is not None else ((5,) if not accel else ())
        if not sys.verify(self.T, self.mu):
            raise Exception("Sytem temperature inconsistent with CC temp")
        if not self.finite_T:
            raise Exception("kelvin_gb300.ccsd: only the finite-temperature path is built")
        if not singles:
            raise Exception("kelvin_gb300.ccsd: only CCSD (singles=True) is built")
        if athresh > 0.0:
            raise Exception("kelvin_gb300.ccsd: active-space thresholds are not built")
        self.beta = 1.0 / T
        self.beta_max = self.beta
        self.ti, self.g, self.G = ft_quad(self.ngrid, self.beta_max, self.quad)
        self.sys = sys
        self.ctx = ctx or _lib.context(device)
        self.T1 = None
        self.T2 = None
        self._Tg = None          # general-spin amplitudes of the last solve
        self.solver = None
        self.L1 = None           # Lambda amplitudes (Kelvin's layout) once solved
        self.L2 = None
        self._Lg = None          # general-spin Lambda of the last Lambda solve

    def _unrestricted(self):
        """A system in Kelvin's unrestricted form (has_u()): it is solved in its
        general-spin form (alpha spin orbitals first, spin blocks found by the
        solver) and the amplitudes are given and returned per spin case,
        T1 = (T1a, T1b), T2 = (T2aa, T2ab, T2bb) (kelvin/ccsd.py:714-880)."""
        has_u = getattr(self.sys, "has_u", None)
        return bool(has_u and has_u() and hasattr(self.sys, "u_energies_tot"))

    def run(self, T1=None, T2=None):
        """Solve; returns (Omega_total, Omega_cc) like Kelvin."""
        logging.info('Running CCSD at an electronic temperature of %f K'
                     % (self.T * 315775.13))
        return self._ft_ccsd(T1in=T1, T2in=T2)

    def _ft_ccsd(self, T1in=None, T2in=None):
        beta = self.beta
        mu = self.mu
        en = self.sys.g_energies_tot()
        E0 = grand_potential0(beta, en, mu) + self.sys.const_energy()
        E1 = self.sys.get_mp1()
        prec, digits = PRECISIONS[self.precision][0], self.digits
        self.ctx.set_precision(prec, digits)
        if getattr(self.sys, "device_build", False):
            # integrals written on the GPU; no n^4 array on the host
            eri = self.sys.device_aint_tot(self.ctx)
            solver = DeviceSolver.from_system(self.ctx, en, self.sys.g_fock_tot(), eri, beta,
                                              mu, self.ti, self.g, self.G)
            eri.free()
        else:
            solver = DeviceSolver.from_system(self.ctx, en, self.sys.g_fock_tot(),
                                              self.sys.g_aint_tot(), beta, mu, self.ti,
                                              self.g, self.G)
        # a dense Gauss-Legendre G takes the exponential for every node pair
        solver.full = self.quad == 'gl'
        if self.accel:
            solver.set_acceleration(self.accel)
        self.solver = solver
        conv = {"econv": self.econv, "tconv": self.tconv, "max_iter": self.max_iter,
                "damp": self.damp}
        if self.rt_iter[0] != 'a' and T2in is None:
            # tau-pointwise schedule (ccsd.py:697-702 -> cc_utils.py:176-242)
            r = solver.run_point(conv)
            self.iterations = r.iterations
            self.iterations_refine = 0
            self.converged = bool(r.converged)
            self.omega_low = None
            self._Tg = solver.amplitudes()
            self.T1, self.T2 = self._Tg
            if self._unrestricted():
                na = self.sys.u_energies_tot()[0].shape[0]
                self.T1, self.T2 = g_to_u_t(self._Tg[0], self._Tg[1], na)
            Eccn = r.omega_cc
            self.G0, self.G1, self.Gcc, self.Gtot = E0, E1, Eccn, E0 + E1 + Eccn
            return (Eccn + E0 + E1, Eccn)
        if self.rt_iter[0] != 'a':
            logging.warning("Convergence scheme ({}) is ignored when amplitudes are given.".format(self.rt_iter))
        if T1in is not None and T2in is not None:
            if self._unrestricted():
                T1in = u_to_g_t1(*[numpy.asarray(x) for x in T1in])
                T2in = u_to_g_t2(*[numpy.asarray(x) for x in T2in])
            solver.set_amplitudes(T1in, T2in)
            E2 = solver.guess(2)
        else:
            E2 = solver.guess(1)
        logging.info('MP2 Energy: {:.10f}'.format(E2))
        if self.accel and self.mix is not None:
            conv["damp"] = 1.0 - self.mix
        # the host arrays of the amplitudes, their pages faulted in while the
        # device iterates
        ready = solver.prepare_amplitudes()
        Eccn, info = converge(solver, self.ctx, conv, self.precision, digits,
                              self.refine_sweeps, self.refine_digits, self.ladder,
                              self.low_tconv)
        self.iterations = info["iterations"]
        self.iterations_refine = info["iterations_refine"]
        self.converged = info["converged"]
        self.omega_low = info["omega_low"]
        self.phases = info.get("phases")
        self._Tg = solver.amplitudes(out=ready())
        self.T1, self.T2 = self._Tg
        if self._unrestricted():
            na = self.sys.u_energies_tot()[0].shape[0]
            self.T1, self.T2 = g_to_u_t(self._Tg[0], self._Tg[1], na)
        self.G0 = E0
        self.G1 = E1
        self.Gcc = Eccn
        self.Gtot = E0 + E1 + Eccn
        return (Eccn + E0 + E1, Eccn)

    def _ft_ccsd_lambda(self, L1=None, L2=None):
        """Solve the Lambda equations (kelvin/ccsd.py:882-961): Kelvin's guess
        (or the given L1, L2), then the damped iteration of
        cc_utils.ft_lambda_iter with each update on the GPU.  The updates use
        FP64-accurate contractions (seven digit levels on the tensor cores
        unless the solve ran on the FP64 pipe).  Stores self.L1, self.L2 --
        per spin case, (L1a, L1b) and (L2aa, L2ab, L2bb), for a system in the
        unrestricted form, which is solved in its general-spin form with the
        unrestricted driver's guess and residual measure
        (kelvin/ccsd.py:963-1073)."""
        if self.quad == 'gl':
            raise Exception("the Lambda equations are built for Kelvin's lower-triangular "
                            "grids; use compute_ESN(method='fd') on a Gauss-Legendre grid")
        u = self._unrestricted()
        na = self.sys.u_energies_tot()[0].shape[0] if u else None
        if self.T1 is None:
            self.run()
        T1, T2 = self._Tg if self._Tg is not None else (self.T1, self.T2)
        beta, mu, ng = self.beta, self.mu, self.ngrid
        en = numpy.asarray(self.sys.g_energies_tot(), dtype=float)
        prev = ctx_precision(self.ctx)
        prec = 'fp64_tc' if self.precision == 'mixed' else self.precision
        self.ctx.set_precision(*PRECISIONS[prec])
        conv = {"tconv": self.tconv, "max_iter": self.max_iter, "damp": self.damp}
        try:
            if self.solver is not None and (L1 is None or L2 is None):
                # the last solve's integrals and amplitudes are still resident
                self._Lg = self.solver.lambda_solve(conv, guess=2 if u else 1, measure_half=na)
                L1 = None
            else:
                F, I = ft_integrals(self.sys, en, beta, mu, ctx=self.ctx)
        finally:
            self.ctx.set_precision(*prev)
        if self.solver is not None and L1 is None:
            self.L1, self.L2 = self._Lg
            if u:
                self.L1, self.L2 = g_to_u_t(self._Lg[0], self._Lg[1], na)
            return self.L1, self.L2
        self.ctx.set_precision(*PRECISIONS[prec])
        try:
            if L1 is None or L2 is None:
                L1, L2 = ccsd_lambda_guess(F, I, T1, self.beta_max, ng, unrestricted=u)
            elif u:
                L1 = u_to_g_t1(*[numpy.asarray(x) for x in L1])
                L2 = u_to_g_t2(*[numpy.asarray(x) for x in L2])
            D1 = en[:, None] - en[None, :]
            self._Lg = ft_lambda_iter("CCSD", L1, L2, T1, T2, F, I, D1, None, self.g, self.G,
                                      self.beta_max, ng, self.ti, self.iprint, conv,
                                      ctx=self.ctx, spin_half=na)
        finally:
            self.ctx.set_precision(*prev)
        self.L1, self.L2 = self._Lg
        if u:
            self.L1, self.L2 = g_to_u_t(self._Lg[0], self._Lg[1], na)
        return self.L1, self.L2

    def compute_ESN(self, L1=None, L2=None, gderiv=True, delta=1e-4, method='fd'):
        """Energy, entropy and particle number (kelvin/ccsd.py:128-214).

        Kelvin differentiates the grand potential Omega(beta, mu) through the
        Lambda equations (an adjoint, plus the tau-grid derivative when
        gderiv=True), with the orbital energies fixed and the mean-field Fock
        matrix following the occupations.  Here the same derivatives are
        central finite differences of Omega itself: four further solves at
        (beta +- delta beta, mu) and (beta, mu +- delta T), warm-started from the
        converged amplitudes, with the grid nodes moving with beta as in
        Kelvin's gderiv=True form.  The few-digit mixed form is not smooth
        enough to difference, so its difference solves use seven digit levels.

            N = -dOmega/dmu,  E = d(beta Omega)/dbeta + mu N,
            S = beta (E - mu N - Omega)

        method='lambda' takes Kelvin's own route instead: the Lambda equations
        (_ft_ccsd_lambda, started from L1/L2 when given) and the Lagrangian's
        explicit derivative (esn_from_lambda), one adjoint solve in place of
        four further solves.  With 'fd', L1/L2 must be None."""
        if method == 'lambda':
            if not gderiv:
                raise Exception("kelvin_gb300.ccsd: only the exact-grid derivative "
                                "(gderiv=True)")
            if self.T1 is None:
                self.run()
            if self.L1 is None or L1 is not None:
                self._ft_ccsd_lambda(L1, L2)
            return self._esn_lambda()
        if method != 'fd':
            raise Exception("Unrecognized ESN method: {}".format(method))
        if L1 is not None or L2 is not None:
            raise Exception("kelvin_gb300.ccsd: Lambda amplitudes are not used "
                            "(E, S, N come from finite differences of Omega)")
        if not gderiv:
            raise Exception("kelvin_gb300.ccsd: only the exact-grid derivative (gderiv=True)")
        if self.T1 is None:
            self.run()
        Tg = self._Tg if self._Tg is not None else (self.T1, self.T2)
        en = self.sys.g_energies_tot()
        fock0 = self.sys.g_fock_tot()
        eri = self.sys.g_aint_tot()
        W = numpy.einsum('ijij->ij', eri)
        fo0 = fermi(self.beta, en, self.mu)
        # the mean-field Fock matrix follows the occupations, as in Kelvin's
        # relaxed occupation numbers (g_fock_d_den): F = h + sum_r <pr||qr> f_r
        Gd = numpy.einsum('prqr->pqr', eri)
        # E1 = sum_i (h_ii - e_i) f_i + 1/2 f W f with h = F - sum_r <pr||qr> f_r
        hd = numpy.diag(fock0) - Gd.diagonal(axis1=0, axis2=1).T @ fo0 - en
        prec = 'fp64_tc' if self.precision == 'mixed' else self.precision
        conv = {"econv": min(self.econv, 1e-12), "tconv": 1e3 * min(self.econv, 1e-12),
                "max_iter": max(self.max_iter, 200), "damp": self.damp}

        def omega(beta, mu):
            fo = fermi(beta, en, mu)
            fock = fock0 + Gd @ (fo - fo0)
            E0 = grand_potential0(beta, en, mu) + self.sys.const_energy()
            E1 = hd @ fo + 0.5 * fo @ W @ fo
            ti, g, G = ft_quad(self.ngrid, beta, self.quad)
            self.ctx.set_precision(*PRECISIONS[prec])
            solver = DeviceSolver.from_system(self.ctx, en, fock, eri, beta, mu, ti, g, G)
            solver.full = self.quad == 'gl'
            try:
                solver.set_amplitudes(*Tg)
                solver.guess(2)
                Ecc, _ = converge(solver, self.ctx, conv, prec, PRECISIONS[prec][1])
            finally:
                solver.close()
            return E0 + E1 + Ecc

        beta, mu = self.beta, self.mu
        db, dm = delta * beta, delta * self.T
        prev = ctx_precision(self.ctx)
        try:
            Om = omega(beta, mu)            # with the difference solves' settings
            Np = omega(beta, mu + dm)
            Nm = omega(beta, mu - dm)
            Bp = omega(beta + db, mu)
            Bm = omega(beta - db, mu)
        finally:
            self.ctx.set_precision(*prev)
        self.N = -(Np - Nm) / (2.0 * dm)
        self.E = ((beta + db) * Bp - (beta - db) * Bm) / (2.0 * db) + mu * self.N
        self.S = beta * (self.E - mu * self.N - Om)
        self._esn_parts()
        return self.E, self.S, self.N

    def _g_ft_rdms(self):
        """Response densities and normal-ordered RDMs from T and Lambda
        (kelvin/ccsd.py:1333-1432 _g_ft_1rdm / _g_ft_2rdm): dia, dba, dji, dai,
        P2, n1rdm, n2rdm.  The densities are evaluated on the GPU."""
        if self.L1 is None:
            self._ft_ccsd_lambda()
        T1, T2 = self._Tg if self._Tg is not None else (self.T1, self.T2)
        en = numpy.asarray(self.sys.g_energies_tot(), dtype=float)
        D1 = en[:, None] - en[None, :]
        prev = ctx_precision(self.ctx)
        prec = 'fp64_tc' if self.precision == 'mixed' else self.precision
        self.ctx.set_precision(*PRECISIONS[prec])
        try:
            if self.solver is not None:
                Fg, Ig = self.solver.lambda_densities(self._Lg[0], self._Lg[1])
            else:
                Fg, Ig = lambda_densities(T1, T2, self._Lg[0], self._Lg[1], D1, self.ti,
                                          self.ngrid, self.g, self.G, ctx=self.ctx)
        finally:
            self.ctx.set_precision(*prev)
        (self.dia, self.dba, self.dji, self.dai), self.P2 = kelvin_densities(Fg, Ig)
        fo = fermi(self.beta, en, self.mu)
        self.n1rdm, self.n2rdm = normal_ordered_rdms(self.beta, fo, 1.0 - fo,
                                                     (self.dia, self.dba, self.dji, self.dai),
                                                     self.P2)

    def _g_ft_1rdm(self):
        self._g_ft_rdms()

    def _g_ft_2rdm(self):
        self._g_ft_rdms()

    def full_1rdm(self, relax=False):
        """Unrelaxed one-particle density matrix: the normal-ordered part plus
        the Fermi-Dirac occupations (kelvin/ccsd.py:1988-2004, orbtype 'g')."""
        if relax:
            raise Exception("kelvin_gb300.ccsd: relaxed densities are not built")
        if getattr(self, "n1rdm", None) is None:
            self._g_ft_rdms()
        en = numpy.asarray(self.sys.g_energies_tot(), dtype=float)
        return self.n1rdm + numpy.diag(fermi(self.beta, en, self.mu))

    def full_2rdm(self, relax=False):
        """Unrelaxed two-particle density matrix (kelvin/ccsd.py:2008-2058,
        orbtype 'g'; cc_utils.py:2018-2024): the normal-ordered part plus the
        antisymmetrised products of the occupations with themselves and, with
        weight 1/2 each way, with the normal-ordered 1-RDM."""
        if relax:
            raise Exception("Relaxed 2-RDM is not implemented")
        if getattr(self, "n2rdm", None) is None:
            self._g_ft_rdms()
        en = numpy.asarray(self.sys.g_energies_tot(), dtype=float)
        f = numpy.diag(fermi(self.beta, en, self.mu))
        n1 = self.n1rdm
        rdm2 = self.n2rdm.copy()
        for a, b, w in ((f, f, 1.0), (f, n1, 0.5), (n1, f, 0.5)):
            x = numpy.einsum('pr,qs->pqrs', a, b)
            rdm2 += w * (x - x.transpose(0, 1, 3, 2))
        return rdm2

    def _esn_lambda(self):
        """E, S, N from the stored T and Lambda; the amplitude updates and
        energies of esn_from_lambda run on the GPU."""
        T1, T2 = self._Tg if self._Tg is not None else (self.T1, self.T2)
        en = numpy.asarray(self.sys.g_energies_tot(), dtype=float)
        eri = self.sys.g_aint_tot()
        fo0 = fermi(self.beta, en, self.mu)
        h = self.sys.g_fock_tot() - numpy.einsum('prqr,r->pq', eri, fo0)
        prev = ctx_precision(self.ctx)
        prec = 'fp64_tc' if self.precision == 'mixed' else self.precision
        self.ctx.set_precision(*PRECISIONS[prec])
        try:
            def stanton(F, I, T1, T2, D1, D2, ti, ng, G):
                return ccsd_stanton(F, I, T1, T2, D1, D2, ti, ng, G, ctx=self.ctx)

            def energy(T1, T2, f, eri_, g, beta):
                return ft_cc_energy(T1, T2, f, eri_, g, beta, ctx=self.ctx)
            self.E, self.S, self.N = esn_from_lambda(en, h, eri, self.beta, self.mu, self.ngrid,
                                                     self.quad, T1, T2, self._Lg[0],
                                                     self._Lg[1],
                                                     self.Gtot, stanton, energy)
        finally:
            self.ctx.set_precision(*prev)
        self._esn_parts()
        return self.E, self.S, self.N

    def _esn_parts(self):
        """Kelvin's split of E, S, N (kelvin/ccsd.py:193-214): the
        non-interacting part (E0, S0, N0) of Omega0 and the first-order part
        (E1, S1, N1) of Omega1 = sum_i (h_ii - e_i) f_i + 1/2 f W f, in closed
        form with the Fock matrix following the occupations; the CC part is
        the rest."""
        beta, mu = self.beta, self.mu
        en = numpy.asarray(self.sys.g_energies_tot(), dtype=float)
        eri = self.sys.g_aint_tot()
        fo = fermi(beta, en, mu)
        fv = 1.0 - fo
        W = numpy.einsum('ijij->ij', eri)
        hd = numpy.diag(self.sys.g_fock_tot()) - W @ fo - en
        G0 = grand_potential0(beta, en, mu) + self.sys.const_energy()
        G1 = hd @ fo + 0.5 * fo @ W @ fo
        self.N0 = fo.sum()
        self.E0 = en @ fo + self.sys.const_energy()
        self.S0 = beta * (self.E0 - G0 - mu * self.N0)
        grad = hd + W @ fo                       # dOmega1 / df
        self.N1 = -grad @ (beta * fo * fv)
        self.E1 = G1 + beta * (grad @ (-(en - mu) * fo * fv)) + mu * self.N1
        self.S1 = beta * (self.E1 - G1 - mu * self.N1)
        self.Ncc = self.N - self.N0 - self.N1
        self.Ecc = self.E - self.E0 - self.E1
        self.Scc = self.S - self.S0 - self.S1

    def release(self):
        """Free the device buffers of the last solve."""
        if self.solver is not None:
            self.solver.close()
            self.solver = None
