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
from .cc_utils import DeviceSolver, iterate
from .ft_cc_equations import g_to_u_t, u_to_g_t1, u_to_g_t2
from .quadrature import ft_quad
from .systems import fermi, grand_potential0

PRECISIONS = {'fp64': (_lib.PREC_FP64, 7), 'fp64_tc': (_lib.PREC_FP64_TC, 7),
              'mixed': (_lib.PREC_MIXED, 3)}


def converge(solver, ctx, conv, precision, digits, refine_sweeps=2, refine_digits=5):
    """Iterate a DeviceSolver to convergence; returns (Omega_cc, info).

    FP64 forms use Kelvin's test (|dE| < econv and res < tconv).  The mixed
    form's few-digit update is a slightly discontinuous map (digit rounding),
    so its iteration settles at a noise floor instead of meeting econv: it
    stops at Kelvin's test or when the residual has stopped falling for three
    sweeps, then runs `refine_sweeps` sweeps from that point with
    `refine_digits` digit levels (5: norm-wise ~1e-9 per contraction, far
    below the 1e-6 Ha per electron the mixed form answers to, at half the
    products of the FP64-grade 7)."""
    if precision != 'mixed':
        E = iterate(solver, conv, "CCSD")
        return E, {"iterations": solver.iterations, "iterations_refine": 0,
                   "converged": solver.converged, "omega_low": None}
    E_low = iterate(solver, conv, "CCSD", stall=3)
    info = {"iterations": solver.iterations, "iterations_refine": 0,
            "converged": solver.converged or getattr(solver, "stalled", False),
            "omega_low": E_low}
    E = E_low
    if refine_sweeps > 0:
        prec = ctx_precision(ctx)
        ctx.set_precision(_lib.PREC_FP64_TC, refine_digits)
        try:
            ref = dict(conv)
            ref["max_iter"] = refine_sweeps
            E = iterate(solver, ref, "CCSD refinement", quiet=True)
        finally:
            ctx.set_precision(*prec)
        info["iterations_refine"] = solver.iterations
    return E, info


def ctx_precision(ctx):
    """(precision, digits) last set on a context through set_precision."""
    return getattr(ctx, "_precision", (_lib.PREC_FP64, 7))


class ccsd(object):
    """Coupled cluster singles and doubles (CCSD) driver, T > 0."""

    def __init__(self, sys, T=0.0, mu=0.0, iprint=0, singles=True, econv=1e-8,
                 tconv=None, max_iter=40, damp=0.0, ngrid=10, realtime=False,
                 athresh=0.0, quad='lin', rt_iter="all", precision='fp64',
                 digits=None, refine_sweeps=2, refine_digits=5, device=0, ctx=None):
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
        # mixed form: sweeps re-evaluated with FP64-accurate contractions once
        # the few-digit iteration has converged (0: none)
        self.refine_sweeps = refine_sweeps
        self.refine_digits = refine_digits
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
        if self.quad == 'gl':
            raise Exception("the dense Gauss-Legendre G needs the full exp convention, "
                            "which the resident solver does not run")
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
        Eccn, info = converge(solver, self.ctx, conv, self.precision, digits,
                              self.refine_sweeps, self.refine_digits)
        self.iterations = info["iterations"]
        self.iterations_refine = info["iterations_refine"]
        self.converged = info["converged"]
        self.omega_low = info["omega_low"]
        self._Tg = solver.amplitudes()
        self.T1, self.T2 = self._Tg
        if self._unrestricted():
            na = self.sys.u_energies_tot()[0].shape[0]
            self.T1, self.T2 = g_to_u_t(self._Tg[0], self._Tg[1], na)
        self.G0 = E0
        self.G1 = E1
        self.Gcc = Eccn
        self.Gtot = E0 + E1 + Eccn
        return (Eccn + E0 + E1, Eccn)

    def compute_ESN(self, L1=None, L2=None, gderiv=True, delta=1e-4):
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

        L1/L2 (given Lambda amplitudes) have no counterpart and must be None."""
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
        prec = 'fp64_tc' if self.precision == 'mixed' else self.precision
        conv = {"econv": min(self.econv, 1e-12), "tconv": 1e3 * min(self.econv, 1e-12),
                "max_iter": max(self.max_iter, 200), "damp": self.damp}

        def omega(beta, mu):
            fo = fermi(beta, en, mu)
            fock = fock0 + Gd @ (fo - fo0)
            E0 = grand_potential0(beta, en, mu) + self.sys.const_energy()
            E1 = 0.5 * fo @ W @ fo
            ti, g, G = ft_quad(self.ngrid, beta, self.quad)
            self.ctx.set_precision(*PRECISIONS[prec])
            solver = DeviceSolver.from_system(self.ctx, en, fock, eri, beta, mu, ti, g, G)
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
        return self.E, self.S, self.N

    def release(self):
        """Free the device buffers of the last solve."""
        if self.solver is not None:
            self.solver.close()
            self.solver = None
