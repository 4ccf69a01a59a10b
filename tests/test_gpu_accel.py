"""Anderson acceleration of the amplitude iteration
(kvft_solver_set_acceleration): the accelerated solve meets Kelvin's
convergence test at the damped iteration's fixed point, in fewer
iterations, for the FP64 forms and for the mixed form's digit ladder."""
import json
import os

import numpy
import pytest

from conftest import GOLDEN
from kelvin_gb300 import _lib, ccsd, systems

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("prec", ["fp64", "fp64_tc"])
def test_anderson_reaches_the_damped_fixed_point(ctx, prec):
    s = systems.UEGSystem(0.1, 2 * numpy.pi, 1.2, mu=0.1, norb=7)
    kw = dict(T=0.1, mu=0.1, max_iter=100, damp=0.2, ngrid=10, econv=1e-11, precision=prec,
              ctx=ctx)
    try:
        ref = ccsd.ccsd(s, **kw)
        E0 = ref.run()[1]
        ref.release()
        acc = ccsd.ccsd(s, accel=2, **kw)
        E1 = acc.run()[1]
        acc.release()
    finally:
        ctx.set_precision(_lib.PREC_FP64, 7)
    assert ref.converged and acc.converged
    # the same fixed point (Kelvin's golden -0.010750238811 was converged to
    # econv 1e-8; both solves here meet 1e-11 and sit 2.8e-9 from it)
    assert abs(E1 - E0) < 1e-9
    assert acc.iterations < ref.iterations


@pytest.mark.parametrize("prec,tol", [("fp64_tc", 1e-9), ("mixed", 1e-9)])
def test_anderson_gauss_legendre_vs_oracle(ctx, prec, tol):
    """The 38-spin-orbital configuration on its Gauss-Legendre grid."""
    meta = json.load(open(os.path.join(GOLDEN, "configs.json")))["ueg38_gl"]
    s = systems.ueg_recipe(14, 4.0, 19, 0.5)
    kw = dict(T=s.T, mu=s.mu, max_iter=100, damp=0.5, ngrid=meta["ngrid"], econv=1e-10,
              quad="gl", precision=prec, ctx=ctx)
    try:
        ref = ccsd.ccsd(s, **kw)
        ref.run()
        ref.release()
        acc = ccsd.ccsd(s, accel=2, **kw)
        Et, Ecc = acc.run()
        acc.release()
    finally:
        ctx.set_precision(_lib.PREC_FP64, 7)
    n_ref = ref.iterations + ref.iterations_refine
    n_acc = acc.iterations + acc.iterations_refine
    print("GL %s: damped %d iterations, Anderson %d; Omega_cc %.12f oracle %.12f"
          % (prec, n_ref, n_acc, Ecc, meta["omega_cc"]))
    assert acc.converged
    assert abs(Ecc - meta["omega_cc"]) < tol
    assert n_acc <= n_ref


@pytest.mark.parametrize("low_tconv", [1e-4, 3e-4])
def test_benchmarked_scheme_vs_oracle(ctx, low_tconv):
    """The mixed form as benchmarked (depth 3, mixing factor 0.7, the
    three-level phase cut at residual 3e-4, and the tighter cut 1e-4) on the
    38-spin-orbital Gauss-Legendre configuration: Kelvin's test passes at the
    oracle's fixed point."""
    meta = json.load(open(os.path.join(GOLDEN, "configs.json")))["ueg38_gl"]
    s = systems.ueg_recipe(14, 4.0, 19, 0.5)
    try:
        cc = ccsd.ccsd(s, T=s.T, mu=s.mu, max_iter=100, damp=0.5, ngrid=meta["ngrid"],
                       econv=1e-10, quad="gl", precision="mixed", accel=3, mix=0.7,
                       low_tconv=low_tconv, ctx=ctx)
        Et, Ecc = cc.run()
        cc.release()
    finally:
        ctx.set_precision(_lib.PREC_FP64, 7)
    print("benchmarked scheme: phases %s, Omega_cc %.12f oracle %.12f"
          % (cc.phases, Ecc, meta["omega_cc"]))
    assert cc.converged
    assert abs(Ecc - meta["omega_cc"]) < 1e-8


def test_history_layouts_agree(ctx):
    """The FP32 history in the compact spin order (spin blocks on) and over
    every element (off) give the same accelerated iterates; turning the spin
    blocks off mid-solve starts a new history in the full layout."""
    from kelvin_gb300.cc_utils import DeviceSolver
    from kelvin_gb300.quadrature import ft_quad
    s = systems.ueg_recipe(14, 4.0, 19, 0.5)
    beta = 1.0 / s.T
    ti, g, G = ft_quad(10, beta, "lin")
    ctx.set_precision(_lib.PREC_FP64, 7)
    hist = {}
    for on in (True, False):
        sv = DeviceSolver.from_system(ctx, s.g_energies_tot(), s.g_fock_tot(), s.g_aint_tot(),
                                      beta, s.mu, ti, g, G)
        try:
            assert (sv.spin_blocks(on) > 0) == on
            sv.set_acceleration(3)
            sv.guess(1)
            hist[on] = [sv.step(0.3) for _ in range(8)]
            if on:
                sv.spin_blocks(False)
                E, res = sv.step(0.3)
                assert numpy.isfinite(E) and res < hist[on][-1][1] * 10
        finally:
            sv.close()
    # the FP32 sums run in another order (the full layout adds the zero
    # elements), so the mixing coefficients agree to FP32 rounding only
    for (e1, r1), (e2, r2) in zip(hist[True], hist[False]):
        assert abs(e1 - e2) < 1e-8 and abs(r1 - r2) < 1e-4 * r2
