"""The benchmark configurations on the GPU.

* 114 spin orbitals (UEG, 38 electrons, rs = 1, 57 plane waves): one tau
  point of the residual (Kelvin's per-point _Stanton call,
  ft_cc_equations.py:105-107) against the oracle, through the spin-blocked
  contractions the solver runs, in every precision; and complete solves at
  Theta = 0.25 and 1.0, mixed against FP64-accurate.
* 38 spin orbitals (UEG, 14 electrons, rs = 4, 19 plane waves) on a
  Gauss-Legendre tau grid: the resident solver against the oracle's solve
  (dense G, the exponential for every node pair).
* The 16-site Hubbard ring in Kelvin's mean-field momentum basis: mixed and
  FP64-accurate solves against the oracle's grand potential.

The oracle's values for the last two are committed fixtures
(tests/golden/make_config_golden.py); the 114-spin-orbital oracle residual is
computed here on the host (about a minute on 16 cores, 15 GB).
"""
import json
import os

import numpy
import pytest

from conftest import GOLDEN
from kelvin_gb300 import _lib, ccsd, systems
from kelvin_gb300.ccsd import PRECISIONS
from kelvin_gb300.ft_cc_equations import F_ORDER, I_ORDER
from oracle import cc_equations, ft_ccsd as oft

pytestmark = pytest.mark.gpu


def _spin_amplitudes(rng, n, scale):
    """Antisymmetric t1[a,i], t2[a,b,i,j] that vanish outside the
    spin-conserving blocks of an alpha-first layout."""
    h = n // 2
    sp = numpy.arange(n) >= h
    t1 = rng.standard_normal((n, n)) * scale * (sp[:, None] == sp[None, :])
    t2 = rng.standard_normal((n, n, n, n)) * scale
    t2 -= t2.transpose(1, 0, 2, 3)
    t2 -= t2.transpose(0, 1, 3, 2)
    cons = (sp[:, None, None, None].astype(int) + sp[None, :, None, None]
            == sp[None, None, :, None].astype(int) + sp[None, None, None, :])
    t2 *= cons
    return t1, t2


@pytest.fixture(scope="module")
def c2_slice():
    """Host integrals, amplitudes and the oracle residual of one tau point of
    the 114-spin-orbital system at Theta = 0.25."""
    s = systems.ueg_recipe(38, 1.0, 57, 0.25)
    en = s.g_energies_tot()
    beta = 1.0 / s.T
    F, I = oft.ft_integrals(s.g_fock_tot(), s.g_aint_tot(), en, beta, s.mu)
    rng = numpy.random.default_rng(114)
    t1, t2 = _spin_amplitudes(rng, en.shape[0], 1e-2)
    R1, R2 = cc_equations.residual(F, I, t1, t2)
    return F, I, t1, t2, R1, R2


# Bars relative to the largest residual element (2.4e-2 here).  FP64 FMA:
# rounding.  Seven digit levels: ~3e-13 of K max|A| max|B| per contraction,
# K = n^2 = 13 000 (measured 3.5e-11, i.e. 9e-13 absolute, far inside the 1e-8
# max-abs amplitude bar).  Three levels (the mixed form's first phase): ~1e-5
# of K max|A| max|B|, which for these random-sign amplitudes is ~1e-3 of the
# largest element (measured 2.7e-3); its solves are held to the 1e-6 Ha per
# electron bar below instead.
@pytest.mark.parametrize("prec,spin,tol", [
    ("fp64_tc", True, 1e-9), ("fp64_tc", False, 1e-9), ("fp64", True, 1e-12),
    ("mixed", True, 1e-2)])
def test_c2_residual_slice_vs_oracle(ctx, c2_slice, prec, spin, tol):
    """kvft_stanton_residual at one tau point of the benchmarked system
    against the oracle's residual, relative to its largest element."""
    F, I, t1, t2, R1, R2 = c2_slice
    n = t1.shape[0]
    ctx.set_precision(*PRECISIONS[prec])
    ctx.set_residual_spin_blocks(n // 2 if spin else 0)
    try:
        dF = [_lib.DeviceArray.from_host(ctx, getattr(F, k)) for k in F_ORDER]
        dI = [_lib.DeviceArray.from_host(ctx, getattr(I, k)) for k in I_ORDER]
        d1, d2 = _lib.DeviceArray.from_host(ctx, t1), _lib.DeviceArray.from_host(ctx, t2)
        o1 = _lib.DeviceArray.from_host(ctx, numpy.zeros_like(t1))
        o2 = _lib.DeviceArray.from_host(ctx, numpy.zeros_like(t2))
        ctx.check(ctx.L.kvft_stanton_residual(ctx.h, 1, n, n, _lib.ptr_array(dF),
                                              _lib.ptr_array(dI), d1.ptr, d2.ptr, 1.0,
                                              o1.ptr, o2.ptr), "kvft_stanton_residual")
        g1, g2 = o1.to_host(), o2.to_host()
    finally:
        ctx.set_residual_spin_blocks(0)
        ctx.set_precision(_lib.PREC_FP64, 7)
        for a in dF + dI:
            a.free()
    e1 = abs(g1 - R1).max() / abs(R1).max()
    e2 = abs(g2 - R2).max() / abs(R2).max()
    print("C2 residual slice %s spin=%s: rel err R1 %.2e R2 %.2e (max|R2| %.3e)"
          % (prec, spin, e1, e2, abs(R2).max()))
    assert e1 < tol and e2 < tol
    if prec != "mixed":
        assert max(abs(g1 - R1).max(), abs(g2 - R2).max()) < 1e-8


@pytest.mark.parametrize("theta", [0.25, 1.0])
def test_c2_solve_mixed_vs_fp64(ctx, theta):
    """Complete solves of the benchmarked system (integrals built on the
    device): the mixed form converges by Kelvin's test through its
    FP64-accurate refinement and lands within 1e-6 Ha per electron of the
    FP64-accurate solve; its few-digit phases end within that bar too."""
    s = systems.ueg_recipe(38, 1.0, 57, theta, device_build=True)
    kw = dict(T=s.T, mu=s.mu, max_iter=100, damp=0.5, ngrid=20, econv=1e-10, ctx=ctx)
    try:
        ref = ccsd.ccsd(s, precision="fp64_tc", **kw)
        E64 = ref.run()[1]
        ref.release()
        mix = ccsd.ccsd(s, precision="mixed", **kw)
        Emx = mix.run()[1]
        mix.release()
    finally:
        ctx.set_precision(_lib.PREC_FP64, 7)
    print("C2 Theta=%.2f: Omega_cc fp64_tc %.12f (%d it), mixed %.12f (phases %s), low %.12f"
          % (theta, E64, ref.iterations, Emx, mix.phases, mix.omega_low))
    assert ref.converged and mix.converged
    assert abs(Emx - E64) < 1e-6 * s.N
    assert abs(mix.omega_low - E64) < 1e-6 * s.N


def test_c1_gauss_legendre_vs_oracle(ctx):
    """The resident solver on a Gauss-Legendre grid (dense G) against the
    oracle's solve of the same system and grid."""
    meta = json.load(open(os.path.join(GOLDEN, "configs.json")))["ueg38_gl"]
    s = systems.ueg_recipe(14, 4.0, 19, 0.5)
    for prec, tol in (("fp64_tc", 1e-10), ("fp64", 1e-10), ("mixed", 1e-6 * s.N)):
        cc = ccsd.ccsd(s, T=s.T, mu=s.mu, max_iter=100, damp=0.5, ngrid=meta["ngrid"],
                       econv=1e-10, quad="gl", precision=prec, ctx=ctx)
        try:
            Et, Ecc = cc.run()
        finally:
            ctx.set_precision(_lib.PREC_FP64, 7)
        assert cc.converged
        assert abs(Ecc - meta["omega_cc"]) < tol, (prec, Ecc, meta["omega_cc"])
        assert abs(Et - meta["omega"]) < tol


def test_hubbard16_vs_oracle(ctx):
    """The 16-site half-filled Hubbard ring (U = 4, mean-field momentum
    basis, ng = 40) at beta = 1: FP64-accurate against the oracle's grand
    potential and its Lambda-based E, S, N; mixed within 1e-6 Ha per electron
    of it."""
    meta = json.load(open(os.path.join(GOLDEN, "configs.json")))["hubbard16"]["1"]
    h = systems.hubbard_mf_recipe(16, 1.0, 4.0, 1.0, device_build=True)
    for prec, tol in (("fp64_tc", 1e-9), ("mixed", 1e-6 * h.N)):
        cc = ccsd.ccsd(h, T=h.T, mu=h.mu, max_iter=meta["max_iter"], damp=meta["damp"],
                       ngrid=meta["ngrid"], econv=1e-10, precision=prec, ctx=ctx)
        try:
            Et, Ecc = cc.run()
            E, S, N = cc.compute_ESN(method="lambda")
        finally:
            cc.release()
            ctx.set_precision(_lib.PREC_FP64, 7)
        print("Hubbard beta=1 %s: Omega_cc %.12f oracle %.12f; E %.10f S %.10f N %.10f"
              % (prec, Ecc, meta["omega_cc"], E, S, N))
        assert cc.converged
        assert abs(Ecc - meta["omega_cc"]) < tol
        assert abs(Et - meta["omega"]) < tol
        assert abs(E - meta["E"]) < 100 * tol and abs(N - meta["N"]) < 100 * tol
        assert abs(S - meta["S"]) < 1000 * tol


@pytest.mark.parametrize("beta", [4.0, 10.0])
def test_hubbard16_low_temperature_diverges(ctx, beta):
    """At beta = 4 and 10 the damped FT-CCSD iteration of this ring diverges
    (the oracle's does too, tests/golden/configs.json): the solver stops with
    Kelvin's error, not a wrong number, and the context stays usable."""
    h = systems.hubbard_mf_recipe(16, 1.0, 4.0, beta, device_build=True)
    cc = ccsd.ccsd(h, T=h.T, mu=h.mu, max_iter=200, damp=0.5, ngrid=40, econv=1e-10,
                   precision="fp64_tc", ctx=ctx)
    try:
        with pytest.raises(Exception, match="diverged"):
            cc.run()
    finally:
        cc.release()
        ctx.set_precision(_lib.PREC_FP64, 7)
    # the device is fine afterwards
    s = systems.hubbard_mf_recipe(8, 1.0, 2.0, 1.0, device_build=True)
    cc = ccsd.ccsd(s, T=s.T, mu=s.mu, max_iter=100, damp=0.5, ngrid=10, econv=1e-9, ctx=ctx)
    cc.run()
    assert cc.converged
    cc.release()
