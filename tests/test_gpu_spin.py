"""Spin blocks: a solver whose integrals vanish outside the spin-conserving
blocks (alpha spin orbitals first, the general-spin ordering of the UEG and
Hubbard builders) runs its n^6 contractions over the 10 nonzero spin-block
products of 64.  The iterates must be those of the full contractions."""
import numpy
import pytest

from kelvin_gb300 import _lib, systems
from kelvin_gb300.cc_utils import DeviceSolver
from kelvin_gb300.quadrature import ft_quad

pytestmark = pytest.mark.gpu


def solver_for(ctx, s, ng=10):
    beta = 1.0 / s.T
    ti, g, G = ft_quad(ng, beta, "lin")
    return DeviceSolver.from_system(ctx, s.g_energies_tot(), s.g_fock_tot(), s.g_aint_tot(),
                                    beta, s.mu, ti, g, G)


def iterate(sv, on, steps=6):
    assert (sv.spin_blocks(on) > 0) == on
    sv.guess(1)
    hist = [sv.step(0.5) for _ in range(steps)]
    T1, T2 = sv.amplitudes()
    return hist, T1, T2


UEG = lambda: systems.ueg_recipe(14, 4.0, 19, 0.5)
# a Hubbard ring whose damped iteration grows (amplitudes reach ~5e4): in
# FP64 the two forms agree to rounding; with digit-sliced contractions the
# spin sub-blocks take their own row exponents, and the growing iteration
# amplifies those last-digit differences (~2e-9 relative after six steps
# at seven levels); three digit levels are compared on the UEG
HUB = lambda: systems.HubbardRing(0.3, 6, t=1.0, U=2.0, mu=0.4)


@pytest.mark.parametrize("make,prec,digits,tol", [
    (UEG, _lib.PREC_FP64, 7, 1e-12), (UEG, _lib.PREC_FP64_TC, 7, 1e-11),
    (UEG, _lib.PREC_FP64_TC, 3, 2e-4),
    (HUB, _lib.PREC_FP64, 7, 1e-12), (HUB, _lib.PREC_FP64_TC, 7, 1e-8)])
def test_spin_blocks_match_full_contractions(ctx, make, prec, digits, tol):
    s = make()
    sv = solver_for(ctx, s)
    try:
        ctx.set_precision(prec, digits)
        assert sv.spin_blocks() == s.g_energies_tot().shape[0] // 2
        h_on, T1_on, T2_on = iterate(sv, True)
        h_off, T1_off, T2_off = iterate(sv, False)
    finally:
        ctx.set_precision(_lib.PREC_FP64, 7)
        sv.close()
    scale = max(abs(T2_off).max(), 1e-3)
    assert abs(T2_on - T2_off).max() < tol * scale
    assert abs(T1_on - T1_off).max() < tol * max(abs(T1_off).max(), 1e-3)
    for (e1, r1), (e0, r0) in zip(h_on, h_off):
        assert abs(e1 - e0) < tol * max(abs(e0), 1e-3)
    # the spin-forbidden blocks of T2 stay exactly zero
    n = T2_on.shape[1]
    sp = numpy.arange(n) >= n // 2
    cons = (sp[:, None, None, None].astype(int) + sp[None, :, None, None]
            == sp[None, None, :, None].astype(int) + sp[None, None, None, :])
    assert not T2_on[:, ~cons].any()


def test_spin_blocks_off_for_a_generic_system(ctx):
    """Random integrals have no spin blocks: the solver finds none."""
    rng = numpy.random.default_rng(5)
    n = 8
    en = numpy.sort(rng.standard_normal(n))
    fock = numpy.diag(en)
    eri = rng.standard_normal((n, n, n, n)) * 0.05
    eri = eri - eri.transpose(0, 1, 3, 2)
    eri = eri - eri.transpose(1, 0, 2, 3)
    ti, g, G = ft_quad(6, 2.0, "lin")
    sv = DeviceSolver.from_system(ctx, en, fock, eri, 2.0, 0.0, ti, g, G)
    try:
        assert sv.spin_blocks() == 0
        assert sv.spin_blocks(True) == 0
    finally:
        sv.close()


def test_spin_breaking_amplitudes_turn_blocks_off(ctx):
    s = systems.ueg_recipe(14, 4.0, 19, 0.5)
    sv = solver_for(ctx, s)
    try:
        h = sv.spin_blocks()
        assert h > 0
        sv.guess(1)
        T1, T2 = sv.amplitudes()
        T2 = T2.copy()
        T2[0, 0, h, 0, 0] = 1e-3          # a <alpha beta || alpha alpha> element
        sv.set_amplitudes(T1, T2)
        assert sv.spin_blocks() == 0
    finally:
        sv.close()


@pytest.mark.parametrize("spin", [True, False])
def test_staged_read_back_is_exact(ctx, spin):
    """kvft_solver_read_amplitudes (pinned staging, host threads; with spin
    blocks and a zeroed destination only the spin-conserving elements) gives
    the bytes of the plain copy, and with dst_zeroed = 0 overwrites every
    element of a dirty destination."""
    ctx.set_precision(_lib.PREC_FP64, 7)
    sv = solver_for(ctx, UEG())
    try:
        assert (sv.spin_blocks(spin) > 0) == spin
        sv.guess(1)
        for _ in range(3):
            sv.step(0.5)
        shp1, shp2 = (sv.ng, sv.nv, sv.no), (sv.ng, sv.nv, sv.nv, sv.no, sv.no)
        P1, P2 = numpy.empty(shp1), numpy.empty(shp2)
        ctx.check(ctx.L.kvft_solver_get_amplitudes(sv.h, P1.ctypes.data_as(_lib.vp),
                                                    P2.ctypes.data_as(_lib.vp)), "get")
        T1, T2 = sv.amplitudes()
        assert numpy.array_equal(T1, P1) and numpy.array_equal(T2, P2)
        D1, D2 = numpy.full(shp1, numpy.nan), numpy.full(shp2, numpy.nan)
        ctx.check(ctx.L.kvft_solver_read_amplitudes(sv.h, D1.ctypes.data_as(_lib.vp),
                                                     D2.ctypes.data_as(_lib.vp), 0), "read")
        assert numpy.array_equal(D1, P1) and numpy.array_equal(D2, P2)
        assert numpy.count_nonzero(P2) > 0
    finally:
        sv.close()
