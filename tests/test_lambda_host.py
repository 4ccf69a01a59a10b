"""Host logic of the Lambda path in kelvin_gb300 (no GPU): Kelvin's guess,
the damped Lambda loop with its residual measure, and the E, S, N assembly
from T and Lambda, each run with the oracle standing in for the device
update / amplitude update / energy."""
import numpy
import pytest

from kelvin_gb300 import cc_utils, ccsd as kccsd
from kelvin_gb300 import ft_cc_equations as fe
from oracle import ft_ccsd, ft_lambda, ft_utils, quadrature, systems


def _ueg7():
    b = systems.UEGBasis(2 * numpy.pi, 1.2, norb=7)
    eri = systems.g2e_loop(b)
    en = systems.ueg_g_energies(b)
    h = numpy.diag(numpy.hstack((b.Es, b.Es)))
    return en, h, eri


@pytest.fixture(scope="module")
def solved():
    en, h, eri = _ueg7()
    T, mu, ng = 0.1, 0.1, 8
    hist = []
    out = ft_lambda.solve(en, h, eri, T, mu, ngrid=ng, damp=0.2, econv=1e-12, lconv=1e-11,
                          max_iter=200, history=hist)
    return (en, h, eri, T, mu, ng, hist) + tuple(out)


def test_energies_from_d1():
    rng = numpy.random.default_rng(1)
    ev, eo = rng.standard_normal(5), rng.standard_normal(3)
    D1 = ev[:, None] - eo[None, :]
    a, b = fe.energies_from_d1(D1)
    assert abs((a[:, None] - b[None, :]) - D1).max() < 1e-15
    bad = D1.copy()
    bad[1, 1] += 1.0
    with pytest.raises(Exception):
        fe.energies_from_d1(bad)
    # large orbital energies: an element near zero carries the rounding of
    # the large ones, and D1 must still be accepted (the bar is relative to
    # max |D1|, as in the solver's own check)
    ev = 1e4 + rng.standard_normal(6)
    eo = 1e4 + rng.standard_normal(4)
    eo[0] = ev[2] - 1e-13
    D1 = ev[:, None] - eo[None, :]
    a, b = fe.energies_from_d1(D1)
    assert abs((a[:, None] - b[None, :]) - D1).max() < 1e-11


def test_lambda_guess_and_loop_match_oracle(solved):
    en, h, eri, T, mu, ng, hist, E, S, N, Om, T1, T2, L1, L2 = solved
    beta = 1.0 / T
    fo = ft_utils.ff(beta, en, mu)
    F, I = ft_ccsd.ft_integrals(ft_lambda.mean_field(h, eri, fo), eri, en, beta, mu)
    g1, g2 = fe.ccsd_lambda_guess(F, I, T1, beta, ng)
    o1, o2 = ft_lambda.lambda_guess(F, I, T1, beta, ng)
    assert abs(g1 - o1).max() < 1e-15 and abs(g2 - o2).max() == 0.0
    ti, g, G = quadrature.ft_quad(ng, beta, 'lin')
    D1, D2 = ft_utils.D1(en, en), ft_utils.D2(en, en)

    def update(F, I, T1, T2, L1, L2, D1, D2, ti, ng, g, G, beta):
        return ft_lambda.lambda_update(F, I, T1, T2, L1, L2, D1, D2, ti, ng, g, G)
    mine = []
    conv = {"tconv": 1e-11, "max_iter": 200, "damp": 0.2}
    M1, M2 = cc_utils.ft_lambda_iter("CCSD", g1, g2, T1, T2, F, I, D1, D2, g, G, beta, ng, ti,
                                     0, conv, update=update, history=mine)
    assert len(mine) == len(hist)
    assert max(abs(a - b) for a, b in zip(mine, hist)) < 1e-13
    assert abs(M1 - L1).max() == 0.0 and abs(M2 - L2).max() == 0.0


def test_esn_from_lambda_matches_oracle(solved):
    """The driver's assembly, sum_y g_y <L_y, Phi_y(dF, dI)> through the
    amplitude update instead of the oracle's int_L, gives the oracle's E, S, N."""
    en, h, eri, T, mu, ng, hist, E, S, N, Om, T1, T2, L1, L2 = solved

    def stanton(F, I, T1, T2, D1, D2, ti, ng, G):
        return ft_ccsd.ccsd_stanton(F, I, T1, T2, D1, D2, ti, ng, G)

    def energy(T1, T2, f, eri_, g, beta):
        return ft_ccsd.ft_cc_energy(T1, T2, f, eri_, g, beta)
    e, s, n = kccsd.esn_from_lambda(en, h, eri, 1.0 / T, mu, ng, 'lin', T1, T2, L1, L2, Om,
                                    stanton, energy)
    assert abs(e - E) < 1e-12 and abs(n - N) < 1e-12 and abs(s - S) < 1e-11


def test_derivative_integrals_match_differences():
    """dF, dI of the driver equal central differences of the scaled blocks."""
    en, h, eri = _ueg7()
    beta, mu = 10.0, 0.1
    for db, dm in ((1.0, 0.0), (0.0, 1.0)):
        dF, dI, _ = kccsd._d_integrals(h, eri, en, beta, mu, db, dm)
        e = 1e-5
        Fp, Ip = kccsd._scaled(h, eri, en, beta + e * db, mu + e * dm)
        Fm, Im = kccsd._scaled(h, eri, en, beta - e * db, mu - e * dm)
        for k in ('oo', 'ov', 'vo', 'vv'):
            ref = (getattr(Fp, k) - getattr(Fm, k)) / (2 * e)
            assert abs(getattr(dF, k) - ref).max() < 1e-7 * max(1.0, abs(ref).max())
        for k in ('vvvv', 'vvoo', 'vovo', 'oovv', 'oooo'):
            ref = (getattr(Ip, k) - getattr(Im, k)) / (2 * e)
            assert abs(getattr(dI, k) - ref).max() < 1e-7 * max(1.0, abs(ref).max())


def test_density_blocks_and_rdms_match_oracle(solved):
    """kelvin_densities / normal_ordered_rdms on the raw integral gradients
    (what kvft_lambda_densities returns) give the oracle's densities and RDMs."""
    en, h, eri, T, mu, ng, hist, E, S, N, Om, T1, T2, L1, L2 = solved
    beta = 1.0 / T
    fo = ft_utils.ff(beta, en, mu)
    F, I = ft_ccsd.ft_integrals(ft_lambda.mean_field(h, eri, fo), eri, en, beta, mu)
    ti, g, G = quadrature.ft_quad(ng, beta, 'lin')
    D1, D2 = ft_utils.D1(en, en), ft_utils.D2(en, en)
    Fs, Is = ft_lambda.integral_gradients(F, I, T1, T2, L1, L2, D1, D2, ti, ng, g, G)
    P1, P2 = fe.kelvin_densities({k: getattr(Fs, k) for k in fe.F_ORDER},
                                 {k: getattr(Is, k) for k in fe.I_ORDER})
    R1, R2 = ft_lambda.response_densities(F, I, T1, T2, L1, L2, D1, D2, ti, ng, g, G)
    for a, b in zip(P1 + P2, R1 + R2):
        assert abs(a - b).max() == 0.0
    n1, n2 = fe.normal_ordered_rdms(beta, fo, 1.0 - fo, P1, P2)
    m1, m2 = ft_lambda.normal_ordered_rdms(beta, fo, 1.0 - fo, R1, R2)
    assert abs(n1 - m1).max() < 1e-15 and abs(n2 - m2).max() < 1e-15


def test_spin_half_detection():
    """The Lambda path's spin blocks are used only when every operand
    vanishes outside the spin-conserving blocks."""
    n, h, ng = 6, 3, 2
    sp = (numpy.arange(n) >= h).astype(int)
    cons = (sp[:, None, None, None] + sp[None, :, None, None]
            == sp[None, None, :, None] + sp[None, None, None, :])
    rng = numpy.random.default_rng(2)
    I4 = rng.standard_normal((n,) * 4) * cons
    F2 = rng.standard_normal((n, n)) * (sp[:, None] == sp[None, :])
    T2 = rng.standard_normal((ng,) + (n,) * 4) * cons
    assert fe.spin_half_of(n, n, [F2, I4, T2]) == h
    T2[1, 0, h, 0, 0] = 1e-300
    assert fe.spin_half_of(n, n, [F2, I4, T2]) == 0
    assert fe.spin_half_of(n, n - 2, [F2]) == 0


def test_esn_from_lambda_hf_shifted_matches_oracle():
    """The driver's assembly with HF-shifted energies (E1's linear term, a
    Fock diagonal that differs from the energies) against the oracle."""
    T, mu, ng = 0.1, 0.12, 4
    b = systems.UEGBasis(2 * numpy.pi, 1.2, norb=7)
    eri = systems.g2e_loop(b)
    en = systems.uegscf_g_energies(b, mu)
    h = numpy.diag(numpy.hstack((b.Es, b.Es)))
    E, S, N, Om, T1, T2, L1, L2 = ft_lambda.solve(en, h, eri, T, mu, ngrid=ng, damp=0.2,
                                                  econv=1e-12, lconv=1e-11, max_iter=200)

    def stanton(F, I, T1, T2, D1, D2, ti, ng, G):
        return ft_ccsd.ccsd_stanton(F, I, T1, T2, D1, D2, ti, ng, G)

    def energy(T1, T2, f, eri_, g, beta):
        return ft_ccsd.ft_cc_energy(T1, T2, f, eri_, g, beta)
    e, s, n = kccsd.esn_from_lambda(en, h, eri, 1.0 / T, mu, ng, 'lin', T1, T2, L1, L2, Om,
                                    stanton, energy)
    assert abs(e - E) < 1e-12 and abs(n - N) < 1e-12 and abs(s - S) < 1e-11
