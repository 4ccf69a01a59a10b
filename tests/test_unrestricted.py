"""The unrestricted update (ft_cc_equations.uccsd_stanton, Kelvin's
ft_cc_equations.py:130-164) runs as one general-spin update with the alpha
spin orbitals first.  These tests check the layout: general-spin blocks built
from the alpha, beta and alpha-beta blocks equal the general-spin blocks of
the same system, and the amplitude and denominator maps are exact."""
import numpy
import pytest

from kelvin_gb300 import ft_cc_equations as fe
from kelvin_gb300 import systems
from oracle import ft_utils

I16 = ("vvvv", "vvvo", "vvov", "vovv", "ovvv", "vvoo", "vovo", "voov", "ovvo", "ovov",
       "oovv", "vooo", "ovoo", "oovo", "ooov", "oooo")


def ueg_blocks():
    s = systems.UEGSystem(0.1, 2 * numpy.pi, 1.2, mu=0.1, norb=7)
    en, eri = s.g_energies_tot(), s.g_aint_tot()
    beta = 1.0 / s.T
    sc = {'o': numpy.sqrt(ft_utils.ff(beta, en, s.mu)),
          'v': numpy.sqrt(ft_utils.ffv(beta, en, s.mu))}

    def blk(t):
        p, q, r, u = (sc[c] for c in t)
        return eri * (p[:, None, None, None] * q[None, :, None, None]
                      * r[None, None, :, None] * u[None, None, None, :])
    return s, en, blk


class B(object):
    pass


def test_two_electron_blocks_from_spin_cases():
    s, en, blk = ueg_blocks()
    n = en.shape[0]
    na = n // 2
    A, Bs = slice(0, na), slice(na, n)
    Ia, Ib, Iabab = B(), B(), B()
    for t in fe.I_ORDER:
        setattr(Ia, t, blk(t)[A, A, A, A])
        setattr(Ib, t, blk(t)[Bs, Bs, Bs, Bs])
    for t in I16:
        # <ab||ab> over alpha (1, 3) and beta (2, 4) indices is the Coulomb <ab|ab>
        setattr(Iabab, t, blk(t)[A, Bs, A, Bs])
    g = fe.u_to_g_two(Ia, Ib, Iabab)
    for t in fe.I_ORDER:
        # the same products of integrals and Fermi factors, up to the order of
        # the factors (one rounding)
        ref = blk(t)
        assert abs(getattr(g, t) - ref).max() <= 1e-15 * abs(ref).max(), t
        assert not getattr(g, t)[ref == 0].any(), t


def test_amplitude_and_denominator_maps():
    rng = numpy.random.default_rng(3)
    ng, na = 3, 4
    n = 2 * na
    sp = (numpy.arange(n) >= na).astype(int)
    cons = (sp[:, None, None, None] + sp[None, :, None, None]
            == sp[None, None, :, None] + sp[None, None, None, :])
    T2 = rng.standard_normal((ng, n, n, n, n))
    T2 = T2 - T2.transpose(0, 2, 1, 3, 4)
    T2 = T2 - T2.transpose(0, 1, 2, 4, 3)
    T2 = T2 * cons
    T1 = rng.standard_normal((ng, n, n)) * (sp[:, None] == sp[None, :])
    (t1a, t1b), (t2aa, t2ab, t2bb) = fe.g_to_u_t(T1, T2, na)
    assert numpy.array_equal(fe.u_to_g_t1(t1a, t1b), T1)
    assert numpy.array_equal(fe.u_to_g_t2(t2aa, t2ab, t2bb), T2)
    e = rng.standard_normal(n)
    ea, eb = e[:na], e[na:]
    D2 = e[:, None, None, None] + e[None, :, None, None] - e[None, None, :, None] \
        - e[None, None, None, :]
    D2aa = ea[:, None, None, None] + ea[None, :, None, None] - ea[None, None, :, None] \
        - ea[None, None, None, :]
    D2bb = eb[:, None, None, None] + eb[None, :, None, None] - eb[None, None, :, None] \
        - eb[None, None, None, :]
    D2ab = ea[:, None, None, None] + eb[None, :, None, None] - ea[None, None, :, None] \
        - eb[None, None, None, :]
    g = fe.u_to_g_d2(D2aa, D2ab, D2bb)
    assert numpy.allclose(g[cons], D2[cons], rtol=0, atol=1e-14)
    assert not g[~cons].any()


@pytest.mark.gpu
def test_uccsd_stanton_vs_oracle(ctx):
    """The unrestricted update against the oracle's general-spin update of the
    same UEG system (Kelvin pins general spin == unrestricted to 1e-12,
    tests/test_ft_cc_ampl.py:41-107)."""
    from kelvin_gb300 import quadrature
    from oracle import ft_ccsd as oft
    s, en, blk = ueg_blocks()
    n = en.shape[0]
    na = n // 2
    A, Bs = slice(0, na), slice(na, n)
    beta, ng = 1.0 / s.T, 6
    F, I = oft.ft_integrals(s.g_fock_tot(), s.g_aint_tot(), en, beta, s.mu)
    ti, g, G = quadrature.ft_quad(ng, beta, "lin")
    D1, D2 = ft_utils.D1(en, en), ft_utils.D2(en, en)
    rng = numpy.random.default_rng(11)
    sp = (numpy.arange(n) >= na).astype(int)
    cons = (sp[:, None, None, None] + sp[None, :, None, None]
            == sp[None, None, :, None] + sp[None, None, None, :])
    T1 = rng.standard_normal((ng, n, n)) * 0.05 * (sp[:, None] == sp[None, :])
    T2 = rng.standard_normal((ng, n, n, n, n)) * 0.05
    T2 = (T2 - T2.transpose(0, 2, 1, 3, 4))
    T2 = (T2 - T2.transpose(0, 1, 2, 4, 3)) * cons
    r1, r2 = oft.ccsd_stanton(F, I, T1, T2, D1, D2, ti, ng, G)
    Fa, Fb = B(), B()
    for t in fe.F_ORDER:
        setattr(Fa, t, getattr(F, t)[A, A])
        setattr(Fb, t, getattr(F, t)[Bs, Bs])
    Ia, Ib, Iabab = B(), B(), B()
    for t in fe.I_ORDER:
        setattr(Ia, t, blk(t)[A, A, A, A])
        setattr(Ib, t, blk(t)[Bs, Bs, Bs, Bs])
    for t in I16:
        setattr(Iabab, t, blk(t)[A, Bs, A, Bs])
    (t1a, t1b), (t2aa, t2ab, t2bb) = fe.g_to_u_t(T1, T2, na)
    (o1a, o1b), (o2aa, o2ab, o2bb) = fe.uccsd_stanton(
        Fa, Fb, Ia, Ib, Iabab, t1a, t1b, t2aa, t2ab, t2bb, D1[A, A], D1[Bs, Bs],
        D2[A, A, A, A], D2[A, Bs, A, Bs], D2[Bs, Bs, Bs, Bs], ti, ng, G, ctx=ctx)
    (e1a, e1b), (e2aa, e2ab, e2bb) = fe.g_to_u_t(r1, r2, na)
    for x, y in ((o1a, e1a), (o1b, e1b), (o2aa, e2aa), (o2ab, e2ab), (o2bb, e2bb)):
        assert abs(x - y).max() < 1e-12


def test_uccsd_lambda_layout(monkeypatch):
    """Kelvin's unrestricted Lambda signatures on the general-spin update: the
    per-spin energies read off D1a/D1b and the spin-case maps reproduce the
    oracle's general-spin Lambda update and guess (the device update replaced
    by the oracle here; the device update itself is checked elsewhere)."""
    from kelvin_gb300 import quadrature
    from oracle import ft_ccsd as oft
    from oracle import ft_lambda
    s, en, blk = ueg_blocks()
    n = en.shape[0]
    na = n // 2
    A, Bs = slice(0, na), slice(na, n)
    beta, ng = 1.0 / s.T, 4
    F, I = oft.ft_integrals(s.g_fock_tot(), s.g_aint_tot(), en, beta, s.mu)
    ti, g, G = quadrature.ft_quad(ng, beta, "lin")
    D1, D2 = ft_utils.D1(en, en), ft_utils.D2(en, en)
    rng = numpy.random.default_rng(12)
    sp = (numpy.arange(n) >= na).astype(int)
    cons = (sp[:, None, None, None] + sp[None, :, None, None]
            == sp[None, None, :, None] + sp[None, None, None, :])
    same = sp[:, None] == sp[None, :]

    def anti(x):
        x = x - x.transpose(0, 2, 1, 3, 4)
        return (x - x.transpose(0, 1, 2, 4, 3)) * cons
    T1 = rng.standard_normal((ng, n, n)) * 0.05 * same
    T2 = anti(rng.standard_normal((ng, n, n, n, n)) * 0.05)
    L1 = rng.standard_normal((ng, n, n)) * 0.05 * same
    L2 = anti(rng.standard_normal((ng, n, n, n, n)) * 0.05)

    def fake(F, I, T1, T2, L1, L2, D1, D2, ti, ng, g, G, beta, ctx=None, precision=None,
             energies=None):
        ev, eo = energies
        d1 = ev[:, None] - eo[None, :]
        d2 = (ev[:, None, None, None] + ev[None, :, None, None] - eo[None, None, :, None]
              - eo[None, None, None, :])
        return ft_lambda.lambda_update(F, I, T1, T2, L1, L2, d1, d2, ti, ng, g, G)
    monkeypatch.setattr(fe, "ccsd_lambda_opt", fake)
    Fa, Fb = B(), B()
    for t in fe.F_ORDER:
        setattr(Fa, t, getattr(F, t)[A, A])
        setattr(Fb, t, getattr(F, t)[Bs, Bs])
    Ia, Ib, Iabab = B(), B(), B()
    for t in fe.I_ORDER:
        setattr(Ia, t, blk(t)[A, A, A, A])
        setattr(Ib, t, blk(t)[Bs, Bs, Bs, Bs])
    for t in I16:
        setattr(Iabab, t, blk(t)[A, Bs, A, Bs])
    (t1a, t1b), (t2aa, t2ab, t2bb) = fe.g_to_u_t(T1, T2, na)
    (l1a, l1b), (l2aa, l2ab, l2bb) = fe.g_to_u_t(L1, L2, na)
    out = fe.uccsd_lambda_opt(Fa, Fb, Ia, Ib, Iabab, t1a, t1b, t2aa, t2ab, t2bb, l1a, l1b,
                              l2aa, l2ab, l2bb, D1[A, A], D1[Bs, Bs], D2[A, A, A, A],
                              D2[A, Bs, A, Bs], D2[Bs, Bs, Bs, Bs], ti, ng, g, G, beta)
    r1, r2 = ft_lambda.lambda_update(F, I, T1, T2, L1, L2, D1, D2, ti, ng, g, G)
    (e1a, e1b), (e2aa, e2ab, e2bb) = fe.g_to_u_t(r1, r2, na)
    for x, y in zip(out, (e1a, e1b, e2aa, e2ab, e2bb)):
        assert abs(x - y).max() < 1e-12 * max(1.0, abs(y).max())
    gu = fe.uccsd_lambda_guess(Fa, Fb, Ia, Ib, Iabab, t1a, t1b, beta, ng)
    q1, q2 = ft_lambda.lambda_guess(F, I, T1, beta, ng, unrestricted=True)
    (f1a, f1b), (f2aa, f2ab, f2bb) = fe.g_to_u_t(q1, q2, na)
    for x, y in zip(gu, (f1a, f1b, f2aa, f2ab, f2bb)):
        assert abs(x - y).max() < 1e-14 * max(1.0, abs(y).max())
