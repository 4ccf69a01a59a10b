"""The oracle's Lambda equations and E, S, N (oracle/ft_lambda.py).

* The reverse pass through the Stanton intermediates is the transposed
  Jacobian of the residual: <m, R'(t) dt> = <R'(t)^T m, dt>, with R'(t) dt from
  a complex-step derivative of the pinned residual (exact to rounding).
* E, S and N from converged Lambda equal central finite differences of the
  grand potential, as Kelvin's own test does (kelvin/tests/test_ft_deriv.py:
  222-275: UEG, 7 plane waves, T = mu = 0.1, ng = 8, damping 0.2); the
  agreement improves as the step squared, so the Lambda route is the exact
  derivative.
* Kelvin's published Lambda run for 19 plane waves (examples/ueg_ft_ccsd_ESN
  .out) -- its per-iteration Lambda residuals and E, S, N -- from the same
  settings (opt-in, a few minutes of CPU: KVFT_SLOW_ORACLE=1)."""
import json
import os

import numpy
import pytest

from conftest import GOLDEN, random_system
from oracle import cc_equations, ft_ccsd, ft_lambda, ft_utils, systems


class _B(object):
    pass


def _complex(blocks):
    out = _B()
    for k, v in vars(blocks).items():
        setattr(out, k, numpy.asarray(v, dtype=complex))
    return out


def _antisym(x):
    x = x - x.transpose(1, 0, 2, 3)
    return x - x.transpose(0, 1, 3, 2)


@pytest.mark.parametrize("no,nv,seed", [(3, 4, 1), (4, 6, 2), (5, 3, 3)])
def test_residual_vjp_adjoint_identity(no, nv, seed):
    rng = numpy.random.default_rng(seed)
    F, I = random_system(rng, no, nv)
    t1 = rng.standard_normal((nv, no)) * 0.1
    t2 = _antisym(rng.standard_normal((nv, nv, no, no)) * 0.1)
    m1 = rng.standard_normal((nv, no))
    m2 = _antisym(rng.standard_normal((nv, nv, no, no)))
    d1 = rng.standard_normal((nv, no))
    d2 = _antisym(rng.standard_normal((nv, nv, no, no)))
    h = 1e-30
    R1, R2 = cc_equations.residual(_complex(F), _complex(I), t1 + 1j * h * d1,
                                   t2 + 1j * h * d2)
    lhs = (m1 * R1.imag / h).sum() + 0.25 * (m2 * R2.imag / h).sum()
    g1, g2 = ft_lambda.residual_vjp(F, I, t1, t2, m1, m2)
    rhs = (g1 * d1).sum() + 0.25 * (g2 * d2).sum()
    assert abs(lhs - rhs) <= 1e-13 * abs(lhs)
    assert abs(g2 + g2.transpose(1, 0, 2, 3)).max() < 1e-13
    assert abs(g2 + g2.transpose(0, 1, 3, 2)).max() < 1e-13


def _ueg(norb):
    b = systems.UEGBasis(2 * numpy.pi, 1.2, norb=norb)
    eri = systems.g2e_loop(b)
    en = systems.ueg_g_energies(b)
    h = numpy.diag(numpy.hstack((b.Es, b.Es)))
    return en, h, eri


UEG7 = dict(T=0.1, mu=0.1, ng=8, damp=0.2)


@pytest.fixture(scope="module")
def ueg7():
    """Kelvin's derivative-test system (test_ft_deriv.py:222-233), solved
    tightly: (en, h, eri, E, S, N, Omega, T1, T2, L1, L2)."""
    en, h, eri = _ueg(7)
    out = ft_lambda.solve(en, h, eri, UEG7["T"], UEG7["mu"], ngrid=UEG7["ng"],
                          damp=UEG7["damp"], econv=1e-12, lconv=1e-11, max_iter=200)
    return (en, h, eri) + tuple(out)


def test_lambda_esn_vs_finite_differences(ueg7):
    T, mu, ng, damp = UEG7["T"], UEG7["mu"], UEG7["ng"], UEG7["damp"]
    en, h, eri, E, S, N, Om, T1, T2, L1, L2 = ueg7

    def omega(T, mu):
        beta = 1.0 / T
        fock = ft_lambda.mean_field(h, eri, ft_utils.ff(beta, en, mu))
        O0, O1 = ft_lambda.omega_ref(en, h, eri, beta, mu)
        return ft_ccsd.ft_ccsd(en, fock, eri, T, mu, ngrid=ng, econv=1e-13, max_iter=200,
                               damp=damp, E1=O1, T1in=T1, T2in=T2)[0]

    d = 2e-5
    Nx = -(omega(T, mu + d) - omega(T, mu - d)) / (2 * d)
    Sx = -(omega(T + d, mu) - omega(T - d, mu)) / (2 * d)      # S = -dOmega/dT
    Ex = Om + T * Sx + mu * Nx
    assert abs(Om - omega(T, mu)) < 1e-11
    assert abs(N - Nx) < 2e-9
    assert abs(E - Ex) < 2e-9
    assert abs(S - Sx) < 2e-8
    # the Lambda amplitudes are a fixed point of Kelvin's update
    ti, g, G = ft_lambda.quadrature.ft_quad(ng, 1.0 / T, 'lin')
    F, I = ft_ccsd.ft_integrals(ft_lambda.mean_field(h, eri, ft_utils.ff(1 / T, en, mu)),
                                eri, en, 1.0 / T, mu)
    L1n, L2n = ft_lambda.lambda_update(F, I, T1, T2, L1, L2, ft_utils.D1(en, en),
                                       ft_utils.D2(en, en), ti, ng, g, G)
    assert abs(L1n - L1).max() < 1e-9 * abs(L1).max()
    assert abs(L2n - L2).max() < 1e-9 * abs(L2).max()


def _omega_cc(en, fock, eri, T1, T2, T=UEG7["T"], mu=UEG7["mu"]):
    return ft_ccsd.ft_ccsd(en, fock, eri, T, mu, ngrid=UEG7["ng"], econv=1e-13,
                           max_iter=200, damp=UEG7["damp"], T1in=T1, T2in=T2)[1]


def test_response_densities_euler_identity(ueg7):
    """At convergence the Lagrangian equals Omega_cc, and all of it but the
    constraint's -<Lambda, T> term is linear in the integrals:
    (1/beta)(sum_b w_b P_b . I_b + one-electron terms)
    = Omega_cc - (1/beta) sum_y g_y <L_y, T_y>, the weighted block sum Kelvin
    forms in test_ft_cc_2rdm.py:125-140."""
    en, h, eri, E, S, N, Om, T1, T2, L1, L2 = ueg7
    T, mu, ng = UEG7["T"], UEG7["mu"], UEG7["ng"]
    beta = 1.0 / T
    fo = ft_utils.ff(beta, en, mu)
    F, I = ft_ccsd.ft_integrals(ft_lambda.mean_field(h, eri, fo), eri, en, beta, mu)
    ti, g, G = ft_lambda.quadrature.ft_quad(ng, beta, 'lin')
    (pia, pba, pji, pai), P2 = ft_lambda.response_densities(
        F, I, T1, T2, L1, L2, ft_utils.D1(en, en), ft_utils.D2(en, en), ti, ng, g, G)
    Ecc = ft_ccsd.ft_cc_energy(T1, T2, F.ov, I.oovv, g, beta)
    tot = (numpy.einsum('ia,ai->', pia, F.vo) + numpy.einsum('ba,ab->', pba, F.vv)
           + numpy.einsum('ji,ij->', pji, F.oo) + numpy.einsum('ai,ia->', pai, F.ov))
    for (name, blk, w, pairs), P in zip(ft_lambda.P2_BLOCKS, P2):
        tot += w * numpy.einsum('pqrs,rspq->', P, getattr(I, blk))
        for p in pairs:                   # antisymmetric in its same-type pairs
            perm = [0, 1, 2, 3]
            perm[p[0]], perm[p[1]] = perm[p[1]], perm[p[0]]
            assert abs(P + P.transpose(perm)).max() < 1e-14 * max(abs(P).max(), 1.0)
    LT = ft_lambda._lam_dot(L1, L2, T1, T2, g) / beta
    assert abs(tot / beta - (Ecc - LT)) < 1e-10 * abs(Ecc)
    # Kelvin's pia and Pijab are the weighted sums of int_L(L) (ft_cc_equations.py:713, 734)
    L1int = ft_lambda.quadrature.int_L1(ng, L1, ti, ft_utils.D1(en, en), g, G)
    L2int = ft_lambda.quadrature.int_L2(ng, L2, ti, ft_utils.D2(en, en), g, G)
    assert abs(pia - numpy.einsum('sia,s->ia', L1int, g)).max() < 1e-15
    assert abs(P2[3] - numpy.einsum('sijab,s->ijab', L2int, g)).max() < 1e-14


def test_rdms_vs_finite_differences(ueg7):
    """The normal-ordered RDMs are the integral derivatives of Omega_cc at
    fixed occupations: sum n1[p,q] dfock[q,p] and 1/4 sum n2[p,q,r,s]
    d<rs||pq> against central differences of converged solves (Kelvin's
    test_ft_cc_2rdm.py:66-104 differentiates the same way)."""
    en, h, eri, E, S, N, Om, T1, T2, L1, L2 = ueg7
    T, mu, ng = UEG7["T"], UEG7["mu"], UEG7["ng"]
    beta = 1.0 / T
    fo, fv = ft_utils.ff(beta, en, mu), ft_utils.ffv(beta, en, mu)
    fock = ft_lambda.mean_field(h, eri, fo)
    F, I = ft_ccsd.ft_integrals(fock, eri, en, beta, mu)
    ti, g, G = ft_lambda.quadrature.ft_quad(ng, beta, 'lin')
    P1, P2 = ft_lambda.response_densities(F, I, T1, T2, L1, L2, ft_utils.D1(en, en),
                                          ft_utils.D2(en, en), ti, ng, g, G)
    n1, n2 = ft_lambda.normal_ordered_rdms(beta, fo, fv, P1, P2)
    rng = numpy.random.default_rng(4)
    n = en.shape[0]
    dV = _antisym(rng.standard_normal((n,) * 4) * 1e-2)
    dV = 0.5 * (dV + dV.transpose(2, 3, 0, 1))
    df = rng.standard_normal((n, n)) * 1e-2
    df = 0.5 * (df + df.T)
    e = 5e-4
    ref2 = (_omega_cc(en, fock, eri + e * dV, T1, T2)
            - _omega_cc(en, fock, eri - e * dV, T1, T2)) / (2 * e)
    ref1 = (_omega_cc(en, fock + e * df, eri, T1, T2)
            - _omega_cc(en, fock - e * df, eri, T1, T2)) / (2 * e)
    out2 = 0.25 * numpy.einsum('pqrs,rspq->', n2, dV)
    out1 = numpy.einsum('pq,qp->', n1, df)
    # both are ~1e-3; the central differences carry ~1e-10 (step squared and
    # the solves' convergence)
    assert abs(out2 - ref2) < 2e-10
    assert abs(out1 - ref1) < 2e-10


@pytest.mark.skipif(not os.environ.get("KVFT_SLOW_ORACLE"),
                    reason="minutes of CPU; set KVFT_SLOW_ORACLE=1")
def test_lambda_ueg19_vs_kelvin():
    meta = json.load(open(os.path.join(GOLDEN, "ueg19_esn.json")))
    en, h, eri = _ueg(meta["norb"])
    hist = []
    E, S, N, Om = ft_lambda.solve(en, h, eri, meta["T"], meta["mu"], ngrid=meta["ngrid"],
                                  damp=meta["damp"], econv=meta["econv"],
                                  lconv=1000 * meta["econv"], max_iter=meta["max_iter"],
                                  history=hist, spin_half=meta["norb"])[:4]
    assert abs(Om - meta["Omega"]) < 1e-9
    ref = meta["lambda_residuals"]
    assert len(hist) == len(ref)
    for r, k in zip(hist, ref):            # printed with 10 decimals
        assert abs(r - k) <= 6e-11
    # measured here: |dE| 2e-15, |dS| 3e-14, |dN| 2e-16
    assert abs(E - meta["E"]) < 1e-12
    assert abs(S - meta["S"]) < 1e-12
    assert abs(N - meta["N"]) < 1e-12


def test_lambda_esn_hf_shifted_vs_finite_differences():
    """The same check with HF-shifted orbital energies (the UEGSCFSystem form,
    ueg_scf_system.py:280-297), where E1 has the sum_i (h_ii - e_i) f_i term
    and the Fock matrix's diagonal differs from the energies; Kelvin's test
    suite runs this comparison for its SCF systems (test_ft_deriv.py:56-110)."""
    T, mu, ng, damp = 0.1, 0.12, 6, 0.2
    b = systems.UEGBasis(2 * numpy.pi, 1.2, norb=7)
    eri = systems.g2e_loop(b)
    en = systems.uegscf_g_energies(b, mu)
    h = numpy.diag(numpy.hstack((b.Es, b.Es)))
    assert abs(numpy.diag(h) - en).max() > 1e-3
    E, S, N, Om, T1, T2, L1, L2 = ft_lambda.solve(en, h, eri, T, mu, ngrid=ng, damp=damp,
                                                  econv=1e-12, lconv=1e-11, max_iter=200)

    def omega(T, mu):
        beta = 1.0 / T
        fock = ft_lambda.mean_field(h, eri, ft_utils.ff(beta, en, mu))
        O0, O1 = ft_lambda.omega_ref(en, h, eri, beta, mu)
        return ft_ccsd.ft_ccsd(en, fock, eri, T, mu, ngrid=ng, econv=1e-13, max_iter=200,
                               damp=damp, E1=O1, T1in=T1, T2in=T2)[0]
    d = 2e-5
    Nx = -(omega(T, mu + d) - omega(T, mu - d)) / (2 * d)
    Sx = -(omega(T + d, mu) - omega(T - d, mu)) / (2 * d)
    Ex = Om + T * Sx + mu * Nx
    assert abs(N - Nx) < 2e-9
    assert abs(E - Ex) < 2e-9
    assert abs(S - Sx) < 2e-8
