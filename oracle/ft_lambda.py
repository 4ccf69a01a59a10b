"""FT-CCSD Lambda equations and the E, S, N they give (oracle; test
infrastructure).

Kelvin's Lambda iteration (kelvin/ft_cc_equations.py:385-409 ccsd_lambda_opt,
:502-512 ccsd_lambda_guess; kelvin/cc_utils.py:414-480 ft_lambda_iter) hands
the per-tau Lambda terms to ``cqcpy.cc_equations._Lambda_opt`` and
``_LS_TS``, which are not vendored.  The Lambda amplitudes are the adjoint of
the amplitude iteration, so they are restated here from that definition:

    Omega_cc = (1/beta) sum_y g_y E(T_y),    T_y = sum_x G[y,x] e^{(t_x-t_y)D} S(T_x),
    S(T) = -(F.vo, I.vvoo) - R(T)            (ft_cc_equations.py:96-113)

and the total derivative of Omega_cc with respect to T_x is (g_x/beta) M_x with

    M_x = E'(T_x) - R'(T_x)^T Mint_x,   Mint_s = sum_{y>=s} g_y G[y,s] e^{(t_s-t_y)D} M_y / g_s,

Mint being exactly Kelvin's int_L1/int_L2 (quadrature.py:320-345).  Kelvin's L
is -M (its energy term is L1 -= F.ov + I.oovv T1, L2 -= I.oovv,
ft_cc_equations.py:403-407, and its grid derivative weighs -L/beta,
ccsd.py:1114-1146).  Inner products of doubles carry Kelvin's factor 1/4:
<L, X> = sum L1[i,a] X1[a,i] + 1/4 sum L2[i,j,a,b] X2[a,b,i,j].

R'(T)^T is ``residual_vjp``: the reverse pass through the same Stanton
intermediates ``cc_equations.residual`` evaluates, term by term.  It is pinned
by the adjoint identity <m, R'(t) dt> = <R'(t)^T m, dt> against a complex-step
derivative of the residual (exact to rounding; tests/test_lambda.py).

E, S and N (kelvin/ccsd.py:167-214 _g_ft_ESN, 1075-1148 _g_nocc_gderiv) follow
from the derivative of the grand potential with respect to beta and mu at
fixed orbital energies, with the mean-field Fock matrix following the
occupations (ueg_scf_system.py:398-417, 481-493) and the tau grid moving with
beta.  The residual and the energy are linear in the integrals, so the
explicit derivative of the Lagrangian is the residual and the energy
evaluated with the derivative integrals (dF, dI), which are exact closed
forms here; the grid enters through dg/dbeta = g/beta, dG/dbeta = G/beta and
dt/dbeta = t/beta, true for every rule of ``quadrature.ft_quad`` (each is beta
times a beta-free rule).
"""
import numpy

from . import cc_equations
from . import ft_ccsd
from . import ft_utils
from . import quadrature

einsum = cc_equations.einsum


def _pab(x):
    return x - x.transpose(1, 0, 2, 3)


def _pij(x):
    return x - x.transpose(0, 1, 3, 2)


class _Grad(object):
    """Gradient accumulator with one zero array per integral block."""

    def __init__(self, blocks):
        for k, v in vars(blocks).items():
            setattr(self, k, numpy.zeros_like(v))


def residual_vjp(F, I, t1, t2, m1, m2, integrals=False):
    """(g1, g2) = R'(t1, t2)^T (m1, m2) in amplitude layout ([a,i], [a,b,i,j]):

        sum g1 dt1 + 1/4 sum g2 dt2 = sum m1 dR1 + 1/4 sum m2 dR2

    for every dt1 and antisymmetric dt2 (m2 antisymmetric); g2 is
    antisymmetric.  Each block below undoes one line of
    ``cc_equations.intermediates`` / ``cc_equations.residual``.

    With ``integrals=True`` also (Fg, Ig): the gradient of
    sum m1 R1 + 1/4 sum m2 R2 with respect to every entry of every F and I
    block the residual reads (R is linear in them), blocks as laid out in F, I."""
    Fae, Fmi, Fme, Wmnij, Wabef, Wmbej, tau = cc_equations.intermediates(F, I, t1, t2)
    R1b = m1
    R2b = 0.25 * m2
    t1b = numpy.zeros_like(t1)
    t2b = numpy.zeros_like(t2)
    Fg, Ig = _Grad(F), _Grad(I)

    # ---- R2 ----
    # x = t1[a,m] <bm||ij>;  R2 += P(ab) x
    xb = _pab(R2b)
    t1b += einsum('abij,bmij->am', xb, I.vooo)
    Ig.vooo += einsum('abij,am->bmij', xb, t1)
    # x = t1[e,i] <ab||ej>;  R2 += P(ij) x
    xb = _pij(R2b)
    t1b += einsum('abij,abej->ei', xb, I.vvvo)
    Ig.vvvo += einsum('abij,ei->abej', xb, t1)
    # x = t2[a,e,i,m] W_mbej + t1[e,i] t1[a,m] vovo[b,m,e,j];  R2 += P(ab)P(ij) x
    xb = R2b - R2b.transpose(1, 0, 2, 3) - R2b.transpose(0, 1, 3, 2) \
        + R2b.transpose(1, 0, 3, 2)
    t2b += einsum('abij,mbej->aeim', xb, Wmbej)
    Wmbejb = einsum('abij,aeim->mbej', xb, t2)
    t1b += einsum('abij,am,bmej->ei', xb, t1, I.vovo)
    t1b += einsum('abij,ei,bmej->am', xb, t1, I.vovo)
    Ig.vovo += einsum('abij,ei,am->bmej', xb, t1, t1)
    # R2 += 1/2 tau[e,f,i,j] W_abef
    taub = 0.5 * einsum('abij,abef->efij', R2b, Wabef)
    Wabefb = 0.5 * einsum('abij,efij->abef', R2b, tau)
    # R2 += 1/2 tau[a,b,m,n] W_mnij
    taub += 0.5 * einsum('abij,mnij->abmn', R2b, Wmnij)
    Wmnijb = 0.5 * einsum('abij,abmn->mnij', R2b, tau)
    # x = t2[a,b,i,m] X_mj, X_mj = F_mi + 1/2 t1[e,j] F_me;  R2 -= P(ij) x
    Xmj = Fmi + 0.5 * einsum('ej,me->mj', t1, Fme)
    xb = -_pij(R2b)
    t2b += einsum('abij,mj->abim', xb, Xmj)
    Xmjb = einsum('abij,abim->mj', xb, t2)
    # x = t2[a,e,i,j] X_be, X_be = F_ae - 1/2 t1[b,m] F_me;  R2 += P(ab) x
    Xbe = Fae - 0.5 * einsum('bm,me->be', t1, Fme)
    xb = _pab(R2b)
    t2b += einsum('abij,be->aeij', xb, Xbe)
    Xbeb = einsum('abij,aeij->be', xb, t2)
    Fmib = Xmjb.copy()
    t1b += 0.5 * einsum('mj,me->ej', Xmjb, Fme)
    Fmeb = 0.5 * einsum('mj,ej->me', Xmjb, t1)
    Faeb = Xbeb.copy()
    t1b -= 0.5 * einsum('be,me->bm', Xbeb, Fme)
    Fmeb -= 0.5 * einsum('be,bm->me', Xbeb, t1)

    # ---- R1 ----
    Faeb += einsum('ai,ei->ae', R1b, t1)
    t1b += einsum('ai,ae->ei', R1b, Fae)
    t1b -= einsum('ai,mi->am', R1b, Fmi)
    Fmib -= einsum('ai,am->mi', R1b, t1)
    t2b += einsum('ai,me->aeim', R1b, Fme)
    Fmeb += einsum('ai,aeim->me', R1b, t2)
    t1b -= einsum('ai,anfi->fn', R1b, I.vovo)
    t2b += 0.5 * einsum('ai,amef->efim', R1b, I.vovv)
    t2b += 0.5 * einsum('ai,nmie->aemn', R1b, I.ooov)
    Ig.vovo -= einsum('ai,fn->anfi', R1b, t1)
    Ig.vovv += 0.5 * einsum('ai,efim->amef', R1b, t2)
    Ig.ooov += 0.5 * einsum('ai,aemn->nmie', R1b, t2)

    # ---- intermediates ----
    # W_abef = vvvv - P(ab) t1[b,m] vovv[a,m,e,f] + 1/4 tau[a,b,m,n] oovv[m,n,e,f]
    xb = -_pab(Wabefb)
    t1b += einsum('abef,amef->bm', xb, I.vovv)
    taub += 0.25 * einsum('abef,mnef->abmn', Wabefb, I.oovv)
    Ig.vvvv += Wabefb
    Ig.vovv += einsum('abef,bm->amef', xb, t1)
    Ig.oovv += 0.25 * einsum('abef,abmn->mnef', Wabefb, tau)
    # W_mnij = oooo + P(ij) t1[e,j] ooov[m,n,i,e] + 1/4 tau[e,f,i,j] oovv[m,n,e,f]
    xb = _pij(Wmnijb)
    t1b += einsum('mnij,mnie->ej', xb, I.ooov)
    taub += 0.25 * einsum('mnij,mnef->efij', Wmnijb, I.oovv)
    Ig.oooo += Wmnijb
    Ig.ooov += einsum('mnij,ej->mnie', xb, t1)
    Ig.oovv += 0.25 * einsum('mnij,efij->mnef', Wmnijb, tau)
    # W_mbej = -<mb||je> - t1[f,j] vovv[b,m,e,f] + t1[b,n] ooov[m,n,j,e]
    #          - (1/2 t2[f,b,j,n] + t1[f,j] t1[b,n]) oovv[m,n,e,f]
    t1b -= einsum('mbej,bmef->fj', Wmbejb, I.vovv)
    t1b += einsum('mbej,mnje->bn', Wmbejb, I.ooov)
    tmpb = -einsum('mbej,mnef->fbjn', Wmbejb, I.oovv)
    Ig.vovo -= Wmbejb.transpose(1, 0, 2, 3)
    Ig.vovv -= einsum('mbej,fj->bmef', Wmbejb, t1)
    Ig.ooov += einsum('mbej,bn->mnje', Wmbejb, t1)
    Ig.oovv -= einsum('mbej,fbjn->mnef', Wmbejb, 0.5 * t2 + einsum('fj,bn->fbjn', t1, t1))
    t2b += 0.5 * tmpb
    t1b += einsum('fbjn,bn->fj', tmpb, t1)
    t1b += einsum('fbjn,fj->bn', tmpb, t1)
    # F_me = ov + t1[f,n] oovv[m,n,e,f]
    t1b += einsum('me,mnef->fn', Fmeb, I.oovv)
    Fg.ov += Fmeb
    Ig.oovv += einsum('me,fn->mnef', Fmeb, t1)
    # F_mi = oo + 1/2 t1[e,i] ov[m,e] + t1[e,n] ooov[m,n,i,e] + 1/2 ttau[e,f,i,n] oovv[m,n,e,f]
    t1b += 0.5 * einsum('mi,me->ei', Fmib, F.ov)
    t1b += einsum('mi,mnie->en', Fmib, I.ooov)
    ttaub = 0.5 * einsum('mi,mnef->efin', Fmib, I.oovv)
    ttau = cc_equations._tau(t1, t2, 0.5)
    Fg.oo += Fmib
    Fg.ov += 0.5 * einsum('mi,ei->me', Fmib, t1)
    Ig.ooov += einsum('mi,en->mnie', Fmib, t1)
    Ig.oovv += 0.5 * einsum('mi,efin->mnef', Fmib, ttau)
    # F_ae = vv - 1/2 ov[m,e] t1[a,m] - t1[f,m] vovv[a,m,f,e] - 1/2 ttau[a,f,m,n] oovv[m,n,e,f]
    t1b -= 0.5 * einsum('ae,me->am', Faeb, F.ov)
    t1b -= einsum('ae,amfe->fm', Faeb, I.vovv)
    ttaub -= 0.5 * einsum('ae,mnef->afmn', Faeb, I.oovv)
    Fg.vv += Faeb
    Fg.ov -= 0.5 * einsum('ae,am->me', Faeb, t1)
    Ig.vovv -= einsum('ae,fm->amfe', Faeb, t1)
    Ig.oovv -= 0.5 * einsum('ae,afmn->mnef', Faeb, ttau)
    # tau = t2 + P(ab) t1 t1, ttau = t2 + 1/2 P(ab) t1 t1
    t2b += taub + ttaub
    ttb = _pab(taub) + 0.5 * _pab(ttaub)
    t1b += einsum('abij,bj->ai', ttb, t1)
    t1b += einsum('abij,ai->bj', ttb, t1)
    g2 = t2b - t2b.transpose(1, 0, 2, 3) - t2b.transpose(0, 1, 3, 2) + t2b.transpose(1, 0, 3, 2)
    if integrals:
        return t1b, g2, Fg, Ig
    return t1b, g2


def energy_grad(F, I, t1):
    """E'(T) in Lambda layout ([i,a], [i,j,a,b]) for
    E = F.ov.T1 + 1/4 I.oovv.T2 + 1/2 I.oovv.T1.T1 (ft_cc_energy.py:7-32)."""
    return F.ov + einsum('ijab,bj->ia', I.oovv, t1), I.oovv


def lambda_guess(F, I, T1, beta, ng, unrestricted=False):
    """Kelvin's starting Lambda, (1/beta)(F.ov + I.oovv T1, I.oovv) at every
    tau point (ft_cc_equations.py:502-512).  Kelvin's unrestricted guess
    adds the I.oovv T1 term without the 1/beta (ft_cc_equations.py:515-526,
    ``_u_LS_TS`` at its default factor); ``unrestricted=True`` reproduces it."""
    it1 = numpy.stack([einsum('ijab,bj->ia', I.oovv, T1[y]) for y in range(ng)])
    L1 = (F.ov[None] + it1) / beta
    if unrestricted:
        L1 = F.ov[None] / beta + it1
    L2 = numpy.repeat(I.oovv[None], ng, axis=0) / beta
    return L1, L2


def lambda_update(F, I, T1, T2, L1old, L2old, D1, D2, ti, ng, g, G):
    """One Lambda update, L = -E'(T) - R'(T)^T int_L(L_old) per tau point
    (ft_cc_equations.py:385-409)."""
    L1int = quadrature.int_L1(ng, L1old, ti, D1, g, G)
    L2int = quadrature.int_L2(ng, L2old, ti, D2, g, G)
    L1 = numpy.empty_like(L1old)
    L2 = numpy.empty_like(L2old)
    for y in range(ng):
        v1, v2 = residual_vjp(F, I, T1[y], T2[y], L1int[y].T,
                              L2int[y].transpose(2, 3, 0, 1))
        e1, e2 = energy_grad(F, I, T1[y])
        L1[y] = -e1 - v1.T
        L2[y] = -e2 - v2.transpose(2, 3, 0, 1)
    return L1, L2


def _spin_cases(L1, L2, na):
    """(L1a, L1b), (L2aa, L2ab, L2bb) of general-spin Lambda with the alpha
    spin orbitals first."""
    a, b = slice(0, na), slice(na, None)
    return ((L1[:, a, a], L1[:, b, b]),
            (L2[:, a, a, a, a], L2[:, a, b, a, b], L2[:, b, b, b, b]))


def _norms(L1, L2, na):
    """Kelvin's normalisers |L1| + 0.1, |L2| + 0.1; per spin case
    |L1a| + |L1b| + 0.1 and |L2aa| + |L2bb| + 4 |L2ab| + 0.1 when na is given
    (cc_utils.py:514-517)."""
    nrm = numpy.linalg.norm
    if na is None:
        return nrm(L1) + 0.1, nrm(L2) + 0.1
    (l1a, l1b), (l2aa, l2ab, l2bb) = _spin_cases(L1, L2, na)
    return nrm(l1a) + nrm(l1b) + 0.1, nrm(l2aa) + nrm(l2bb) + 4 * nrm(l2ab) + 0.1


def _res(L1, L2, L1old, L2old, nl1, nl2, na):
    nrm = numpy.linalg.norm
    if na is None:
        return nrm(L1 - L1old) / nl1 + nrm(L2 - L2old) / nl2
    d1, d2 = _spin_cases(L1 - L1old, L2 - L2old, na)
    return sum(nrm(x) for x in d1) / nl1 + sum(nrm(x) for x in d2) / nl2


def ft_lambda_iter(L1old, L2old, T1, T2, F, I, D1, D2, g, G, beta, ng, ti, conv_options,
                   history=None, spin_half=None):
    """Damped Lambda iteration with Kelvin's residual measure and stop rule
    (cc_utils.py:414-480): res = |L - L_old| / (|L_old| + 0.1) summed over
    L1, L2; stop when it drops below tconv or at max_iter.  With ``spin_half``
    (the number of alpha spin orbitals, listed first) the measure is the
    unrestricted driver's, summed over the spin cases (cc_utils.py:482-560),
    so that a general-spin run reproduces an unrestricted run's history."""
    thresh = conv_options["tconv"]
    max_iter = conv_options["max_iter"]
    alpha = conv_options["damp"]
    nl1, nl2 = _norms(L1old, L2old, spin_half)
    for _ in range(max_iter):
        L1, L2 = lambda_update(F, I, T1, T2, L1old, L2old, D1, D2, ti, ng, g, G)
        res = _res(L1, L2, L1old, L2old, nl1, nl2, spin_half)
        L1old = alpha * L1old + (1.0 - alpha) * L1
        L2old = alpha * L2old + (1.0 - alpha) * L2
        nl1, nl2 = _norms(L1old, L2old, spin_half)
        if history is not None:
            history.append(res)
        if res < thresh:
            break
    return L1old, L2old


def _lam_dot(L1, L2, X1, X2, w):
    """sum_y w_y <L_y, X_y> with the doubles factor 1/4."""
    return einsum('y,yia,yai->', w, L1, X1) + 0.25 * einsum('y,yijab,yabij->', w, L2, X2)


def _tbar(F, I, T1, T2, ng):
    """S(T) = -(F.vo, I.vvoo) - R(T) at every tau point."""
    S1 = numpy.repeat(-F.vo[None], ng, axis=0)
    S2 = numpy.repeat(-I.vvoo[None], ng, axis=0)
    for y in range(ng):
        cc_equations.stanton(S1[y], S2[y], F, I, T1[y], T2[y], fac=-1.0)
    return S1, S2


def mean_field(h, eri, fo):
    """Fock matrix h + sum_r <pr||qr> f_r (ueg_scf_system.py:398-417)."""
    return h + einsum('prqr,r->pq', eri, fo)


def omega_ref(en, h, eri, beta, mu, E_const=0.0):
    """Omega_0 + Omega_1: orbital grand potentials plus
    sum_i (h_ii - e_i) f_i + 1/2 sum_ij <ij||ij> f_i f_j (ueg_scf_system.py:125-160)."""
    fo = ft_utils.ff(beta, en, mu)
    W = einsum('ijij->ij', eri)
    return (ft_utils.GP0(beta, en, mu).sum() + E_const,
            (numpy.diag(h) - en) @ fo + 0.5 * fo @ W @ fo)


def _d_integrals(h, eri, en, beta, mu, dbeta, dmu):
    """Exact directional derivatives (dF, dI) of the Fermi-scaled integrals
    (cc_utils.py:569-602) along (dbeta, dmu), the Fock matrix following the
    occupations, and the occupation derivative dfo."""
    fo = ft_utils.ff(beta, en, mu)
    fv = ft_utils.ffv(beta, en, mu)
    so, sv = numpy.sqrt(fo), numpy.sqrt(fv)
    rate = beta * dmu - (en - mu) * dbeta            # d(beta (mu - e))
    dfo = fo * fv * rate
    dso = 0.5 * so * fv * rate
    dsv = -0.5 * sv * fo * rate
    fock = mean_field(h, eri, fo)
    fmo = fock - numpy.diag(en)
    dfock = einsum('prqr,r->pq', eri, dfo)
    s = {'o': so, 'v': sv}
    ds = {'o': dso, 'v': dsv}
    blk1 = []
    for b in ('oo', 'ov', 'vo', 'vv'):
        p, q, dp, dq = s[b[0]], s[b[1]], ds[b[0]], ds[b[1]]
        blk1.append(dfock * p[:, None] * q[None, :]
                    + fmo * (dp[:, None] * q[None, :] + p[:, None] * dq[None, :]))
    dF = ft_utils.one_e_blocks(*blk1)
    blk2 = {}
    for name in ft_utils.two_e_blocks.NAMES:
        f = [s[c] for c in name]
        d = [ds[c] for c in name]
        acc = 0.0
        for k in range(4):
            v = [d[m] if m == k else f[m] for m in range(4)]
            acc = acc + (v[0][:, None, None, None] * v[1][None, :, None, None]
                         * v[2][None, None, :, None] * v[3][None, None, None, :])
        blk2[name] = eri * acc
    return dF, ft_utils.two_e_blocks(**blk2), dfo


def omega_derivative(en, h, eri, beta, mu, ngrid, quad, T1, T2, L1, L2, dbeta, dmu):
    """dOmega along (dbeta, dmu) from converged T and Lambda (Kelvin's L = -M)."""
    ti, g, G = quadrature.ft_quad(ngrid, beta, quad)
    ng = ngrid
    fo = ft_utils.ff(beta, en, mu)
    F, I = ft_ccsd.ft_integrals(mean_field(h, eri, fo), eri, en, beta, mu)
    D1 = ft_utils.D1(en, en)
    D2 = ft_utils.D2(en, en)
    dF, dI, dfo = _d_integrals(h, eri, en, beta, mu, dbeta, dmu)

    # Omega_0 + Omega_1
    gp0 = ft_utils.GP0(beta, en, mu)
    d0 = (-fo * dmu + (-gp0 / beta + (en - mu) * fo / beta) * dbeta).sum()
    W = einsum('ijij->ij', eri)
    d1 = (numpy.diag(h) - en) @ dfo + fo @ W @ dfo

    # Omega_cc: explicit integral dependence, (1/beta) sum_x g_x [E(T_x; dF, dI) + <M_int, dS>]
    L1int = quadrature.int_L1(ng, L1, ti, D1, g, G)
    L2int = quadrature.int_L2(ng, L2, ti, D2, g, G)
    dS1 = numpy.repeat(-dF.vo[None], ng, axis=0)
    dS2 = numpy.repeat(-dI.vvoo[None], ng, axis=0)
    for y in range(ng):
        cc_equations.stanton(dS1[y], dS2[y], dF, dI, T1[y], T2[y], fac=-1.0)
    dcc = ft_ccsd.ft_cc_energy(T1, T2, dF.ov, dI.oovv, g, beta)
    dcc -= _lam_dot(L1int, L2int, dS1, dS2, g) / beta
    if dbeta != 0.0:
        # 1/beta and g = beta g^: their beta derivatives cancel.  G = beta G^ and
        # t = beta t^: d/dbeta of sum_x G[y,x] e^{(t_x-t_y)D} S_x (ccsd.py:1114-1146)
        S1, S2 = _tbar(F, I, T1, T2, ng)
        Gd = G / beta
        Gt = G * (ti[None, :] - ti[:, None]) / beta
        P1 = quadrature.int_tbar1(ng, S1, ti, D1, Gd) \
            + D1[None] * quadrature.int_tbar1(ng, S1, ti, D1, Gt)
        P2 = quadrature.int_tbar2(ng, S2, ti, D2, Gd) \
            + D2[None] * quadrature.int_tbar2(ng, S2, ti, D2, Gt)
        dcc -= dbeta * _lam_dot(L1, L2, P1, P2, g) / beta
    return d0 + d1 + dcc


def ft_esn(en, h, eri, beta, mu, ngrid, quad, T1, T2, L1, L2, E_const=0.0):
    """(E, S, N, Omega) from converged T and Lambda (ccsd.py:167-214):
    N = -dOmega/dmu, E = Omega + beta dOmega/dbeta + mu N,
    S = beta (E - Omega - mu N)."""
    fo = ft_utils.ff(beta, en, mu)
    F, I = ft_ccsd.ft_integrals(mean_field(h, eri, fo), eri, en, beta, mu)
    ti, g, G = quadrature.ft_quad(ngrid, beta, quad)
    O0, O1 = omega_ref(en, h, eri, beta, mu, E_const)
    Om = O0 + O1 + ft_ccsd.ft_cc_energy(T1, T2, F.ov, I.oovv, g, beta)
    dmu = omega_derivative(en, h, eri, beta, mu, ngrid, quad, T1, T2, L1, L2, 0.0, 1.0)
    dbe = omega_derivative(en, h, eri, beta, mu, ngrid, quad, T1, T2, L1, L2, 1.0, 0.0)
    N = -dmu
    E = Om + beta * dbe + mu * N
    S = beta * (E - Om - mu * N)
    return E, S, N, Om


def solve(en, h, eri, T, mu, ngrid=10, quad='lin', damp=0.0, econv=1e-10, max_iter=100,
          lconv=1e-10, E_const=0.0, T1in=None, T2in=None, history=None, spin_half=None):
    """T solve (ft_ccsd.ft_ccsd), Lambda solve from Kelvin's guess, then
    (E, S, N, Omega, T1, T2, L1, L2).  ``history`` receives the Lambda
    residuals; ``spin_half`` (alpha spin orbitals first) starts and measures
    the Lambda iteration as Kelvin's unrestricted driver does."""
    beta = 1.0 / T
    fo = ft_utils.ff(beta, en, mu)
    fock = mean_field(h, eri, fo)
    O0, O1 = omega_ref(en, h, eri, beta, mu, E_const)
    _, T1, T2 = ft_ccsd.ft_ccsd(en, fock, eri, T, mu, ngrid=ngrid, quad=quad, econv=econv,
                                max_iter=max_iter, damp=damp, E_const=E_const, E1=O1,
                                T1in=T1in, T2in=T2in, return_amplitudes=True)
    ti, g, G = quadrature.ft_quad(ngrid, beta, quad)
    F, I = ft_ccsd.ft_integrals(fock, eri, en, beta, mu)
    L1, L2 = lambda_guess(F, I, T1, beta, ngrid, unrestricted=spin_half is not None)
    conv = {"tconv": lconv, "max_iter": max_iter, "damp": damp}
    L1, L2 = ft_lambda_iter(L1, L2, T1, T2, F, I, ft_utils.D1(en, en), ft_utils.D2(en, en),
                            g, G, beta, ngrid, ti, conv, history=history,
                            spin_half=spin_half)
    E, S, N, Om = ft_esn(en, h, eri, beta, mu, ngrid, quad, T1, T2, L1, L2, E_const)
    return E, S, N, Om, T1, T2, L1, L2


def _asym(x, pairs):
    """Antisymmetric part of x in each listed index pair ((0, 1) and/or (2, 3))."""
    for p in pairs:
        perm = [0, 1, 2, 3]
        perm[p[0]], perm[p[1]] = perm[p[1]], perm[p[0]]
        x = 0.5 * (x - x.transpose(perm))
    return x


# Kelvin's two-electron response densities: (name, integral block, weight,
# antisymmetric pairs of the density); the density is the integral block's
# gradient with bra and ket swapped, Omega_cc = (1/beta) sum_b w_b P_b . I_b
# (kelvin/tests/test_ft_cc_2rdm.py:127-135)
P2_BLOCKS = (("cdab", "vvvv", 0.25, ((0, 1), (2, 3))),
             ("ciab", "vvvo", 0.5, ((2, 3),)),
             ("bcai", "vovv", 0.5, ((0, 1),)),
             ("ijab", "vvoo", 0.25, ((0, 1), (2, 3))),
             ("bjai", "vovo", 1.0, ()),
             ("abij", "oovv", 0.25, ((0, 1), (2, 3))),
             ("jkai", "vooo", 0.5, ((0, 1),)),
             ("kaij", "ooov", 0.5, ((2, 3),)),
             ("klij", "oooo", 0.25, ((0, 1), (2, 3))))


def response_densities(F, I, T1, T2, L1, L2, D1, D2, ti, ng, g, G):
    """Kelvin's unrelaxed response densities (ft_cc_equations.py:704-753):
    (pia, pba, pji, pai) and the nine P2 blocks in P2_BLOCKS order, the
    gradients (times beta) of the Lagrangian

        (1/beta) sum_x g_x [E(T_x) + <int_L(L)_x, F.vo + I.vvoo + R(T_x)>]

    with respect to the integral blocks, which equals Omega_cc at convergence
    and is linear in the integrals."""
    Fs, Is = integral_gradients(F, I, T1, T2, L1, L2, D1, D2, ti, ng, g, G)
    pia, pba, pji, pai = Fs.vo.T, Fs.vv.T, Fs.oo.T, Fs.ov.T
    P2 = tuple(_asym(getattr(Is, blk).transpose(2, 3, 0, 1) / w, pairs)
               for _, blk, w, pairs in P2_BLOCKS)
    return (pia, pba, pji, pai), P2


def integral_gradients(F, I, T1, T2, L1, L2, D1, D2, ti, ng, g, G):
    """The Lagrangian's gradients with respect to every entry of every F and
    I block, in the blocks' own layouts (containers like F, I)."""
    L1int = quadrature.int_L1(ng, L1, ti, D1, g, G)
    L2int = quadrature.int_L2(ng, L2, ti, D2, g, G)
    Fs, Is = _Grad(F), _Grad(I)
    for y in range(ng):
        _, _, Fg, Ig = residual_vjp(F, I, T1[y], T2[y], L1int[y].T,
                                    L2int[y].transpose(2, 3, 0, 1), integrals=True)
        for k in vars(Fs):
            getattr(Fs, k).__iadd__(g[y] * getattr(Fg, k))
        for k in vars(Is):
            getattr(Is, k).__iadd__(g[y] * getattr(Ig, k))
    # the energy functional's own dependence (ft_cc_energy.py:7-32)
    Fs.ov += einsum('y,yai->ia', g, T1)
    Is.oovv += einsum('y,yabij->ijab', g, 0.25 * T2 + 0.5 * einsum('yai,ybj->yabij', T1, T1))
    # the driving terms F.vo and I.vvoo enter with int_L(L) itself
    Fs.vo += einsum('y,yia->ai', g, L1int)
    Is.vvoo += 0.25 * einsum('y,yijab->abij', g, L2int)
    return Fs, Is


def normal_ordered_rdms(beta, fo, fv, P1, P2):
    """Normal-ordered 1- and 2-RDMs from the response densities
    (ccsd.py:1333-1388 _g_ft_1rdm, cc_utils.py:1449-1466 g_n2rdm_full):
    sum_pq n1[p,q] dfock[q,p] + 1/4 sum_pqrs n2[p,q,r,s] d<rs||pq> = dOmega_cc
    at fixed occupations."""
    so, sv = numpy.sqrt(fo), numpy.sqrt(fv)
    pia, pba, pji, pai = P1
    n1 = (pia * so[:, None] * sv[None, :] + pba * sv[:, None] * sv[None, :]
          + pji * so[:, None] * so[None, :] + pai * sv[:, None] * so[None, :]) / beta
    s = {'o': so, 'v': sv}
    n2 = 0.0
    for (name, blk, w, pairs), P in zip(P2_BLOCKS, P2):
        f = [s[c] for c in blk[2:] + blk[:2]]          # density index types
        x = P * (f[0][:, None, None, None] * f[1][None, :, None, None]
                 * f[2][None, None, :, None] * f[3][None, None, None, :]) / beta
        # spread over the index orders that the antisymmetry of <pq||rs> makes
        # equivalent and that the block itself does not already cover
        terms = [x]
        if (0, 1) not in pairs and blk[2] != blk[3]:
            terms += [-t.transpose(1, 0, 2, 3) for t in terms]
        if (2, 3) not in pairs and blk[0] != blk[1]:
            terms += [-t.transpose(0, 1, 3, 2) for t in terms]
        n2 = n2 + sum(terms)
    return n1, n2
