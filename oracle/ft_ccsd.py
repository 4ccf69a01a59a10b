"""FT-CCSD amplitude iteration, general-spin (oracle; test infrastructure).

Restates, in numpy FP64:

* ``ccsd_stanton``   -- kelvin/ft_cc_equations.py:96-113
* ``ft_cc_energy``   -- kelvin/ft_cc_energy.py:7-32
* ``ft_cc_iter``     -- kelvin/cc_utils.py:111-173
* ``ft_cc_iter_extrap`` -- kelvin/cc_utils.py:176-242 (tau-pointwise schedule)
* ``ft_integrals``   -- kelvin/cc_utils.py:569-602
* ``ft_ccsd``        -- kelvin/ccsd.py:595-712 (finite-T, orbtype 'g')
"""
import logging
import numpy

from . import cc_equations
from . import ft_utils
from . import quadrature

einsum = cc_equations.einsum


def ccsd_stanton(F, I, T1old, T2old, D1, D2, ti, ng, G, full=False):
    """One FT-CCSD amplitude update (ft_cc_equations.py:96-113)."""
    T1new = numpy.repeat(-F.vo[None], ng, axis=0)
    T2new = numpy.repeat(-I.vvoo[None], ng, axis=0)
    for y in range(ng):
        cc_equations.stanton(T1new[y], T2new[y], F, I, T1old[y], T2old[y],
                             fac=-1.0)
    T1new = quadrature.int_tbar1(ng, T1new, ti, D1, G, full=full)
    T2new = quadrature.int_tbar2(ng, T2new, ti, D2, G, full=full)
    return T1new, T2new


def ccsd_stanton_single(ig, F, I, T1old, T2old, T1bar, T2bar, D1, D2, ti, ng, G):
    """Pointwise update at grid point ig (ft_cc_equations.py:116-127)."""
    T1new = -F.vo.copy()
    T2new = -I.vvoo.copy()
    cc_equations.stanton(T1new, T2new, F, I, T1old, T2old, fac=-1.0)
    T1bar[ig] = T1new
    T2bar[ig] = T2new
    return (quadrature.int_tbar1_single(ng, ig, T1bar, ti, D1, G),
            quadrature.int_tbar2_single(ng, ig, T2bar, ti, D2, G))


def ft_cc_energy(T1, T2, f, eri, g, beta, Qterm=True):
    """FT-CC grand potential correction (ft_cc_energy.py:7-32)."""
    if Qterm:
        t2 = 0.25 * T2 + 0.5 * einsum('yai,ybj->yabij', T1, T1)
    else:
        t2 = 0.25 * T2
    t1n = einsum('y,yai->ai', g, T1)
    t2n = einsum('y,yabij->abij', g, t2)
    return (einsum('ai,ia->', t1n, f) + einsum('abij,ijab->', t2n, eri)) / beta


def ft_cc_iter(method, T1old, T2old, F, I, D1, D2, g, G, beta, ng, ti,
               iprint, conv_options, full=False, history=None):
    """Damped fixed-point iteration (cc_utils.py:111-173).

    ``history``, when a list, receives (E, res1 + res2) per iteration.
    """
    if method != "CCSD":
        raise Exception("Unrecognized method keyword")
    ethresh = conv_options["econv"]
    tthresh = conv_options["tconv"]
    max_iter = conv_options["max_iter"]
    alpha = conv_options["damp"]
    converged = False
    Eold = 888888888.888888888
    nl1 = numpy.linalg.norm(T1old) + 0.1
    nl2 = numpy.linalg.norm(T2old) + 0.1
    i = 0
    while i < max_iter and not converged:
        T1, T2 = ccsd_stanton(F, I, T1old, T2old, D1, D2, ti, ng, G, full=full)
        res1 = numpy.linalg.norm(T1 - T1old) / nl1
        res2 = numpy.linalg.norm(T2 - T2old) / nl2
        T1old = alpha * T1old + (1.0 - alpha) * T1
        T2old = alpha * T2old + (1.0 - alpha) * T2
        nl1 = numpy.linalg.norm(T1old) + 0.1
        nl2 = numpy.linalg.norm(T2old) + 0.1
        E = ft_cc_energy(T1old, T2old, F.ov, I.oovv, g, beta)
        logging.info(' %2d  %.10f   %.4E' % (i + 1, E, res1 + res2))
        if history is not None:
            history.append((E, res1 + res2))
        i += 1
        if numpy.abs(E - Eold) < ethresh and res1 + res2 < tthresh:
            converged = True
        Eold = E
    if not converged:
        logging.warning("{} did not converge!".format(method))
    return Eold, T1old, T2old


def ft_cc_iter_extrap(method, F, I, D1, D2, g, G, beta, ng, ti, iprint,
                      conv_options):
    """Converge grid point by grid point (cc_utils.py:176-242)."""
    thresh = conv_options["tconv"]
    max_iter = conv_options["max_iter"]
    alpha = conv_options["damp"]
    nv, no = F.vo.shape
    t1bar = numpy.zeros((ng, nv, no))
    t2bar = numpy.zeros((ng, nv, nv, no, no))
    T1new = numpy.zeros((ng, nv, no))
    T2new = numpy.zeros((ng, nv, nv, no, no))
    for ig in range(ng):
        if ig == 0:
            t1bar[0] = -F.vo
            t2bar[0] = -I.vvoo
            continue
        elif ig == 1:
            t1bar[ig] = -F.vo
            t2bar[ig] = -I.vvoo
            T1new[ig] = quadrature.int_tbar1_single(ng, ig, t1bar, ti, D1, G)
            T2new[ig] = quadrature.int_tbar2_single(ng, ig, t2bar, ti, D2, G)
        else:
            c = (ti[ig] - ti[ig - 1]) / (ti[ig - 2] - ti[ig - 1])
            T1new[ig] = T1new[ig - 1] + (T1new[ig - 2] - T1new[ig - 1]) * c
            T2new[ig] = T2new[ig - 1] + (T2new[ig - 2] - T2new[ig - 1]) * c
        nl1 = numpy.sqrt(float(T1new[ig].size))
        nl2 = numpy.sqrt(float(T2new[ig].size))
        converged = False
        i = 0
        while i < max_iter and not converged:
            T1, T2 = ccsd_stanton_single(ig, F, I, T1new[ig], T2new[ig],
                                         t1bar, t2bar, D1, D2, ti, ng, G)
            res1 = numpy.linalg.norm(T1 - T1new[ig]) / nl1
            res2 = numpy.linalg.norm(T2 - T2new[ig]) / nl2
            T1new[ig] = alpha * T1new[ig] + (1.0 - alpha) * T1
            T2new[ig] = alpha * T2new[ig] + (1.0 - alpha) * T2
            i += 1
            if res1 + res2 < thresh:
                converged = True
    return T1new, T2new


def ft_integrals(fock, eri, en, beta, mu):
    """Fermi-factor-scaled Fock and ERI blocks (cc_utils.py:569-602).

    ``fock`` is the full FT Fock matrix (System.g_fock_tot), ``eri`` the
    antisymmetrised integrals (System.g_aint_tot), ``en`` the orbital energies.
    """
    sfo = numpy.sqrt(ft_utils.ff(beta, en, mu))
    sfv = numpy.sqrt(ft_utils.ffv(beta, en, mu))
    fmo = fock - numpy.diag(en)
    s = {'o': sfo, 'v': sfv}
    F = ft_utils.one_e_blocks(
        *[fmo * s[b[0]][:, None] * s[b[1]][None, :] for b in ('oo', 'ov', 'vo', 'vv')])
    blocks = {}
    for name in ft_utils.two_e_blocks.NAMES:
        p, q, r, t = (s[c] for c in name)
        blocks[name] = eri * (p[:, None, None, None] * q[None, :, None, None]
                              * r[None, None, :, None] * t[None, None, None, :])
    return F, ft_utils.two_e_blocks(**blocks)


def ft_ccsd(en, fock, eri, T, mu, ngrid=10, quad='lin', econv=1e-8, tconv=None,
            max_iter=40, damp=0.0, E_const=0.0, E1=0.0, T1in=None, T2in=None,
            full=None, history=None, return_amplitudes=False):
    """Finite-T general-spin CCSD (ccsd.py:43-76 set-up, 595-712 solve).

    Returns (Omega_total, Omega_cc) like ``ccsd.run``; E1 is the first-order
    grand potential ``System.get_mp1()`` and E_const ``System.const_energy()``.
    """
    beta = 1.0 / T
    tconv = tconv if tconv is not None else 1000.0 * econv
    ti, g, G = quadrature.ft_quad(ngrid, beta, quad)
    if full is None:
        full = (quad == 'gl')
    ng = ngrid
    n = en.shape[0]
    D1 = ft_utils.D1(en, en)
    D2 = ft_utils.D2(en, en)
    E0 = ft_utils.GP0(beta, en, mu).sum() + E_const
    F, I = ft_integrals(fock, eri, en, beta, mu)
    if T1in is not None and T2in is not None:
        T1old, T2old = T1in, T2in
    else:
        T1old = quadrature.int_tbar1(ng, numpy.repeat(-F.vo[None], ng, 0), ti, D1, G, full=full)
        T2old = quadrature.int_tbar2(ng, numpy.repeat(-I.vvoo[None], ng, 0), ti, D2, G, full=full)
    conv = {"econv": econv, "tconv": tconv, "max_iter": max_iter, "damp": damp}
    Ecc, T1, T2 = ft_cc_iter("CCSD", T1old, T2old, F, I, D1, D2, g, G, beta,
                             ng, ti, 0, conv, full=full, history=history)
    out = (Ecc + E0 + E1, Ecc)
    if return_amplitudes:
        return out, T1, T2
    return out
