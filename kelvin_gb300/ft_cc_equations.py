"""FT-CCSD amplitude update on the GPU, drop-in for kelvin/ft_cc_equations.py.

``ccsd_stanton(F, I, T1old, T2old, D1, D2, ti, ng, G)`` has Kelvin's signature
and semantics (ft_cc_equations.py:96-113): for every tau point the CCSD
residual with Stanton-Gauss intermediates gives tbar = -F.vo - R1(t),
-I.vvoo - R2(t); the result is integrated in imaginary time.  Inputs are
never modified; new arrays are returned.  numpy inputs give numpy outputs;
``DeviceArray`` amplitudes give device outputs.
"""
import zlib

import numpy

from . import _lib

F_ORDER = ("oo", "ov", "vo", "vv")
I_ORDER = ("vvvv", "vvvo", "vovv", "vvoo", "vovo", "oovv", "vooo", "ooov", "oooo")


class DeviceBlocks(object):
    """Device copies of Kelvin's one_e_blocks / two_e_blocks containers."""

    def __init__(self, ctx, F, I):
        self.F = [_lib.as_device(ctx, getattr(F, b)) for b in F_ORDER]
        self.I = [_lib.as_device(ctx, getattr(I, b)) for b in I_ORDER]
        nv, no = self.F[2].shape
        self.nv, self.no = nv, no
        self.Fp = _lib.ptr_array(self.F)
        self.Ip = _lib.ptr_array(self.I)


_cache = {}


def _fingerprint(F, I):
    """Content key of the host blocks of (F, I): shape and a CRC of the bytes
    of every block, so that a block changed in place is uploaded again.  Device blocks are used where they lie and need no key beyond
    their address."""
    key = []
    for c, order in ((F, F_ORDER), (I, I_ORDER)):
        for b in order:
            a = getattr(c, b)
            if isinstance(a, _lib.DeviceArray):
                key.append(("d", a.ptr.value))
                continue
            a = numpy.ascontiguousarray(a, dtype=float)
            key.append((a.shape, zlib.crc32(memoryview(a).cast("B"))))
    return tuple(key)


def device_blocks(ctx, F, I):
    """Device blocks for (F, I), reused while the same contents are passed."""
    key = (ctx.device, _fingerprint(F, I))
    hit = _cache.get(key)
    if hit is not None:
        return hit
    blk = DeviceBlocks(ctx, F, I)
    _cache.clear()
    _cache[key] = blk
    return blk


def ccsd_stanton(F, I, T1old, T2old, D1, D2, ti, ng, G, full=False, ctx=None,
                 precision=None):
    """Time-dependent CCSD iteration with Stanton-Gauss intermediates."""
    ctx = ctx or _lib.context()
    if precision is not None:
        ctx.set_precision(*precision) if isinstance(precision, tuple) \
            else ctx.set_precision(precision)
    host = not isinstance(T1old, _lib.DeviceArray)
    blk = device_blocks(ctx, F, I)
    nv, no = blk.nv, blk.no
    if tuple(T1old.shape) != (ng, nv, no) or tuple(T2old.shape) != (ng, nv, nv, no, no):
        raise Exception("ccsd_stanton: amplitude shapes do not match F.vo / ng")
    d1, d2 = _lib.as_device(ctx, T1old), _lib.as_device(ctx, T2old)
    dD1, dD2, dti, dG = (_lib.as_device(ctx, a) for a in (D1, D2, ti, G))
    o1 = _lib.DeviceArray(ctx, (ng, nv, no))
    o2 = _lib.DeviceArray(ctx, (ng, nv, nv, no, no))
    ctx.check(ctx.L.kvft_ccsd_stanton(ctx.h, ng, nv, no, blk.Fp, blk.Ip, d1.ptr, d2.ptr,
                                      dD1.ptr, dD2.ptr, dti.ptr, dG.ptr, int(bool(full)),
                                      o1.ptr, o2.ptr), "ccsd_stanton")
    if host:
        return o1.to_host(), o2.to_host()
    return o1, o2


def stanton_residual(T1, T2, F, I, t1, t2, fac=1.0, ctx=None):
    """In-place T1 += fac R1(t1,t2), T2 += fac R2 for one tau point: the
    contract of cqcpy.cc_equations._Stanton called at ft_cc_equations.py:106."""
    ctx = ctx or _lib.context()
    blk = device_blocks(ctx, F, I)
    nv, no = blk.nv, blk.no
    dT1, dT2 = _lib.as_device(ctx, T1), _lib.as_device(ctx, T2)
    dt1, dt2 = _lib.as_device(ctx, t1), _lib.as_device(ctx, t2)
    ctx.check(ctx.L.kvft_stanton_residual(ctx.h, 1, nv, no, blk.Fp, blk.Ip, dt1.ptr, dt2.ptr,
                                          float(fac), dT1.ptr, dT2.ptr), "stanton_residual")
    if isinstance(T1, numpy.ndarray):
        dT1.to_host(T1)
        dT2.to_host(T2)


# ---- unrestricted (spin-blocked) form -------------------------------------------
# Kelvin's unrestricted update (ft_cc_equations.py:130-164) takes the alpha and
# beta blocks separately: Fa, Fb (one_e_blocks), Ia, Ib (antisymmetrised
# same-spin two_e_blocks), Iabab (<ab|ab> with alpha indices 1, 3 and beta 2, 4,
# all sixteen o/v blocks), T1a, T1b, T2aa, T2ab[a,b,i,j] (a, i alpha; b, j beta),
# T2bb and their denominators.  Here they are laid out as one general-spin
# problem with the alpha spin orbitals first; the solver finds its spin blocks
# and contracts only those, so the work is that of the spin-blocked equations.

class _Blocks(object):
    def __init__(self, **kw):
        self.__dict__.update(kw)


def u_to_g_one(Fa, Fb):
    """General-spin one_e_blocks from the alpha and beta blocks."""
    out = {}
    for t in F_ORDER:
        fa, fb = getattr(Fa, t), getattr(Fb, t)
        na, nb = fa.shape[0], fb.shape[0]
        g = numpy.zeros((na + nb, na + nb), dtype=fa.dtype)
        g[:na, :na] = fa
        g[na:, na:] = fb
        out[t] = g
    return _Blocks(**out)


def u_to_g_two(Ia, Ib, Iabab):
    """General-spin antisymmetrised blocks <pq||rs> from Ia, Ib and Iabab."""
    out = {}
    for t in I_ORDER:
        ia, ib = getattr(Ia, t), getattr(Ib, t)
        na, nb = ia.shape[0], ib.shape[0]
        n = na + nb
        A, B = slice(0, na), slice(na, n)
        g = numpy.zeros((n, n, n, n), dtype=ia.dtype)
        g[A, A, A, A] = ia
        g[B, B, B, B] = ib
        g[A, B, A, B] = getattr(Iabab, t)
        # <Pq||Rs> = <qP||sR>, <pQ||Rs> = -<pQ||sR>, <Pq||rS> = -<qP||rS>
        g[B, A, B, A] = getattr(Iabab, t[1] + t[0] + t[3] + t[2]).transpose(1, 0, 3, 2)
        g[A, B, B, A] = -getattr(Iabab, t[0] + t[1] + t[3] + t[2]).transpose(0, 1, 3, 2)
        g[B, A, A, B] = -getattr(Iabab, t[1] + t[0] + t[2] + t[3]).transpose(1, 0, 2, 3)
        out[t] = g
    return _Blocks(**out)


def u_to_g_t1(T1a, T1b):
    """[ng][n][n] from [ng][na][na] and [ng][nb][nb] (spin-diagonal)."""
    ng, na, nb = T1a.shape[0], T1a.shape[1], T1b.shape[1]
    g = numpy.zeros((ng, na + nb, na + nb), dtype=T1a.dtype)
    g[:, :na, :na] = T1a
    g[:, na:, na:] = T1b
    return g


def u_to_g_t2(T2aa, T2ab, T2bb):
    """[ng][n]^4 from the three spin cases (antisymmetric completion)."""
    ng, na, nb = T2aa.shape[0], T2aa.shape[1], T2bb.shape[1]
    n = na + nb
    A, B = slice(0, na), slice(na, n)
    g = numpy.zeros((ng, n, n, n, n), dtype=T2aa.dtype)
    g[:, A, A, A, A] = T2aa
    g[:, B, B, B, B] = T2bb
    g[:, A, B, A, B] = T2ab
    g[:, B, A, B, A] = T2ab.transpose(0, 2, 1, 4, 3)
    g[:, A, B, B, A] = -T2ab.transpose(0, 1, 2, 4, 3)
    g[:, B, A, A, B] = -T2ab.transpose(0, 2, 1, 3, 4)
    return g


def u_to_g_d1(D1a, D1b):
    na, nb = D1a.shape[0], D1b.shape[0]
    g = numpy.zeros((na + nb, na + nb), dtype=D1a.dtype)
    g[:na, :na] = D1a
    g[na:, na:] = D1b
    return g


def u_to_g_d2(D2aa, D2ab, D2bb):
    """Denominators of the spin-conserving blocks (zero elsewhere: those
    amplitudes vanish and stay zero)."""
    na, nb = D2aa.shape[0], D2bb.shape[0]
    n = na + nb
    A, B = slice(0, na), slice(na, n)
    g = numpy.zeros((n, n, n, n), dtype=D2aa.dtype)
    g[A, A, A, A] = D2aa
    g[B, B, B, B] = D2bb
    g[A, B, A, B] = D2ab
    g[B, A, B, A] = D2ab.transpose(1, 0, 3, 2)
    g[A, B, B, A] = D2ab.transpose(0, 1, 3, 2)
    g[B, A, A, B] = D2ab.transpose(1, 0, 2, 3)
    return g


def g_to_u_t(T1, T2, na):
    """Unrestricted blocks ((T1a, T1b), (T2aa, T2ab, T2bb)) of general-spin
    amplitudes with the alpha spin orbitals first."""
    A, B = slice(0, na), slice(na, T1.shape[1])
    return ((T1[:, A, A].copy(), T1[:, B, B].copy()),
            (T2[:, A, A, A, A].copy(), T2[:, A, B, A, B].copy(), T2[:, B, B, B, B].copy()))


def uccsd_stanton(Fa, Fb, Ia, Ib, Iabab, T1aold, T1bold, T2aaold, T2abold, T2bbold,
                  D1a, D1b, D2aa, D2ab, D2bb, ti, ng, G, ctx=None, precision=None):
    """Unrestricted FT-CCSD update (ft_cc_equations.py:130-164): returns
    ((T1a, T1b), (T2aa, T2ab, T2bb)).  Runs as one general-spin update with
    the alpha spin orbitals first, restricted to its spin-conserving blocks."""
    F = u_to_g_one(Fa, Fb)
    I = u_to_g_two(Ia, Ib, Iabab)
    T1 = u_to_g_t1(numpy.asarray(T1aold), numpy.asarray(T1bold))
    T2 = u_to_g_t2(numpy.asarray(T2aaold), numpy.asarray(T2abold), numpy.asarray(T2bbold))
    D1 = u_to_g_d1(D1a, D1b)
    D2 = u_to_g_d2(D2aa, D2ab, D2bb)
    o1, o2 = ccsd_stanton(F, I, T1, T2, D1, D2, ti, ng, G, ctx=ctx, precision=precision)
    return g_to_u_t(o1, o2, Fa.vo.shape[0])


# ---- Lambda equations -------------------------------------------------------------
# Kelvin's Lambda update (ft_cc_equations.py:385-409) and guess (:502-512).  The
# Lambda terms are the transpose of the residual's Jacobian, evaluated on the
# device (kvft_ccsd_lambda) as the reverse pass through the Stanton
# intermediates; L1[y][i][a] and L2[y][i][j][a][b] keep Kelvin's layout.


def energies_from_d1(D1):
    """Orbital energies (ev, eo) with ev[a] - eo[i] = D1[a, i]; the
    exponentials of the integrals depend on these differences only."""
    D1 = numpy.asarray(D1, dtype=float)
    ev, eo = D1[:, 0].copy(), D1[0, 0] - D1[0, :]
    if abs(ev[:, None] - eo[None, :] - D1).max() > 1e-12 * (1.0 + abs(D1).max()):
        raise Exception("D1 is not a difference of orbital energies")
    return numpy.ascontiguousarray(ev), numpy.ascontiguousarray(eo)


def spin_half_of(nv, no, arrays):
    """h when every array (host arrays: integral blocks, or amplitudes with a
    leading tau axis) vanishes outside the spin-conserving blocks of an
    alpha-first layout with nv = no = 2h, else 0: the condition under which
    the Lambda path may run its contractions over spin-block products only."""
    if nv != no or nv % 2 or nv == 0:
        return 0
    h = nv // 2
    sp = (numpy.arange(nv) >= h).astype(int)
    one = sp[:, None] != sp[None, :]
    two = (sp[:, None, None, None] + sp[None, :, None, None]
           != sp[None, None, :, None] + sp[None, None, None, :])
    for a in arrays:
        if isinstance(a, _lib.DeviceArray):
            return 0
        a = numpy.asarray(a)
        mask = one if a.ndim in (2, 3) else two
        if a.ndim in (3, 5):
            a = numpy.abs(a).max(axis=0)
        if numpy.any(a[mask] != 0.0):
            return 0
    return h


class _SpinBlocks(object):
    """Spin blocks of the Lambda path for the duration of a call."""

    def __init__(self, ctx, h):
        self.ctx, self.h = ctx, h

    def __enter__(self):
        self.ctx.check(self.ctx.L.kvft_set_lambda_spin_blocks(self.ctx.h, self.h),
                       "set_lambda_spin_blocks")

    def __exit__(self, *exc):
        self.ctx.L.kvft_set_lambda_spin_blocks(self.ctx.h, 0)


def ccsd_lambda_guess(F, I, T1old, beta, ng, unrestricted=False):
    """Kelvin's starting Lambda: (1/beta)(F.ov + I.oovv T1, I.oovv) at every
    tau point (host arrays, ft_cc_equations.py:502-512); ``unrestricted``
    gives its unrestricted driver's guess, whose I.oovv T1 term has no 1/beta
    (ft_cc_equations.py:515-526)."""
    T1 = numpy.asarray(T1old)
    it1 = numpy.einsum('ijab,ybj->yia', I.oovv, T1)
    L1 = numpy.asarray(F.ov)[None] / beta + (it1 if unrestricted else it1 / beta)
    L2 = numpy.repeat(numpy.asarray(I.oovv)[None] / beta, ng, axis=0)
    return L1, L2


def ccsd_lambda_opt(F, I, T1old, T2old, L1old, L2old, D1, D2, ti, ng, g, G, beta, ctx=None,
                    precision=None, energies=None):
    """One Lambda update on the GPU: L = -E'(T) - R'(T)^T int_L(L_old) per
    tau point, with Kelvin's signature (ft_cc_equations.py:385-409; beta and
    D2 are implied by the grid and D1).  numpy Lambda gives numpy outputs,
    DeviceArray Lambda device outputs.  ``energies`` = (ev, eo) replaces the
    orbital energies read off D1."""
    ctx = ctx or _lib.context()
    if precision is not None:
        ctx.set_precision(*precision) if isinstance(precision, tuple) \
            else ctx.set_precision(precision)
    host = not isinstance(L1old, _lib.DeviceArray)
    blk = device_blocks(ctx, F, I)
    nv, no = blk.nv, blk.no
    if tuple(T1old.shape) != (ng, nv, no) or tuple(L1old.shape) != (ng, no, nv) or \
            tuple(L2old.shape) != (ng, no, no, nv, nv):
        raise Exception("ccsd_lambda_opt: amplitude shapes do not match F.vo / ng")
    ev, eo = energies if energies is not None else energies_from_d1(D1)
    dT1, dT2 = _lib.as_device(ctx, T1old), _lib.as_device(ctx, T2old)
    dL1, dL2 = _lib.as_device(ctx, L1old), _lib.as_device(ctx, L2old)
    dev, deo, dti, dg, dG = (_lib.as_device(ctx, numpy.ascontiguousarray(a, dtype=float))
                             for a in (ev, eo, ti, g, G))
    o1 = _lib.DeviceArray(ctx, (ng, no, nv))
    o2 = _lib.DeviceArray(ctx, (ng, no, no, nv, nv))
    blocks = [getattr(F, b) for b in F_ORDER] + [getattr(I, b) for b in I_ORDER]
    with _SpinBlocks(ctx, spin_half_of(nv, no, blocks + [T1old, T2old, L1old, L2old])):
        ctx.check(ctx.L.kvft_ccsd_lambda(ctx.h, ng, nv, no, blk.Fp, blk.Ip, dT1.ptr, dT2.ptr,
                                         dL1.ptr, dL2.ptr, dev.ptr, deo.ptr, dti.ptr, dg.ptr,
                                         dG.ptr, o1.ptr, o2.ptr), "ccsd_lambda_opt")
    if host:
        return o1.to_host(), o2.to_host()
    return o1, o2


# ---- response densities ------------------------------------------------------------
# Kelvin's ccsd_1rdm / ccsd_2rdm (ft_cc_equations.py:704-753) from T and Lambda.
# They are the gradients of the Lagrangian with respect to the integral blocks,
# which do not depend on the integrals' values (the Lagrangian is linear in
# them); kvft_lambda_densities evaluates them on the device.  Two-electron
# densities carry Kelvin's names, weights and index orders: Omega_cc =
# (1/beta) sum_b w_b P_b . I_b (kelvin/tests/test_ft_cc_2rdm.py:127-135),
# antisymmetric in their same-type index pairs.
P2_BLOCKS = (("cdab", "vvvv", 0.25, ((0, 1), (2, 3))),
             ("ciab", "vvvo", 0.5, ((2, 3),)),
             ("bcai", "vovv", 0.5, ((0, 1),)),
             ("ijab", "vvoo", 0.25, ((0, 1), (2, 3))),
             ("bjai", "vovo", 1.0, ()),
             ("abij", "oovv", 0.25, ((0, 1), (2, 3))),
             ("jkai", "vooo", 0.5, ((0, 1),)),
             ("kaij", "ooov", 0.5, ((2, 3),)),
             ("klij", "oooo", 0.25, ((0, 1), (2, 3))))


def _antisym_pairs(x, pairs):
    for p in pairs:
        perm = [0, 1, 2, 3]
        perm[p[0]], perm[p[1]] = perm[p[1]], perm[p[0]]
        x = 0.5 * (x - x.transpose(perm))
    return x


def kelvin_densities(Fg, Ig):
    """(pia, pba, pji, pai), P2 from the integral gradients Fg (oo, ov, vo,
    vv) and Ig (Kelvin's nine blocks, I_ORDER), as dicts or sequences."""
    Fg = Fg if isinstance(Fg, dict) else dict(zip(F_ORDER, Fg))
    Ig = Ig if isinstance(Ig, dict) else dict(zip(I_ORDER, Ig))
    P1 = (Fg["vo"].T.copy(), Fg["vv"].T.copy(), Fg["oo"].T.copy(), Fg["ov"].T.copy())
    P2 = tuple(_antisym_pairs(Ig[blk].transpose(2, 3, 0, 1) / w, pairs)
               for _, blk, w, pairs in P2_BLOCKS)
    return P1, P2


def lambda_densities(T1, T2, L1, L2, D1, ti, ng, g, G, ctx=None):
    """Integral gradients (Fg, Ig) of the Lagrangian on the device."""
    ctx = ctx or _lib.context()
    _, nv, no = T1.shape
    ev, eo = energies_from_d1(D1)
    shp1 = {"oo": (no, no), "ov": (no, nv), "vo": (nv, no), "vv": (nv, nv)}
    ext = {"o": no, "v": nv}
    zF = [_lib.DeviceArray(ctx, shp1[b]) for b in F_ORDER]
    zI = [_lib.DeviceArray(ctx, tuple(ext[c] for c in b)) for b in I_ORDER]
    for a in zF + zI:
        a.zero()
    oF = [_lib.DeviceArray(ctx, shp1[b]) for b in F_ORDER]
    oI = [_lib.DeviceArray(ctx, tuple(ext[c] for c in b)) for b in I_ORDER]
    d = [_lib.as_device(ctx, a) for a in (T1, T2, L1, L2)]
    dv = [_lib.as_device(ctx, numpy.ascontiguousarray(a, dtype=float))
          for a in (ev, eo, ti, g, G)]
    with _SpinBlocks(ctx, spin_half_of(nv, no, [T1, T2, L1, L2])):
        ctx.check(ctx.L.kvft_lambda_densities(ctx.h, ng, nv, no, _lib.ptr_array(zF),
                                              _lib.ptr_array(zI), d[0].ptr, d[1].ptr, d[2].ptr,
                                              d[3].ptr, dv[0].ptr, dv[1].ptr, dv[2].ptr,
                                              dv[3].ptr, dv[4].ptr, _lib.ptr_array(oF),
                                              _lib.ptr_array(oI)), "lambda_densities")
    return [a.to_host() for a in oF], [a.to_host() for a in oI]


def ccsd_1rdm(T1, T2, L1, L2, D1, D2, ti, ng, g, G, ctx=None):
    """Kelvin's one-electron response densities (pia, pba, pji, pai)
    (ft_cc_equations.py:704-722)."""
    Fg, Ig = lambda_densities(T1, T2, L1, L2, D1, ti, ng, g, G, ctx=ctx)
    return kelvin_densities(Fg, Ig)[0]


def ccsd_2rdm(T1, T2, L1, L2, D1, D2, ti, ng, g, G, ctx=None):
    """Kelvin's nine two-electron response densities (Pcdab, Pciab, Pbcai,
    Pijab, Pbjai, Pabij, Pjkai, Pkaij, Pklij) (ft_cc_equations.py:725-753)."""
    Fg, Ig = lambda_densities(T1, T2, L1, L2, D1, ti, ng, g, G, ctx=ctx)
    return kelvin_densities(Fg, Ig)[1]


def normal_ordered_rdms(beta, fo, fv, P1, P2):
    """Normal-ordered 1- and 2-RDMs (ccsd.py:1333-1388 _g_ft_1rdm,
    cc_utils.py:1449-1466 g_n2rdm_full): sum n1[p,q] dfock[q,p] +
    1/4 sum n2[p,q,r,s] d<rs||pq> = dOmega_cc at fixed occupations."""
    so, sv = numpy.sqrt(fo), numpy.sqrt(fv)
    pia, pba, pji, pai = P1
    n1 = (pia * numpy.outer(so, sv) + pba * numpy.outer(sv, sv)
          + pji * numpy.outer(so, so) + pai * numpy.outer(sv, so)) / beta
    s = {'o': so, 'v': sv}
    n2 = 0.0
    for (name, blk, w, pairs), P in zip(P2_BLOCKS, P2):
        f = [s[c] for c in blk[2:] + blk[:2]]          # the density's index types
        x = P * numpy.einsum('p,q,r,s->pqrs', *f) / beta
        terms = [x]
        if (0, 1) not in pairs and blk[2] != blk[3]:
            terms += [-t.transpose(1, 0, 2, 3) for t in terms]
        if (2, 3) not in pairs and blk[0] != blk[1]:
            terms += [-t.transpose(0, 1, 3, 2) for t in terms]
        n2 = n2 + sum(terms)
    return n1, n2


# ---- unrestricted Lambda ----------------------------------------------------------
# Kelvin's uccsd_lambda_opt / uccsd_lambda_guess (ft_cc_equations.py:412-458,
# 515-526) take the spin cases separately; as for uccsd_stanton they are laid
# out as one general-spin problem (alpha spin orbitals first), which the
# unrestricted equations are the spin-blocked form of.  Lambda keeps Kelvin's
# layout per spin case: L1a[y][i][a], L2ab[y][i][j][a][b] (i, a alpha; j, b beta).


def uccsd_lambda_guess(Fa, Fb, Ia, Ib, Iabab, T1aold, T1bold, beta, ng):
    """Kelvin's unrestricted starting Lambda: (1/beta) F.ov plus I.oovv T1
    without the 1/beta (its _u_LS_TS at the default factor), and
    (1/beta) I.oovv, per spin case."""
    F, I = u_to_g_one(Fa, Fb), u_to_g_two(Ia, Ib, Iabab)
    T1 = u_to_g_t1(numpy.asarray(T1aold), numpy.asarray(T1bold))
    na = numpy.asarray(T1aold).shape[1]
    L1 = F.ov[None] / beta + numpy.einsum('ijab,ybj->yia', I.oovv, T1)
    L2 = numpy.repeat(I.oovv[None] / beta, ng, axis=0)
    (l1a, l1b), (l2aa, l2ab, l2bb) = g_to_u_t(L1, L2, na)
    return l1a, l1b, l2aa, l2ab, l2bb


def uccsd_lambda_opt(Fa, Fb, Ia, Ib, Iabab, T1aold, T1bold, T2aaold, T2abold, T2bbold,
                     L1aold, L1bold, L2aaold, L2abold, L2bbold, D1a, D1b, D2aa, D2ab, D2bb,
                     ti, ng, g, G, beta, ctx=None, precision=None):
    """One unrestricted Lambda update (ft_cc_equations.py:412-458) as the
    general-spin update on the device; returns (L1a, L1b, L2aa, L2ab, L2bb)."""
    na = numpy.asarray(T1aold).shape[1]
    F, I = u_to_g_one(Fa, Fb), u_to_g_two(Ia, Ib, Iabab)
    T1 = u_to_g_t1(numpy.asarray(T1aold), numpy.asarray(T1bold))
    T2 = u_to_g_t2(numpy.asarray(T2aaold), numpy.asarray(T2abold), numpy.asarray(T2bbold))
    L1 = u_to_g_t1(numpy.asarray(L1aold), numpy.asarray(L1bold))
    L2 = u_to_g_t2(numpy.asarray(L2aaold), numpy.asarray(L2abold), numpy.asarray(L2bbold))
    # energies per spin: D1a, D1b fix them up to one shift per spin, which
    # cancels in every spin-conserving denominator
    (eva, eoa), (evb, eob) = energies_from_d1(D1a), energies_from_d1(D1b)
    en = (numpy.concatenate((eva, evb)), numpy.concatenate((eoa, eob)))
    D1 = u_to_g_d1(numpy.asarray(D1a), numpy.asarray(D1b))
    o1, o2 = ccsd_lambda_opt(F, I, T1, T2, L1, L2, D1, None, ti, ng, g, G, beta, ctx=ctx,
                             precision=precision, energies=en)
    (l1a, l1b), (l2aa, l2ab, l2bb) = g_to_u_t(o1, o2, na)
    return l1a, l1b, l2aa, l2ab, l2bb
