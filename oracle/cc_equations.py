"""Spin-orbital CCSD residual with Stanton-Gauss intermediates (oracle).

Kelvin calls ``cqcpy.cc_equations._Stanton(T1, T2, F, I, t1, t2, fac)`` once per
tau point (kelvin/ft_cc_equations.py:105-107).  cqcpy is not vendored and has
no pinned version, so the residual is restated here from the published
equations (J. F. Stanton, J. Gauss, J. D. Watts, R. J. Bartlett, J. Chem.
Phys. 94, 4334 (1991)) in Kelvin's conventions:

* t1[a,i] = t_i^a, t2[a,b,i,j] = t_ij^ab (virtual indices first);
* F.oo[i,j], F.ov[i,a], F.vo[a,i], F.vv[a,b] -- Fock blocks whose diagonal
  orbital energies were already removed by the caller (cc_utils.py:578);
* I.<blk>[p,q,r,s] = <pq||rs> with p..s of the block's o/v types.

``stanton(T1, T2, F, I, t1, t2, fac)`` adds ``fac * R`` to T1/T2 in place,
where R is the CCSD residual without its driving terms F.vo / I.vvoo (the
caller seeds T1 = -F.vo, T2 = -I.vvoo and passes fac = -1, so that
T1bar = -(F.vo + R1), ft_cc_equations.py:101-107).

Integral identities used (antisymmetry of <pq||rs> in each pair):
<ma||fe> = -vovv[a,m,f,e];  <na||if> = vovo[a,n,f,i];
<nm||ei> = -ooov[n,m,i,e];  <mb||ej> = -vovo[b,m,e,j];
<mb||ef> = -vovv[b,m,e,f];  <mn||ej> = -ooov[m,n,j,e];
<mb||ij> = -vooo[b,m,i,j].
"""
import functools

import numpy

# Kelvin uses pyscf.lib.einsum, which hands pairwise contractions to BLAS;
# numpy's einsum does the same with optimize=True.
einsum = functools.partial(numpy.einsum, optimize=True)


def _tau(t1, t2, half):
    """tau (half=1) or tau-tilde (half=0.5) = t2 + half*P(ab)(t1 t1)."""
    tt = einsum('ai,bj->abij', t1, t1)
    return t2 + half * (tt - tt.transpose(1, 0, 2, 3))


def intermediates(F, I, t1, t2):
    """F_ae, F_mi, F_me, W_mnij, W_abef, W_mbej of Stanton et al. (1991)."""
    ttau = _tau(t1, t2, 0.5)
    tau = _tau(t1, t2, 1.0)

    Fae = F.vv.copy()
    Fae -= 0.5 * einsum('me,am->ae', F.ov, t1)
    Fae -= einsum('fm,amfe->ae', t1, I.vovv)
    Fae -= 0.5 * einsum('afmn,mnef->ae', ttau, I.oovv)

    Fmi = F.oo.copy()
    Fmi += 0.5 * einsum('ei,me->mi', t1, F.ov)
    Fmi += einsum('en,mnie->mi', t1, I.ooov)
    Fmi += 0.5 * einsum('efin,mnef->mi', ttau, I.oovv)

    Fme = F.ov.copy()
    Fme += einsum('fn,mnef->me', t1, I.oovv)

    Wmnij = I.oooo.copy()
    x = einsum('ej,mnie->mnij', t1, I.ooov)
    Wmnij += x - x.transpose(0, 1, 3, 2)
    Wmnij += 0.25 * einsum('efij,mnef->mnij', tau, I.oovv)

    Wabef = I.vvvv.copy()
    x = einsum('bm,amef->abef', t1, I.vovv)
    Wabef -= x - x.transpose(1, 0, 2, 3)
    Wabef += 0.25 * einsum('abmn,mnef->abef', tau, I.oovv)

    Wmbej = -I.vovo.transpose(1, 0, 2, 3).copy()            # <mb||ej>
    Wmbej -= einsum('fj,bmef->mbej', t1, I.vovv)
    Wmbej += einsum('bn,mnje->mbej', t1, I.ooov)
    tmp = 0.5 * t2 + einsum('fj,bn->fbjn', t1, t1)
    Wmbej -= einsum('fbjn,mnef->mbej', tmp, I.oovv)
    return Fae, Fmi, Fme, Wmnij, Wabef, Wmbej, tau


def residual(F, I, t1, t2):
    """R1[a,i], R2[a,b,i,j]: CCSD residual minus the driving terms."""
    Fae, Fmi, Fme, Wmnij, Wabef, Wmbej, tau = intermediates(F, I, t1, t2)

    R1 = einsum('ae,ei->ai', Fae, t1)
    R1 -= einsum('am,mi->ai', t1, Fmi)
    R1 += einsum('aeim,me->ai', t2, Fme)
    R1 -= einsum('fn,anfi->ai', t1, I.vovo)
    R1 += 0.5 * einsum('efim,amef->ai', t2, I.vovv)
    R1 += 0.5 * einsum('aemn,nmie->ai', t2, I.ooov)

    Xbe = Fae - 0.5 * einsum('bm,me->be', t1, Fme)
    x = einsum('aeij,be->abij', t2, Xbe)
    R2 = x - x.transpose(1, 0, 2, 3)
    Xmj = Fmi + 0.5 * einsum('ej,me->mj', t1, Fme)
    x = einsum('abim,mj->abij', t2, Xmj)
    R2 -= x - x.transpose(0, 1, 3, 2)
    R2 += 0.5 * einsum('abmn,mnij->abij', tau, Wmnij)
    R2 += 0.5 * einsum('efij,abef->abij', tau, Wabef)
    x = einsum('aeim,mbej->abij', t2, Wmbej)
    # - t_i^e t_m^a <mb||ej> = + t1[e,i] t1[a,m] vovo[b,m,e,j]
    x += einsum('ei,am,bmej->abij', t1, t1, I.vovo, optimize=True)
    R2 += x - x.transpose(1, 0, 2, 3) - x.transpose(0, 1, 3, 2) \
        + x.transpose(1, 0, 3, 2)
    x = einsum('ei,abej->abij', t1, I.vvvo)
    R2 += x - x.transpose(0, 1, 3, 2)
    x = einsum('am,bmij->abij', t1, I.vooo)
    R2 += x - x.transpose(1, 0, 2, 3)
    return R1, R2


def stanton(T1, T2, F, I, t1, t2, fac=1.0):
    """In-place T1 += fac*R1, T2 += fac*R2 (cqcpy _Stanton contract)."""
    R1, R2 = residual(F, I, t1, t2)
    T1 += fac * R1
    T2 += fac * R2
