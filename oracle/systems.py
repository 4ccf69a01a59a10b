"""Model systems feeding the FT-CCSD path (oracle; test infrastructure).

Loop-based restatements of Kelvin's uniform-electron-gas builders, kept
close to the reference's own control flow so that the vectorised product
builders can be checked against them at small n:

* ``UEGBasis``          -- kelvin/ueg_utils.py:21-54 (k-cube, stable sort by
                           |n|^2, truncation to norb);
* ``g2e_loop``          -- kelvin/ueg_utils.py:109-138 (antisymmetrised,
                           momentum-conserving Coulomb, q = 0 dropped);
* ``ueg_g_energies`` / ``ueg_g_fock`` -- kelvin/ueg_system.py:266-267,400-419;
* ``uegscf_g_energies`` / fock         -- kelvin/ueg_scf_system.py:280-297,398-417;
* ``get_mp1``           -- kelvin/ueg_system.py:126-131 (general spin, T > 0).
"""
import numpy

from . import ft_utils


class UEGBasis(object):
    """Plane waves below an energy cutoff (ueg_utils.py:21-54)."""

    def __init__(self, L, cutoff, norb=None):
        self.L = L
        kmax = numpy.sqrt(2 * cutoff)
        imax = int(numpy.ceil(L * kmax / (2 * numpy.pi)) + 0.1)
        basis = []
        for i in range(-imax, imax):
            for j in range(-imax, imax):
                for l in range(-imax, imax):
                    k2 = 4.0 * numpy.pi * numpy.pi / (L * L) * (i * i + j * j + l * l)
                    if k2 < 2.0 * cutoff:
                        basis.append((i, j, l))
        basis.sort(key=lambda x: x[0] * x[0] + x[1] * x[1] + x[2] * x[2])
        if norb is not None:
            basis = basis[:norb]
        self.basis = basis
        c = 2.0 * numpy.pi / L
        self.ks = [numpy.array((c * x[0], c * x[1], c * x[2])) for x in basis]
        self.Es = [0.5 * float(k @ k) for k in self.ks]


def g2e_loop(basis, anti=True):
    """Spin-orbital Coulomb integrals by the reference's 4-deep loop."""
    nb = len(basis.ks)
    n = 2 * nb
    V = numpy.zeros((n, n, n, n))
    pref = 4.0 * numpy.pi / basis.L ** 3
    for p in range(n):
        kp = basis.ks[p % nb]
        for q in range(n):
            kq = basis.ks[q % nb]
            for r in range(n):
                kr = basis.ks[r % nb]
                for s in range(n):
                    ks = basis.ks[s % nb]
                    if p == r or q == s:
                        continue
                    if p // nb != r // nb or q // nb != s // nb:
                        continue
                    if numpy.linalg.norm(kp + kq - kr - ks) < 1e-12:
                        d = kp - kr
                        V[p, q, r, s] = pref / float(d @ d)
    if anti:
        return V - V.transpose(0, 1, 3, 2)
    return V


def ueg_g_energies(basis):
    """Bare k^2/2 spin-orbital energies (ueg_system.py:266-267)."""
    e = numpy.asarray(basis.Es)
    return numpy.hstack((e, e))


def uegscf_g_energies(basis, mu):
    """HF-shifted energies e_p = k^2/2 + sum_{i occ at T=0}(2J - K)
    (ueg_scf_system.py:280-297); occupied = plane waves with k^2/2 < mu."""
    e0 = numpy.asarray(basis.Es)
    nb = e0.shape[0]
    Vg = g2e_loop(basis, anti=False)
    V = Vg[:nb, :nb, :nb, :nb]       # spatial <pq|rs>, same-spin block
    oidx = [p for p in range(nb) if e0[p] < mu]
    e = e0.copy()
    for i in oidx:
        e += 2 * V[:, i, :, i].diagonal() - V[:, i, i, :].diagonal()
    return numpy.hstack((e, e))


def g_fock_tot(basis, eri, en, T, mu):
    """FT Fock matrix T + JK[f] over the given energies (ueg_system.py:400-419)."""
    kin = numpy.asarray(basis.Es)
    tmat = numpy.diag(numpy.hstack((kin, kin)))
    fo = ft_utils.ff(1.0 / T, en, mu)
    return tmat + numpy.einsum('prqr,r->pq', eri, fo)


def get_mp1(eri, en, T, mu):
    """First-order grand potential 1/2 sum_ij <ij||ij> f_i f_j (ueg_system.py:126-131)."""
    fo = ft_utils.ff(1.0 / T, en, mu)
    return 0.5 * numpy.einsum('ijij,i,j->', eri, fo, fo)
