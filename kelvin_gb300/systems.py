"""Model systems for the FT-CCSD engine (input generators).

Each class offers the part of Kelvin's ``System`` interface (kelvin/system.py)
that the finite-temperature general-spin path consumes: ``verify``,
``has_u``, ``g_energies_tot``, ``g_fock_tot``, ``g_aint_tot``, ``get_mp1``,
``const_energy``.  The builders are vectorised numpy (Kelvin's are 4-deep
Python loops, kelvin/ueg_utils.py:109-138) and give the same tensors.

* ``UEGSystem``  -- uniform electron gas in plane waves (kelvin/ueg_system.py),
  optionally with Kelvin's UEGSCFSystem HF exchange shift of the orbital
  energies (kelvin/ueg_scf_system.py:280-297);
* ``HubbardRing`` -- the 1D Hubbard ring in its momentum basis:
  e_k = -2t cos(2 pi k / L), <k1 k2|k3 k4> = (U/L) delta(k1+k2 = k3+k4 mod L)
  between opposite spins, antisymmetrised in spin-orbital form;
* ``ueg_recipe`` / ``hubbard_recipe`` -- the benchmark systems by (N, rs,
  plane waves, Theta) or (sites, t, U, beta).
"""
import numpy


def fermi(beta, e, mu):
    """Occupation 1/(1 + exp(beta (e - mu))), overflow-free."""
    x = beta * (numpy.asarray(e, dtype=float) - mu)
    ex = numpy.exp(-numpy.abs(x))
    return numpy.where(x > 0, ex / (1.0 + ex), 1.0 / (1.0 + ex))


def grand_potential0(beta, e, mu):
    """sum_p -(1/beta) ln(1 + exp(-beta (e_p - mu)))."""
    x = -beta * (numpy.asarray(e, dtype=float) - mu)
    return float(numpy.sum(-(numpy.maximum(x, 0.0) + numpy.log1p(numpy.exp(-numpy.abs(x))))
                           / beta))


def mu_for_filling(beta, e, N, lo=None, hi=None):
    """Chemical potential with sum_p f(e_p) = N (bisection)."""
    e = numpy.asarray(e, dtype=float)
    lo = e.min() - 50.0 / beta - 1.0 if lo is None else lo
    hi = e.max() + 50.0 / beta + 1.0 if hi is None else hi
    for _ in range(200):
        mid = 0.5 * (lo + hi)
        if fermi(beta, e, mid).sum() < N:
            lo = mid
        else:
            hi = mid
    return 0.5 * (lo + hi)


def plane_waves(L, cutoff=None, norb=None):
    """Integer k-vectors sorted by |n|^2 (stable, Kelvin's enumeration order
    i, j, l over [-imax, imax)), truncated to norb (kelvin/ueg_utils.py:31-54)."""
    if cutoff is None:
        # smallest cube holding the norb lowest shells
        m = 1
        while True:
            r = numpy.arange(-m, m)
            g = numpy.stack(numpy.meshgrid(r, r, r, indexing='ij'), -1).reshape(-1, 3)
            n2 = (g * g).sum(1)
            if (n2 <= (m - 1) ** 2).sum() >= (norb or 1):
                break
            m += 1
        sel = g[n2 <= (m - 1) ** 2]
    else:
        kmax = numpy.sqrt(2 * cutoff)
        imax = int(numpy.ceil(L * kmax / (2 * numpy.pi)) + 0.1)
        r = numpy.arange(-imax, imax)
        g = numpy.stack(numpy.meshgrid(r, r, r, indexing='ij'), -1).reshape(-1, 3)
        k2 = 4.0 * numpy.pi ** 2 / (L * L) * (g * g).sum(1)
        sel = g[k2 < 2.0 * cutoff]
    order = numpy.argsort((sel * sel).sum(1), kind='stable')
    sel = sel[order]
    if norb is not None:
        sel = sel[:norb]
    return sel


class UEGSystem(object):
    """Spin-orbital uniform electron gas ('g' ordering: alpha block, beta block).

    ``hf_shift=True`` adds the exchange shift of the ``nref`` lowest plane
    waves (closed-shell T = 0 reference), as Kelvin's UEGSCFSystem does with
    its occupied set (ueg_scf_system.py:53-78, 280-289).

    ``device_build=True``: the n^4 integrals are written on the GPU by
    ``device_aint_tot`` (kvft_ueg_eri) and the Fock matrix, the first-order
    energy and the exchange shift use their closed forms -- by momentum
    conservation the direct terms vanish and each is a sum over pairs of
    plane waves -- so no n^4 array exists on the host.
    """

    def __init__(self, T, L, cutoff=None, mu=None, norb=None, hf_shift=False,
                 nref=None, N=None, device_build=False):
        self.T = T
        self.L = L
        self.nvec = plane_waves(L, cutoff, norb)
        nb = self.nvec.shape[0]
        self.nb = nb
        c = 2.0 * numpy.pi / L
        self.kvec = c * self.nvec
        self.ekin = 0.5 * (self.kvec ** 2).sum(1)
        self.pref = 4.0 * numpy.pi / L ** 3
        self.hf_shift = hf_shift
        self.device_build = device_build
        e = self.ekin.copy()
        if hf_shift:
            if nref is None:
                if mu is None:
                    raise Exception("hf_shift needs nref or mu")
                occ = numpy.nonzero(self.ekin < mu)[0]
            else:
                occ = numpy.arange(nref)
            if device_build:
                # <pi|pi> = 0 (q = 0 excluded), <pi|ip> = v(n_p - n_i)
                e = e - self._vq()[:, occ].sum(1)
            else:
                V = self._spatial()
                e = e + 2 * numpy.einsum('pipi->p', V[:, occ][:, :, :, occ]) \
                    - numpy.einsum('piip->p', V[:, occ][:, :, occ, :])
        self.e_spatial = e
        beta = 1.0 / T
        if mu is None:
            if N is None:
                raise Exception("give mu or N")
            # mean-field (non-interacting) filling with the energies in use
            mu = mu_for_filling(beta, numpy.hstack((e, e)), N)
        self.mu = mu
        self.N = float(fermi(beta, self.g_energies_tot(), mu).sum())
        self._eri = None

    def _coulomb_const(self):
        """c of <pq|rs> = c / |n_p - n_r|^2, evaluated as in ``_spatial``."""
        return self.pref * (2 * numpy.pi / self.L) ** -2

    def _vq(self):
        """v[p, r] = c / |n_p - n_r|^2 (0 for p = r): the nb x nb exchange kernel."""
        n = self.nvec
        dq = n[:, None, :] - n[None, :, :]
        q2 = (dq * dq).sum(-1).astype(float)
        with numpy.errstate(divide='ignore'):
            return numpy.where(q2 > 0, self._coulomb_const() / q2, 0.0)

    def device_aint_tot(self, ctx):
        """g_aint_tot() written on the device: a DeviceArray (n, n, n, n)."""
        from . import _lib
        n = 2 * self.nb
        out = _lib.DeviceArray(ctx, (n, n, n, n))
        nv = numpy.ascontiguousarray(self.nvec, dtype=numpy.int32)
        ctx.check(ctx.L.kvft_ueg_eri(ctx.h, self.nb, nv.ctypes.data_as(_lib.vp),
                                     float(self._coulomb_const()), out.ptr), "kvft_ueg_eri")
        return out

    def _spatial(self):
        """<pq|rs> = pref/|k_p-k_r|^2 if n_p+n_q = n_r+n_s, p != r, q != s."""
        n = self.nvec
        nb = self.nb
        dq = n[:, None, :] - n[None, :, :]                    # n_p - n_r  [p, r]
        q2 = (dq * dq).sum(-1).astype(float)
        with numpy.errstate(divide='ignore'):
            vq = numpy.where(q2 > 0, self.pref * (2 * numpy.pi / self.L) ** -2 / q2, 0.0)
        # momentum conservation: n_p - n_r == n_s - n_q
        cons = numpy.all(dq[:, None, :, None, :] == -dq[None, :, None, :, :], axis=-1)
        V = numpy.where(cons, vq[:, None, :, None], 0.0)         # [p, q, r, s]
        idx = numpy.arange(nb)
        qs = (idx[:, None] == idx[None, :])                      # q == s
        V = V * (~qs)[None, :, None, :]
        return V

    # --- Kelvin System interface (general spin) ---------------------------
    def has_u(self):
        return False

    def has_g(self):
        return True

    def verify(self, T, mu):
        return T == self.T and mu == self.mu

    def const_energy(self):
        return 0.0

    def g_energies_tot(self):
        return numpy.hstack((self.e_spatial, self.e_spatial))

    def g_aint_tot(self):
        if self._eri is None:
            V = self._spatial()
            nb = self.nb
            n = 2 * nb
            g = numpy.zeros((n, n, n, n))
            for s1 in (0, 1):
                for s2 in (0, 1):
                    g[s1 * nb:(s1 + 1) * nb, s2 * nb:(s2 + 1) * nb,
                      s1 * nb:(s1 + 1) * nb, s2 * nb:(s2 + 1) * nb] = V
            g -= g.transpose(0, 1, 3, 2)
            self._eri = g
        return self._eri

    def g_fock_tot(self):
        beta = 1.0 / self.T
        fo = fermi(beta, self.g_energies_tot(), self.mu)
        kin = numpy.hstack((self.ekin, self.ekin))
        if self.device_build:
            # F_pq = delta_pq (k_p^2/2 - sum_{r, same spin} v(n_p - n_r) f_r)
            v = self._vq()
            nb = self.nb
            x = numpy.hstack((v @ fo[:nb], v @ fo[nb:]))
            return numpy.diag(kin - x)
        return numpy.diag(kin) + numpy.einsum('prqr,r->pq', self.g_aint_tot(), fo)

    def get_mp1(self):
        """First-order grand potential sum_i (h_ii - e_i) f_i +
        1/2 sum_ij <ij||ij> f_i f_j, h the kinetic energy (ueg_scf_system.py:
        146-157; the first sum is the exchange shift's and vanishes without
        it)."""
        en = self.g_energies_tot()
        fo = fermi(1.0 / self.T, en, self.mu)
        e1 = (numpy.hstack((self.ekin, self.ekin)) - en) @ fo
        if self.device_build:
            # 1/2 sum_ij <ij||ij> f_i f_j = -1/2 sum_{ij, same spin} v(n_i - n_j) f_i f_j
            v = self._vq()
            nb = self.nb
            return e1 - 0.5 * (fo[:nb] @ v @ fo[:nb] + fo[nb:] @ v @ fo[nb:])
        return e1 + 0.5 * numpy.einsum('ijij,i,j->', self.g_aint_tot(), fo, fo)


class HubbardRing(object):
    """1D Hubbard ring in the momentum basis (spin orbitals: alpha k, beta k).

    ``device_build=True``: integrals written on the GPU (kvft_hubbard_eri);
    Fock matrix and first-order energy from their closed forms (the on-site
    U couples opposite spins only: F_pp = e_p + (U/L) N_other spin,
    E1 = (U/L) N_alpha N_beta)."""

    def __init__(self, T, sites, t=1.0, U=4.0, mu=0.0, device_build=False, shift=0.0):
        self.T = T
        self.device_build = device_build
        self.L = sites
        self.t = t
        self.U = U
        self.mu = mu
        # orbital energies e_k = eps_k + shift: shift = U n with n the
        # reference density per site and spin gives the mean-field orbitals
        # of Kelvin's HubbardSystem (hubbard_system.py:48-73), 0 the bare band
        self.shift = float(shift)
        k = numpy.arange(sites)
        self.ek = -2.0 * t * numpy.cos(2.0 * numpy.pi * k / sites)
        self._eri = None
        self.N = float(fermi(1.0 / T, self.g_energies_tot(), mu).sum())

    def has_u(self):
        return False

    def has_g(self):
        return True

    def verify(self, T, mu):
        return T == self.T and mu == self.mu

    def const_energy(self):
        return 0.0

    def g_energies_tot(self):
        return numpy.hstack((self.ek, self.ek)) + self.shift

    def g_aint_tot(self):
        if self._eri is None:
            L = self.L
            k = numpy.arange(L)
            cons = ((k[:, None, None, None] + k[None, :, None, None]
                     - k[None, None, :, None] - k[None, None, None, :]) % L) == 0
            Vk = numpy.where(cons, self.U / L, 0.0)
            n = 2 * L
            V = numpy.zeros((n, n, n, n))
            V[:L, L:, :L, L:] = Vk          # <k1 a, k2 b | k3 a, k4 b>
            V[L:, :L, L:, :L] = Vk          # <k1 b, k2 a | k3 b, k4 a>
            self._eri = V - V.transpose(0, 1, 3, 2)
        return self._eri

    def device_aint_tot(self, ctx):
        """g_aint_tot() written on the device: a DeviceArray (n, n, n, n)."""
        from . import _lib
        n = 2 * self.L
        out = _lib.DeviceArray(ctx, (n, n, n, n))
        ctx.check(ctx.L.kvft_hubbard_eri(ctx.h, self.L, float(self.U / self.L), out.ptr),
                  "kvft_hubbard_eri")
        return out

    def g_fock_tot(self):
        fo = fermi(1.0 / self.T, self.g_energies_tot(), self.mu)
        if self.device_build:
            L = self.L
            na, nb = fo[:L].sum(), fo[L:].sum()
            return numpy.diag(numpy.hstack((self.ek, self.ek)) + (self.U / L) *
                              numpy.hstack((numpy.full(L, nb), numpy.full(L, na))))
        h = numpy.diag(numpy.hstack((self.ek, self.ek)))
        return h + numpy.einsum('prqr,r->pq', self.g_aint_tot(), fo)

    def get_mp1(self):
        """sum_i (h_ii - e_i) f_i + 1/2 f W f (the first-order grand potential
        of Kelvin's HubbardSystem.get_mp1, hubbard_system.py:120-133)."""
        fo = fermi(1.0 / self.T, self.g_energies_tot(), self.mu)
        if self.device_build:
            L = self.L
            return (self.U / L) * fo[:L].sum() * fo[L:].sum() - self.shift * fo.sum()
        return (0.5 * numpy.einsum('ijij,i,j->', self.g_aint_tot(), fo, fo)
                - self.shift * fo.sum())


def ueg_recipe(N, rs, norb, theta, hf_shift=True, device_build=False):
    """UEG of N electrons at Wigner-Seitz radius rs in a cubic box
    L = (4 pi N / 3)^(1/3) rs, the norb lowest plane waves, T = theta T_F with
    T_F = k_F^2 / 2, k_F = (9 pi / 4)^(1/3) / rs, mu from non-interacting
    Fermi-Dirac filling to N electrons, closed-shell HF exchange shift."""
    L = (4.0 * numpy.pi * N / 3.0) ** (1.0 / 3.0) * rs
    kF = (9.0 * numpy.pi / 4.0) ** (1.0 / 3.0) / rs
    T = theta * 0.5 * kF * kF
    return UEGSystem(T, L, norb=norb, N=N, hf_shift=hf_shift, nref=int(round(N)) // 2,
                     device_build=device_build)


def hubbard_recipe(sites, t, U, beta, device_build=False):
    """Half-filled Hubbard ring at inverse temperature beta (mu = 0)."""
    return HubbardRing(1.0 / beta, sites, t=t, U=U, mu=0.0, device_build=device_build)


def hubbard_mf_recipe(sites, t, U, beta, device_build=False):
    """Half-filled Hubbard ring in the mean-field momentum basis of Kelvin's
    HubbardSystem: the uniform reference density 1/2 per site and spin gives
    e_k = -2t cos(2 pi k / sites) + U/2, and mu = U/2 fills half the band at
    every temperature (the band is symmetric about U/2, so the Fock matrix
    equals diag(e) and F - diag(e) vanishes)."""
    return HubbardRing(1.0 / beta, sites, t=t, U=U, mu=0.5 * U, device_build=device_build,
                       shift=0.5 * U)
