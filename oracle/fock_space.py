"""Exact CC residual from second-quantised operators (oracle; test infrastructure).

An independent check of the restated Stanton-Gauss residual: for no occupied
and nv virtual spin orbitals (no + nv <= 10) the Fock space is small, so

    R_mu = <Phi_mu| exp(-T) H exp(T) |Phi_0>

is evaluated by applying Jordan-Wigner fermion operators to state vectors.
H is built from the same blocks the CC code consumes: a Fock operator with
blocks F.oo/F.ov/F.vo/F.vv (normal-ordered with respect to |Phi_0>) and an
antisymmetrised two-electron operator assembled from the nine blocks.  H need
not be Hermitian; the CC residual is a polynomial identity in the blocks.
"""
import itertools
import numpy


class _Space(object):
    def __init__(self, nso):
        self.n = nso
        self.dim = 1 << nso
        b = numpy.arange(self.dim)
        self.ann = []
        self.cre = []
        for p in range(nso):
            occ = (b >> p) & 1
            below = numpy.array([bin(x & ((1 << p) - 1)).count("1") for x in b])
            sign = numpy.where(below % 2 == 0, 1.0, -1.0)
            src = numpy.nonzero(occ)[0]
            self.ann.append((src, src ^ (1 << p), sign[src]))
            src = numpy.nonzero(occ == 0)[0]
            self.cre.append((src, src | (1 << p), sign[src]))

    @staticmethod
    def _apply(op, v):
        src, dst, sgn = op
        out = numpy.zeros_like(v)
        out[dst] = sgn * v[src]
        return out

    def a(self, p, v):
        return self._apply(self.ann[p], v)

    def ad(self, p, v):
        return self._apply(self.cre[p], v)


def _full_tensors(F, I, no, nv):
    """Full f[p,q] and antisymmetric g[p,q,r,s] over o (0..no-1), v (no..)."""
    n = no + nv
    o = slice(0, no)
    v = slice(no, n)
    f = numpy.zeros((n, n))
    f[o, o] = F.oo
    f[o, v] = F.ov
    f[v, o] = F.vo
    f[v, v] = F.vv
    g = numpy.zeros((n, n, n, n))
    blocks = {
        (v, v, v, v): I.vvvv, (v, v, v, o): I.vvvo, (v, o, v, v): I.vovv,
        (v, v, o, o): I.vvoo, (v, o, v, o): I.vovo, (o, o, v, v): I.oovv,
        (v, o, o, o): I.vooo, (o, o, o, v): I.ooov, (o, o, o, o): I.oooo,
    }
    for (p, q, r, s), blk in blocks.items():
        # the four index orderings related by antisymmetry of each pair
        g[p, q, r, s] = blk
        g[q, p, r, s] = -blk.transpose(1, 0, 2, 3)
        g[p, q, s, r] = -blk.transpose(0, 1, 3, 2)
        g[q, p, s, r] = blk.transpose(1, 0, 3, 2)
    return f, g


def exact_residual(F, I, t1, t2):
    """Return (R1[a,i], R2[a,b,i,j]) = projections of exp(-T) H exp(T)|0>,
    including the driving terms F.vo and I.vvoo."""
    nv, no = t1.shape
    n = no + nv
    sp = _Space(n)
    f, g = _full_tensors(F, I, no, nv)
    occ = range(no)
    vir = range(no, n)
    # normal-ordered H = sum f {p+q} + 1/4 sum g {p+q+ s r}; the reference
    # energy shift does not touch excited projections, so use the one-body
    # part h = f - sum_i g[p,i,q,i] with plain (non-normal-ordered) products.
    h = f - numpy.einsum('piqi->pq', g[:, :no, :, :no])

    ref = numpy.zeros(sp.dim)
    ref[(1 << no) - 1] = 1.0

    def apply_T(v, sign):
        out = numpy.zeros_like(v)
        for a, i in itertools.product(vir, occ):
            c = t1[a - no, i]
            if c != 0.0:
                out += sign * c * sp.ad(a, sp.a(i, v))
        for i, j in itertools.combinations(occ, 2):
            w = sp.a(j, sp.a(i, v))
            if not w.any():
                continue
            for a, b in itertools.combinations(vir, 2):
                c = t2[a - no, b - no, i, j]
                if c != 0.0:
                    out += sign * c * sp.ad(a, sp.ad(b, w))
        return out

    def exp_T(v, sign):
        out = v.copy()
        term = v.copy()
        for k in range(1, n + 2):
            term = apply_T(term, sign) / k
            if not term.any():
                break
            out += term
        return out

    def apply_H(v):
        out = numpy.zeros_like(v)
        for p, q in itertools.product(range(n), repeat=2):
            if h[p, q] != 0.0:
                out += h[p, q] * sp.ad(p, sp.a(q, v))
        for r, s in itertools.product(range(n), repeat=2):
            w = sp.a(s, sp.a(r, v))
            if not w.any():
                continue
            for p, q in itertools.product(range(n), repeat=2):
                c = g[p, q, r, s]
                if c != 0.0:
                    out += 0.25 * c * sp.ad(p, sp.ad(q, w))
        return out

    hbar = exp_T(apply_H(exp_T(ref, 1.0)), -1.0)

    R1 = numpy.zeros((nv, no))
    for a, i in itertools.product(vir, occ):
        R1[a - no, i] = sp.ad(a, sp.a(i, ref)) @ hbar
    R2 = numpy.zeros((nv, nv, no, no))
    for a, b, i, j in itertools.product(vir, vir, occ, occ):
        if a != b and i != j:
            R2[a - no, b - no, i, j] = sp.ad(a, sp.ad(b, sp.a(j, sp.a(i, ref)))) @ hbar
    return R1, R2


def grand_potential(h, eri, T, mu):
    """Exact grand potential -T ln Tr exp(-(H - mu N)/T) for
    H = sum h[p,q] a+_p a_q + 1/4 sum <pq||rs> a+_p a+_q a_s a_r over n <= 10
    spin orbitals, by diagonalising H - mu N in the 2^n-dimensional Fock space
    (the finite-temperature FCI of kelvin/fci.py:88-103)."""
    n = h.shape[0]
    sp = _Space(n)
    dim = sp.dim
    H = numpy.zeros((dim, dim))
    for col in range(dim):
        v = numpy.zeros(dim)
        v[col] = 1.0
        out = numpy.zeros(dim)
        for p in range(n):
            for q in range(n):
                if h[p, q] != 0.0:
                    out += h[p, q] * sp.ad(p, sp.a(q, v))
        for p, q, r, s in itertools.product(range(n), repeat=4):
            if eri[p, q, r, s] != 0.0:
                out += 0.25 * eri[p, q, r, s] * sp.ad(p, sp.ad(q, sp.a(s, sp.a(r, v))))
        H[:, col] = out
    N = numpy.array([bin(x).count("1") for x in range(dim)], dtype=float)
    w = numpy.linalg.eigvalsh(0.5 * (H + H.T) - mu * numpy.diag(N))
    w0 = w.min()
    return w0 - T * numpy.log(numpy.exp(-(w - w0) / T).sum())
