"""The device Lambda terms (kvft_lambda_residual) and the device Lambda
update (kvft_ccsd_lambda), checked on the CPU.

A dry-run context records every launch the call makes -- the strided GEMM
and strided axpby descriptors, over host buffers and NaN-filled host scratch
-- without a GPU.  These tests replay the recorded launches in numpy with
the kernels' documented semantics, check that every access stays inside its
buffer, and compare the result with the oracle's reverse pass and Lambda
update (oracle/ft_lambda.residual_vjp, lambda_update).  What is left for the GPU is the kernels
themselves, which the GPU tests check separately (test_gpu_tc.py,
test_gpu_kernels.py)."""
import ctypes

import numpy
import pytest

from conftest import random_system
from kelvin_gb300 import _lib
from oracle import ft_lambda

F_ORDER = ("oo", "ov", "vo", "vv")
I_ORDER = ("vvvv", "vvvo", "vovv", "vvoo", "vovo", "oovv", "vooo", "ooov", "oooo")


def _L():
    return _lib.lib()


def _offsets(sizes, strides):
    s, t = sizes, strides
    return (numpy.arange(s[0])[:, None, None] * t[0] + numpy.arange(s[1])[None, :, None] * t[1]
            + numpy.arange(s[2])[None, None, :] * t[2]).reshape(-1)


def _plan(nv, no, a, b, c):
    mnk = (ctypes.c_int * 3)()
    sizes = (ctypes.c_int * 18)()
    strides = (ctypes.c_longlong * 18)()
    st = _L().kvft_einsum_plan(nv, no, a.encode(), b.encode(), c.encode(), mnk, sizes, strides)
    assert st == 0, (a, b, c)
    views = [(list(sizes[3 * k:3 * k + 3]), list(strides[3 * k:3 * k + 3])) for k in range(6)]
    return list(mnk), views


SPECS = [("abij,bmij", "am"), ("ia,me", "aeim"), ("ai,bj", "abij"), ("bi,aj", "abij"),
         ("me,am", "ae"), ("fm,amfe", "ae"), ("ej,mnie", "mnji"), ("abij,am", "bijm"),
         ("ijab,abef", "efij"), ("mbej,mnef", "fbjn"), ("ia,nmie", "aemn"),
         ("abef,mnef", "abmn"), ("fbjn,fj", "bn"), ("mi,mnef", "efin")]


@pytest.mark.parametrize("ab,c", SPECS)
def test_einsum_plan_is_the_contraction(ab, c):
    """The strided-GEMM form of each index-string contraction reproduces
    numpy.einsum (nv != no, so a virtual/occupied mix-up shows)."""
    nv, no = 4, 3
    a, b = ab.split(",")
    ext = lambda s: tuple(nv if ch in "abcdefgh" else no for ch in s)
    rng = numpy.random.default_rng(len(a) * 7 + len(c))
    A = rng.standard_normal(ext(a))
    B = rng.standard_normal(ext(b))
    (M, N, K), v = _plan(nv, no, a, b, c)
    ar, ac, br, bc, cr, cc = [_offsets(*x) for x in v]
    assert (len(ar), len(ac), len(bc)) == (M, K, N)
    Am = A.reshape(-1)[ar[:, None] + ac[None, :]]
    Bm = B.reshape(-1)[br[:, None] + bc[None, :]]
    C = numpy.full(int(numpy.prod(ext(c))), numpy.nan)
    idx = cr[:, None] + cc[None, :]
    assert len(numpy.unique(idx)) == C.size            # every element written once
    C[idx] = Am @ Bm
    ref = numpy.einsum("%s,%s->%s" % (a, b, c), A, B)
    assert abs(C.reshape(ref.shape) - ref).max() < 1e-13


def test_einsum_plan_rejects_bad_strings():
    mnk = (ctypes.c_int * 3)()
    sizes = (ctypes.c_int * 18)()
    strides = (ctypes.c_longlong * 18)()
    for a, b, c in (("abij", "bj", "abij"), ("ai", "bj", "ab"), ("az", "zb", "ab"),
                    ("aai", "ai", "ai")):
        assert _L().kvft_einsum_plan(3, 2, a.encode(), b.encode(), c.encode(), mnk, sizes,
                                     strides) != 0


class _Memory(object):
    """Host buffers the recorded launches address, by base pointer."""

    def __init__(self):
        self.bufs = []

    def add(self, arr):
        flat = arr.reshape(-1)
        assert flat.base is arr or flat is arr or numpy.shares_memory(flat, arr)
        self.bufs.append((arr.ctypes.data, flat.size, flat))

    def add_raw(self, ptr, nbytes):
        n = nbytes // 8
        flat = numpy.ctypeslib.as_array((ctypes.c_double * n).from_address(ptr))
        self.bufs.append((ptr, n, flat))

    def find(self, ptr):
        for base, n, flat in self.bufs:
            if base <= ptr < base + 8 * n:
                assert (ptr - base) % 8 == 0
                return flat, (ptr - base) // 8
        raise AssertionError("pointer outside every buffer")

    def view(self, ptr, offs):
        flat, start = self.find(ptr)
        idx = start + offs
        assert idx.min() >= 0 and idx.max() < flat.size, "access out of bounds"
        return flat, idx


def _replay(ctx, mem, sums=None):
    L = _L()
    n = ctypes.c_int()
    assert L.kvft_dryrun_count(ctx, ctypes.byref(n)) == 0
    ints = (ctypes.c_int * 32)()
    longs = (ctypes.c_longlong * 32)()
    dbls = (ctypes.c_double * 2)()
    ptrs = (ctypes.c_void_p * 11)()
    kinds = []
    for i in range(n.value):
        assert L.kvft_dryrun_op(ctx, i, ints, longs, dbls, ptrs) == 0
        kind, M, N, K, batch = ints[0:5]
        alpha, beta = dbls[0], dbls[1]
        kinds.append(kind)
        if kind == 0:
            v = [_offsets(ints[5 + 3 * k:8 + 3 * k], longs[3 * k:3 * k + 3]) for k in range(6)]
            ar, ac, br, bc, cr, cc = v
            assert (len(ar), len(ac), len(br), len(bc), len(cr), len(cc)) == (M, K, K, N, M, N)
            assert not (M == 1 and N > 1)       # single rows go as transposed products
            abst, bbst, cbst = longs[18], longs[19], longs[20]
            for b in range(batch):
                fa, ia = mem.view(ptrs[0] + 8 * b * abst, ar[:, None] + ac[None, :])
                fb, ib = mem.view(ptrs[1] + 8 * b * bbst, br[:, None] + bc[None, :])
                fc, ic = mem.view(ptrs[2] + 8 * b * cbst, cr[:, None] + cc[None, :])
                prod = alpha * (fa[ia] @ fb[ib])
                fc[ic] = prod if beta == 0.0 else prod + beta * fc[ic]
        elif kind == 1:
            dims = ints[23:27]
            ss, ds = longs[21:25], longs[25:29]
            sbst, dbst = longs[29], longs[30]
            grid = numpy.indices(dims).reshape(4, -1)
            so = sum(grid[k] * ss[k] for k in range(4))
            do = sum(grid[k] * ds[k] for k in range(4))
            for b in range(batch):
                fs, is_ = mem.view(ptrs[3] + 8 * b * sbst, so)
                fd, id_ = mem.view(ptrs[4] + 8 * b * dbst, do)
                val = alpha * fs[is_]
                fd[id_] = val if beta == 0.0 else val + beta * fd[id_]
        elif kind == 2:
            ng, rank, full, nv, no = ints[27:32]
            P = longs[31]
            ft, it = mem.view(ptrs[5], numpy.arange(ng))
            ti = ft[it]
            fg, ig = mem.view(ptrs[6], numpy.arange(ng * ng))
            G = fg[ig].reshape(ng, ng)
            fev, iev = mem.view(ptrs[7], numpy.arange(nv))
            feo, ieo = mem.view(ptrs[8], numpy.arange(no))
            ev, eo = fev[iev], feo[ieo]
            if rank == 1:
                d = (ev[:, None] - eo[None, :]).reshape(-1)
            else:
                d = (ev[:, None, None, None] + ev[None, :, None, None]
                     - eo[None, None, :, None] - eo[None, None, None, :]).reshape(-1)
            assert d.size == P
            fs, is_ = mem.view(ptrs[3], numpy.arange(ng * P))
            tb = fs[is_].reshape(ng, P)
            out = numpy.zeros((ng, P))
            for y in range(ng):
                for x in range(ng):
                    w = numpy.exp((ti[x] - ti[y]) * d) if (x <= y or full) else 1.0
                    out[y] += G[y, x] * w * tb[x]
            fo, io = mem.view(ptrs[4], numpy.arange(ng * P))
            fo[io] = out.reshape(-1)
        elif kind == 4:
            dims = ints[23:27]
            xs, ys = longs[21:25], longs[25:29]
            xbst, ybst = longs[29], longs[30]
            grid = numpy.indices(dims).reshape(4, -1)
            xo = sum(grid[k] * xs[k] for k in range(4))
            yo = sum(grid[k] * ys[k] for k in range(4))
            acc = 0.0
            for b in range(batch):
                fx, ix = mem.view(ptrs[3] + 8 * b * xbst, xo)
                val = alpha * fx[ix]
                if ptrs[9]:
                    fy, iy = mem.view(ptrs[9] + 8 * b * ybst, yo)
                    val = val + beta * fy[iy]
                acc += float((val * val).sum())
            fr, ir = mem.view(ptrs[10], numpy.arange(1))
            fr[ir] = acc
            if sums is not None:
                sums.append(acc)
        elif kind == 3:
            cr = _offsets(ints[17:20], longs[12:15])
            cc = _offsets(ints[20:23], longs[15:18])
            for b in range(batch):
                fc, ic = mem.view(ptrs[2] + 8 * b * longs[20], cr[:, None] + cc[None, :])
                fc[ic] = 0.0 if beta == 0.0 else beta * fc[ic]
        else:
            raise AssertionError("unexpected launch kind %d" % kind)
    return kinds


@pytest.mark.parametrize("no,nv,nb,prec", [(3, 4, 2, 0), (4, 3, 1, 2)])
def test_lambda_residual_dry_run_vs_oracle(no, nv, nb, prec):
    rng = numpy.random.default_rng(10 * no + nv)
    F, I = random_system(rng, no, nv)
    anti = lambda x: (x - x.swapaxes(-1, -2)) - (x - x.swapaxes(-1, -2)).swapaxes(-3, -4)
    t1 = rng.standard_normal((nb, nv, no)) * 0.1
    t2 = anti(rng.standard_normal((nb, nv, nv, no, no)) * 0.1)
    m1 = rng.standard_normal((nb, no, nv))
    m2 = anti(rng.standard_normal((nb, no, no, nv, nv)))
    g1 = numpy.full((nb, nv, no), numpy.nan)
    g2 = numpy.full((nb, nv, nv, no, no), numpy.nan)
    Fb = [numpy.ascontiguousarray(getattr(F, k)) for k in F_ORDER]
    Ib = [numpy.ascontiguousarray(getattr(I, k)) for k in I_ORDER]
    L = _L()
    ctx = ctypes.c_void_p()
    assert L.kvft_dryrun_create(prec, 5, ctypes.byref(ctx)) == 0
    try:
        Fp = (ctypes.c_void_p * 4)(*[a.ctypes.data for a in Fb])
        Ip = (ctypes.c_void_p * 9)(*[a.ctypes.data for a in Ib])
        st = L.kvft_lambda_residual(ctx, nb, nv, no, Fp, Ip, t1.ctypes.data, t2.ctypes.data,
                                    m1.ctypes.data, m2.ctypes.data, g1.ctypes.data,
                                    g2.ctypes.data)
        assert st == 0
        assert numpy.isnan(g1).all() and numpy.isnan(g2).all()      # nothing ran
        mem = _Memory()
        for a in Fb + Ib + [t1, t2, m1, m2, g1, g2]:
            mem.add(a)
        i = 0
        ptr, nbytes = ctypes.c_void_p(), ctypes.c_size_t()
        while L.kvft_dryrun_scratch(ctx, i, ctypes.byref(ptr), ctypes.byref(nbytes)) == 0:
            mem.add_raw(ptr.value, nbytes.value)
            i += 1
        assert i >= 1
        kinds = _replay(ctx, mem)
        assert set(kinds) <= {0, 1}
    finally:
        L.kvft_ctx_destroy(ctx)
    for y in range(nb):
        r1, r2 = ft_lambda.residual_vjp(F, I, t1[y], t2[y], m1[y].T,
                                        m2[y].transpose(2, 3, 0, 1))
        assert abs(g1[y] - r1).max() < 1e-12 * max(1.0, abs(r1).max())
        assert abs(g2[y] - r2).max() < 1e-12 * max(1.0, abs(r2).max())


def test_dry_run_context_rejects_device_calls():
    L = _L()
    ctx = ctypes.c_void_p()
    assert L.kvft_dryrun_create(0, 7, ctypes.byref(ctx)) == 0
    try:
        assert L.kvft_sync(ctx) != 0
        assert L.kvft_flush_l2(ctx) != 0
    finally:
        assert L.kvft_ctx_destroy(ctx) == 0


@pytest.mark.parametrize("no,nv,ng", [(3, 4, 4), (3, 3, 5)])
def test_ccsd_lambda_dry_run_vs_oracle(no, nv, ng):
    """kvft_ccsd_lambda (Kelvin's ccsd_lambda_opt: int_L, the Lambda terms,
    the energy terms) replayed against the oracle's lambda_update."""
    from oracle import quadrature
    rng = numpy.random.default_rng(7 * no + nv + ng)
    F, I = random_system(rng, no, nv)
    anti = lambda x: (x - x.swapaxes(-1, -2)) - (x - x.swapaxes(-1, -2)).swapaxes(-3, -4)
    ev = rng.standard_normal(nv) * 0.5 + 1.0
    eo = rng.standard_normal(no) * 0.5 - 1.0
    D1 = ev[:, None] - eo[None, :]
    D2 = (ev[:, None, None, None] + ev[None, :, None, None] - eo[None, None, :, None]
          - eo[None, None, None, :])
    beta = 2.0
    ti, g, G = quadrature.ft_quad(ng, beta, 'lin')
    T1 = rng.standard_normal((ng, nv, no)) * 0.1
    T2 = anti(rng.standard_normal((ng, nv, nv, no, no)) * 0.1)
    L1o = rng.standard_normal((ng, no, nv)) * 0.1
    L2o = anti(rng.standard_normal((ng, no, no, nv, nv)) * 0.1)
    L1 = numpy.full(L1o.shape, numpy.nan)
    L2 = numpy.full(L2o.shape, numpy.nan)
    Fb = [numpy.ascontiguousarray(getattr(F, k)) for k in F_ORDER]
    Ib = [numpy.ascontiguousarray(getattr(I, k)) for k in I_ORDER]
    grid = [numpy.ascontiguousarray(x) for x in (ti, g, G)]
    L = _L()
    ctx = ctypes.c_void_p()
    assert L.kvft_dryrun_create(0, 7, ctypes.byref(ctx)) == 0
    try:
        Fp = (ctypes.c_void_p * 4)(*[a.ctypes.data for a in Fb])
        Ip = (ctypes.c_void_p * 9)(*[a.ctypes.data for a in Ib])
        st = L.kvft_ccsd_lambda(ctx, ng, nv, no, Fp, Ip, T1.ctypes.data, T2.ctypes.data,
                                L1o.ctypes.data, L2o.ctypes.data, ev.ctypes.data,
                                eo.ctypes.data, grid[0].ctypes.data, grid[1].ctypes.data,
                                grid[2].ctypes.data, L1.ctypes.data, L2.ctypes.data)
        assert st == 0
        mem = _Memory()
        for a in Fb + Ib + grid + [T1, T2, L1o, L2o, L1, L2, ev, eo]:
            mem.add(a)
        i = 0
        ptr, nbytes = ctypes.c_void_p(), ctypes.c_size_t()
        while L.kvft_dryrun_scratch(ctx, i, ctypes.byref(ptr), ctypes.byref(nbytes)) == 0:
            mem.add_raw(ptr.value, nbytes.value)
            i += 1
        kinds = _replay(ctx, mem)
        assert kinds.count(2) == 2
    finally:
        L.kvft_ctx_destroy(ctx)
    r1, r2 = ft_lambda.lambda_update(F, I, T1, T2, L1o, L2o, D1, D2, ti, ng, g, G)
    assert abs(L1 - r1).max() < 1e-12 * abs(r1).max()
    assert abs(L2 - r2).max() < 1e-12 * abs(r2).max()


def test_lambda_densities_dry_run_vs_oracle():
    """kvft_lambda_densities (the Lagrangian's integral gradients) replayed
    against the oracle's response densities (Kelvin's block names)."""
    from oracle import quadrature
    no, nv, ng, beta = 3, 4, 4, 2.0
    rng = numpy.random.default_rng(5)
    F, I = random_system(rng, no, nv)
    anti = lambda x: (x - x.swapaxes(-1, -2)) - (x - x.swapaxes(-1, -2)).swapaxes(-3, -4)
    ev = rng.standard_normal(nv) * 0.5 + 1.0
    eo = rng.standard_normal(no) * 0.5 - 1.0
    D1 = ev[:, None] - eo[None, :]
    D2 = (ev[:, None, None, None] + ev[None, :, None, None] - eo[None, None, :, None]
          - eo[None, None, None, :])
    ti, g, G = quadrature.ft_quad(ng, beta, 'lin')
    T1 = rng.standard_normal((ng, nv, no)) * 0.1
    T2 = anti(rng.standard_normal((ng, nv, nv, no, no)) * 0.1)
    L1 = rng.standard_normal((ng, no, nv)) * 0.1
    L2 = anti(rng.standard_normal((ng, no, no, nv, nv)) * 0.1)
    Fb = [numpy.ascontiguousarray(getattr(F, k)) for k in F_ORDER]
    Ib = [numpy.ascontiguousarray(getattr(I, k)) for k in I_ORDER]
    Fg = [numpy.full(a.shape, numpy.nan) for a in Fb]
    Ig = [numpy.full(a.shape, numpy.nan) for a in Ib]
    grid = [numpy.ascontiguousarray(x) for x in (ti, g, G)]
    L = _L()
    ctx = ctypes.c_void_p()
    assert L.kvft_dryrun_create(0, 7, ctypes.byref(ctx)) == 0
    try:
        P = lambda arrs: (ctypes.c_void_p * len(arrs))(*[a.ctypes.data for a in arrs])
        st = L.kvft_lambda_densities(ctx, ng, nv, no, P(Fb), P(Ib), T1.ctypes.data,
                                     T2.ctypes.data, L1.ctypes.data, L2.ctypes.data,
                                     ev.ctypes.data, eo.ctypes.data, grid[0].ctypes.data,
                                     grid[1].ctypes.data, grid[2].ctypes.data, P(Fg), P(Ig))
        assert st == 0
        mem = _Memory()
        for a in Fb + Ib + Fg + Ig + grid + [T1, T2, L1, L2, ev, eo]:
            mem.add(a)
        i = 0
        ptr, nbytes = ctypes.c_void_p(), ctypes.c_size_t()
        while L.kvft_dryrun_scratch(ctx, i, ctypes.byref(ptr), ctypes.byref(nbytes)) == 0:
            mem.add_raw(ptr.value, nbytes.value)
            i += 1
        _replay(ctx, mem)
    finally:
        L.kvft_ctx_destroy(ctx)
    (pia, pba, pji, pai), P2 = ft_lambda.response_densities(F, I, T1, T2, L1, L2, D1, D2, ti,
                                                            ng, g, G)
    Foo, Fov, Fvo, Fvv = Fg
    for mine, ref in ((Fvo.T, pia), (Fvv.T, pba), (Foo.T, pji), (Fov.T, pai)):
        assert abs(mine - ref).max() < 1e-12 * max(1.0, abs(ref).max())
    for (name, blk, w, pairs), ref in zip(ft_lambda.P2_BLOCKS, P2):
        mine = ft_lambda._asym(Ig[I_ORDER.index(blk)].transpose(2, 3, 0, 1) / w, pairs)
        assert abs(mine - ref).max() < 1e-12 * max(1.0, abs(ref).max()), name


@pytest.mark.parametrize("spin,blocks", [(False, False), (True, False), (False, True),
                                         (True, True)])
def test_lambda_solve_dry_run_vs_oracle(spin, blocks):
    """kvft_lambda_solve (the resident damped loop) for three iterations,
    replayed: the Lambda it leaves and the residual history rebuilt from its
    recorded norms equal the oracle's loop (Kelvin's measure, or its
    unrestricted driver's over the spin cases), with the contractions dense or
    over their nonzero spin-block products."""
    from oracle import ft_ccsd as oft, ft_utils, quadrature, systems
    b = systems.UEGBasis(2 * numpy.pi, 1.2, norb=3)
    eri = systems.g2e_loop(b)
    en = systems.ueg_g_energies(b)
    n, h, ng, beta, mu, damp, its = en.shape[0], en.shape[0] // 2, 4, 10.0, 0.1, 0.2, 3
    fock = systems.g_fock_tot(b, eri, en, 1.0 / beta, mu)
    F, I = oft.ft_integrals(fock, eri, en, beta, mu)
    ti, g, G = quadrature.ft_quad(ng, beta, 'lin')
    D1, D2 = ft_utils.D1(en, en), ft_utils.D2(en, en)
    _, T1, T2 = oft.ft_ccsd(en, fock, eri, 1.0 / beta, mu, ngrid=ng, damp=damp, max_iter=30,
                            return_amplitudes=True)
    L10, L20 = ft_lambda.lambda_guess(F, I, T1, beta, ng, unrestricted=spin)
    hist = []
    R1, R2 = ft_lambda.ft_lambda_iter(L10.copy(), L20.copy(), T1, T2, F, I, D1, D2, g, G, beta,
                                      ng, ti, {"tconv": 0.0, "max_iter": its, "damp": damp},
                                      history=hist, spin_half=h if spin else None)
    L1, L2 = numpy.ascontiguousarray(L10), numpy.ascontiguousarray(L20)
    Fb = [numpy.ascontiguousarray(getattr(F, k)) for k in F_ORDER]
    Ib = [numpy.ascontiguousarray(getattr(I, k)) for k in I_ORDER]
    ev = numpy.ascontiguousarray(en)
    grid = [numpy.ascontiguousarray(x) for x in (ti, g, G, T1, T2)]
    Lib = _L()
    ctx = ctypes.c_void_p()
    iters = ctypes.c_int()
    assert Lib.kvft_dryrun_create(0, 7, ctypes.byref(ctx)) == 0
    sums = []
    try:
        assert Lib.kvft_set_lambda_spin_blocks(ctx, h if blocks else 0) == 0
        P = lambda arrs: (ctypes.c_void_p * len(arrs))(*[a.ctypes.data for a in arrs])
        st = Lib.kvft_lambda_solve(ctx, ng, n, n, P(Fb), P(Ib), grid[3].ctypes.data,
                                   grid[4].ctypes.data, ev.ctypes.data, ev.ctypes.data,
                                   grid[0].ctypes.data, grid[1].ctypes.data,
                                   grid[2].ctypes.data, damp, 0.0, its, h if spin else 0,
                                   L1.ctypes.data, L2.ctypes.data, None, ctypes.byref(iters))
        assert st == 0 and iters.value == its
        mem = _Memory()
        for a in Fb + Ib + grid + [L1, L2, ev]:
            mem.add(a)
        i = 0
        ptr, nbytes = ctypes.c_void_p(), ctypes.c_size_t()
        while Lib.kvft_dryrun_scratch(ctx, i, ctypes.byref(ptr), ctypes.byref(nbytes)) == 0:
            mem.add_raw(ptr.value, nbytes.value)
            i += 1
        kinds = _replay(ctx, mem, sums)
        assert (3 in kinds) == blocks            # spin blocks scale C, then add pieces
    finally:
        Lib.kvft_ctx_destroy(ctx)
    assert abs(L1 - R1).max() < 1e-12 * abs(R1).max()
    assert abs(L2 - R2).max() < 1e-12 * abs(R2).max()
    # the residual history from the recorded norms: nb initial norms, then per
    # iteration nb change norms and nb norms of the damped Lambda
    nb = 5 if spin else 2
    rank1 = [True, True, False, False, False] if spin else [True, False]

    def normalisers(w):
        n1 = 0.1 + sum(numpy.sqrt(x) for x, r in zip(w, rank1) if r)
        n2 = 0.1 + sum((4.0 if spin and k == 3 else 1.0) * numpy.sqrt(x)
                       for k, (x, r) in enumerate(zip(w, rank1)) if not r)
        return n1, n2
    assert len(sums) == nb + 2 * nb * its
    nl = normalisers(sums[:nb])
    for it in range(its):
        blk = sums[nb + 2 * nb * it: nb + 2 * nb * (it + 1)]
        res = sum(numpy.sqrt(x) / (nl[0] if r else nl[1]) for x, r in zip(blk[:nb], rank1))
        assert abs(res - hist[it]) < 1e-12 * hist[it]
        nl = normalisers(blk[nb:])


@pytest.mark.parametrize("unrestricted", [0, 1])
def test_lambda_guess_dry_run_vs_oracle(unrestricted):
    no, nv, ng, beta = 3, 4, 3, 2.0
    rng = numpy.random.default_rng(4 + unrestricted)
    F, I = random_system(rng, no, nv)
    T1 = rng.standard_normal((ng, nv, no)) * 0.1
    L1 = numpy.full((ng, no, nv), numpy.nan)
    L2 = numpy.full((ng, no, no, nv, nv), numpy.nan)
    Fb = [numpy.ascontiguousarray(getattr(F, k)) for k in F_ORDER]
    Ib = [numpy.ascontiguousarray(getattr(I, k)) for k in I_ORDER]
    Lib = _L()
    ctx = ctypes.c_void_p()
    assert Lib.kvft_dryrun_create(0, 7, ctypes.byref(ctx)) == 0
    try:
        P = lambda arrs: (ctypes.c_void_p * len(arrs))(*[a.ctypes.data for a in arrs])
        assert Lib.kvft_lambda_guess(ctx, ng, nv, no, P(Fb), P(Ib), T1.ctypes.data, beta,
                                     unrestricted, L1.ctypes.data, L2.ctypes.data) == 0
        mem = _Memory()
        for a in Fb + Ib + [T1, L1, L2]:
            mem.add(a)
        _replay(ctx, mem)
    finally:
        Lib.kvft_ctx_destroy(ctx)
    r1, r2 = ft_lambda.lambda_guess(F, I, T1, beta, ng, unrestricted=bool(unrestricted))
    assert abs(L1 - r1).max() < 1e-14 and abs(L2 - r2).max() < 1e-15


def test_lambda_densities_spin_blocked_dry_run_vs_oracle():
    """kvft_lambda_densities over spin-block products on a spin-blocked UEG
    (T and Lambda from the oracle's solves) against the oracle's densities."""
    from oracle import ft_ccsd as oft, ft_utils, quadrature, systems
    b = systems.UEGBasis(2 * numpy.pi, 1.2, norb=3)
    eri = systems.g2e_loop(b)
    en = systems.ueg_g_energies(b)
    n, h, ng, T, mu = en.shape[0], en.shape[0] // 2, 4, 0.1, 0.1
    E, S, N, Om, T1, T2, L1, L2 = ft_lambda.solve(en, numpy.diag(numpy.hstack((b.Es, b.Es))),
                                                  eri, T, mu, ngrid=ng, damp=0.2,
                                                  econv=1e-11, lconv=1e-10, max_iter=100)
    beta = 1.0 / T
    fock = systems.g_fock_tot(b, eri, en, T, mu)
    F, I = oft.ft_integrals(fock, eri, en, beta, mu)
    ti, g, G = quadrature.ft_quad(ng, beta, 'lin')
    D1, D2 = ft_utils.D1(en, en), ft_utils.D2(en, en)
    Fb = [numpy.ascontiguousarray(getattr(F, k)) for k in F_ORDER]
    Ib = [numpy.ascontiguousarray(getattr(I, k)) for k in I_ORDER]
    Fg = [numpy.full(a.shape, numpy.nan) for a in Fb]
    Ig = [numpy.full(a.shape, numpy.nan) for a in Ib]
    arrs = [numpy.ascontiguousarray(x) for x in (T1, T2, L1, L2, en, ti, g, G)]
    Lib = _L()
    ctx = ctypes.c_void_p()
    assert Lib.kvft_dryrun_create(0, 7, ctypes.byref(ctx)) == 0
    try:
        assert Lib.kvft_set_lambda_spin_blocks(ctx, h) == 0
        P = lambda a: (ctypes.c_void_p * len(a))(*[x.ctypes.data for x in a])
        d = [a.ctypes.data for a in arrs]
        assert Lib.kvft_lambda_densities(ctx, ng, n, n, P(Fb), P(Ib), d[0], d[1], d[2], d[3],
                                         d[4], d[4], d[5], d[6], d[7], P(Fg), P(Ig)) == 0
        mem = _Memory()
        for a in Fb + Ib + Fg + Ig + arrs:
            mem.add(a)
        i = 0
        ptr, nbytes = ctypes.c_void_p(), ctypes.c_size_t()
        while Lib.kvft_dryrun_scratch(ctx, i, ctypes.byref(ptr), ctypes.byref(nbytes)) == 0:
            mem.add_raw(ptr.value, nbytes.value)
            i += 1
        assert 3 in _replay(ctx, mem)
    finally:
        Lib.kvft_ctx_destroy(ctx)
    R1, R2 = ft_lambda.response_densities(F, I, T1, T2, L1, L2, D1, D2, ti, ng, g, G)
    Foo, Fov, Fvo, Fvv = Fg
    for mine, ref in zip((Fvo.T, Fvv.T, Foo.T, Fov.T), R1):
        assert abs(mine - ref).max() < 1e-12 * max(1.0, abs(ref).max())
    for (name, blk, w, pairs), ref in zip(ft_lambda.P2_BLOCKS, R2):
        mine = ft_lambda._asym(Ig[I_ORDER.index(blk)].transpose(2, 3, 0, 1) / w, pairs)
        assert abs(mine - ref).max() < 1e-12 * max(1.0, abs(ref).max()), name
