"""The digit-sliced BF16 tensor-core contraction engine (tcgen05) against
FP64.  Error bounds are norm-wise: |C - A B| <= tol * K * max_k|A_mk| max_k|B_kn|,
with tol from the digit count (7 levels: FP64-grade)."""
import json
import os

import numpy
import pytest

from conftest import GOLDEN, random_system, random_T
from kelvin_gb300 import _lib, ccsd, ft_cc_equations, systems
from oracle import cc_equations as occ

pytestmark = pytest.mark.gpu

TOL = {2: 2e-3, 3: 5e-5, 4: 5e-7, 5: 5e-9, 7: 5e-12}


@pytest.fixture
def tc_ctx(ctx):
    yield ctx
    ctx.set_precision(_lib.PREC_FP64, 7)


def gemm(ctx, A, B, prec, digits):
    batch = A.shape[0] if A.ndim == 3 else 1
    A3 = A.reshape(batch, A.shape[-2], A.shape[-1])
    B3 = B.reshape(batch, B.shape[-2], B.shape[-1])
    M, K = A3.shape[1:]
    N = B3.shape[2]
    dA, dB = _lib.DeviceArray.from_host(ctx, A3), _lib.DeviceArray.from_host(ctx, B3)
    dC = _lib.DeviceArray(ctx, (batch, M, N))
    ctx.check(ctx.L.kvft_gemm(ctx.h, M, N, K, batch, prec, digits, dA.ptr, dB.ptr, dC.ptr),
              "kvft_gemm")
    return dC.to_host()


def normwise(C, A, B):
    A3 = A.reshape(-1, A.shape[-2], A.shape[-1])
    B3 = B.reshape(-1, B.shape[-2], B.shape[-1])
    ref = A3 @ B3
    K = A3.shape[2]
    bound = abs(A3).max(2)[:, :, None] * abs(B3).max(1)[:, None, :] * K
    bound = numpy.where(bound == 0, 1.0, bound)
    return (abs(C.reshape(ref.shape) - ref) / bound).max()


@pytest.mark.parametrize("M,N,K,batch", [(37, 50, 300, 1), (128, 128, 1444, 1),
                                         (200, 64, 2048, 2), (130, 260, 4100, 1),
                                         (300, 1444, 1444, 1)])
@pytest.mark.parametrize("digits", [3, 5, 7])
def test_tc_gemm_accuracy(ctx, M, N, K, batch, digits):
    rng = numpy.random.default_rng(M * 7 + N + K + digits)
    A = rng.standard_normal((batch, M, K)) * numpy.exp(rng.standard_normal((batch, M, 1)) * 3)
    B = rng.standard_normal((batch, K, N)) * 1e-3
    A[:, 0, :] = 0.0                          # an all-zero row
    C = gemm(ctx, A, B, _lib.PREC_FP64_TC, digits)
    assert normwise(C, A, B) < TOL[digits]


# Unit schedules of the persistent kernel: K chunks summed inside one unit
# (>= two waves of tiles), K chunks as separate units added by atomics (few
# tiles), C's contiguous index kept on the columns (narrow N, long K), skinny
# products (N = 1, 8) against a long K, and many waves of persistent tiles
# with ragged edges in both directions (31 m-tiles, 24 or 47 n-tiles).
@pytest.mark.parametrize("M,N,K,batch", [(2048, 2560, 4200, 1), (640, 640, 2500, 8),
                                         (300, 40, 1000, 1), (3000, 8, 5000, 1),
                                         (1444, 1, 1444, 6), (3900, 3000, 2100, 1)])
@pytest.mark.parametrize("digits", [3, 7])
def test_tc_gemm_unit_schedules(ctx, M, N, K, batch, digits):
    rng = numpy.random.default_rng(M + 3 * N + K + digits)
    A = rng.standard_normal((batch, M, K)) * numpy.exp(rng.standard_normal((batch, M, 1)))
    B = rng.standard_normal((batch, K, N))
    C = gemm(ctx, A, B, _lib.PREC_FP64_TC, digits)
    assert normwise(C, A, B) < TOL[digits]


# Short contractions (K <= 256) are packed in one pass that holds whole rows
# in shared memory: one, two and four 64-wide k tiles, odd K, rows whose
# contiguous index is K (A) or the row index (B), all-zero rows on both sides.
# With few terms the rounding errors of the digit products do not average
# out against the K in the norm-wise bound, so it grows as sqrt(256 / K)
# (an exact emulation of the digit arithmetic gives 9.1e-5 for K = 16 at
# three levels).
@pytest.mark.parametrize("K", [16, 57, 64, 114, 129, 200, 256])
@pytest.mark.parametrize("digits", [3, 5, 7])
def test_tc_gemm_short_k(ctx, K, digits):
    rng = numpy.random.default_rng(K + 1000 * digits)
    A = rng.standard_normal((3, 333, K)) * numpy.exp(rng.standard_normal((3, 333, 1)) * 4)
    B = rng.standard_normal((3, K, 517)) * numpy.exp(rng.standard_normal((3, 1, 517)) * 4)
    A[:, 5, :] = 0.0
    B[:, :, 7] = 0.0
    C = gemm(ctx, A, B, _lib.PREC_FP64_TC, digits)
    assert normwise(C, A, B) < TOL[digits] * max(1.0, (256 / K) ** 0.5)
    assert not C[:, 5, :].any() and not C[:, :, 7].any()


# FP32-pair levels (four or more digits) with a short K run on 32-wide tiles
# with two accumulator sets: partial and exact tile widths, one or several
# n-tiles, partial m-tiles, a batch.
@pytest.mark.parametrize("M,N,K,batch", [(300, 20, 57, 2), (333, 57, 57, 1),
                                         (128, 64, 100, 3), (57, 900, 57, 2)])
@pytest.mark.parametrize("digits", [4, 6, 7])
def test_tc_gemm_short_k_narrow_pair_levels(ctx, M, N, K, batch, digits):
    rng = numpy.random.default_rng(M + 7 * N + K + digits)
    A = rng.standard_normal((batch, M, K)) * numpy.exp(rng.standard_normal((batch, M, 1)) * 3)
    B = rng.standard_normal((batch, K, N)) * numpy.exp(rng.standard_normal((batch, 1, N)) * 3)
    C = gemm(ctx, A, B, _lib.PREC_FP64_TC, digits)
    tol = TOL.get(digits, 5e-11 if digits == 6 else None)
    assert normwise(C, A, B) < tol * max(1.0, (256 / K) ** 0.5)


# Few output columns after the orientation swap (C's contiguous index on the
# tile rows, the short extent on the columns): 64-wide tiles at two and three
# digit levels, with one or several K chunks.
@pytest.mark.parametrize("M,N,K,batch", [(57, 3000, 114, 2), (40, 2000, 600, 1),
                                         (64, 1000, 2500, 1), (9, 5000, 57, 3)])
@pytest.mark.parametrize("digits", [2, 3])
def test_tc_gemm_narrow_tiles(ctx, M, N, K, batch, digits):
    rng = numpy.random.default_rng(M + N + K + digits)
    A = rng.standard_normal((batch, M, K)) * numpy.exp(rng.standard_normal((batch, M, 1)))
    B = rng.standard_normal((batch, K, N))
    C = gemm(ctx, A, B, _lib.PREC_FP64_TC, digits)
    assert normwise(C, A, B) < TOL[digits] * max(1.0, (256 / K) ** 0.5)


@pytest.mark.parametrize("digits", [2, 3, 4, 5, 6, 7])
def test_tc_gemm_every_digit_count(ctx, digits):
    """Each digit count is its own kernel instance (levels fixed at compile
    time); the error falls by ~2^-7 per level."""
    rng = numpy.random.default_rng(100 + digits)
    A = rng.standard_normal((2, 300, 2500))
    B = rng.standard_normal((2, 2500, 260))
    C = gemm(ctx, A, B, _lib.PREC_FP64_TC, digits)
    tol = TOL.get(digits, 5e-11 if digits == 6 else None)
    assert normwise(C, A, B) < tol


def test_tc_gemm_matches_fp64_engine(ctx):
    rng = numpy.random.default_rng(3)
    A = rng.standard_normal((1, 96, 777))
    B = rng.standard_normal((1, 777, 333))
    C64 = gemm(ctx, A, B, _lib.PREC_FP64, 7)
    Ctc = gemm(ctx, A, B, _lib.PREC_FP64_TC, 7)
    assert normwise(C64, A, B) < 1e-15 * 777
    assert abs(Ctc - C64).max() < 5e-12 * 777 * abs(A).max() * abs(B).max()


@pytest.mark.parametrize("no,nv,digits", [(6, 6, 7), (5, 9, 7), (8, 8, 5)])
def test_stanton_residual_tc_vs_oracle(tc_ctx, no, nv, digits):
    rng = numpy.random.default_rng(no * 10 + nv)
    F, I = random_system(rng, no, nv)
    t1, t2 = random_T(rng, 1, nv, no, 0.2)
    R1, R2 = occ.residual(F, I, t1[0], t2[0])
    tc_ctx.set_precision(_lib.PREC_FP64_TC, digits)
    T1 = numpy.zeros((nv, no))
    T2 = numpy.zeros((nv, nv, no, no))
    ft_cc_equations.stanton_residual(T1, T2, F, I, t1[0], t2[0], fac=1.0, ctx=tc_ctx)
    scale = max(abs(R2).max(), 1.0)
    tol = 1e-11 if digits == 7 else 1e-7
    assert abs(T1 - R1).max() < tol * scale
    assert abs(T2 - R2).max() < tol * scale


def test_ueg7_fp64_tc_vs_kelvin(tc_ctx):
    meta = json.load(open(os.path.join(GOLDEN, "ueg7.json")))
    s = systems.UEGSystem(meta["T"], meta["L"], meta["cutoff"], mu=meta["mu"], norb=7)
    cc = ccsd.ccsd(s, T=meta["T"], mu=meta["mu"], max_iter=50, damp=meta["damp"], ngrid=10,
                   precision="fp64_tc", ctx=tc_ctx)
    Et, Ecc = cc.run()
    assert abs(Ecc - meta["Omega_cc"]) < 1e-10
    assert abs(Et - meta["Omega_total"]) < 1e-10


def test_ueg19_fp64_tc_vs_kelvin_example(tc_ctx):
    s = systems.UEGSystem(0.1, 2 * numpy.pi, 1.2, mu=0.1, norb=19)
    cc = ccsd.ccsd(s, T=0.1, mu=0.1, max_iter=50, damp=0.2, ngrid=10, precision="fp64_tc",
                   ctx=tc_ctx)
    Et, Ecc = cc.run()
    assert abs(Ecc - (-0.015646626108)) < 1e-10


def test_mixed_vs_fp64_on_benchmark_system(tc_ctx):
    """UEG 14 e-, rs=4, 38 spin orbitals, ng=10: the few-digit phases end
    within 1e-6 Ha per electron of FP64, and the FP64-accurate refinement
    sweeps then meet Kelvin's own test, landing on the FP64 answer."""
    s = systems.ueg_recipe(14, 4.0, 19, 0.5)
    kw = dict(T=s.T, mu=s.mu, max_iter=100, damp=0.5, ngrid=10, econv=1e-10, ctx=tc_ctx)
    ref = ccsd.ccsd(s, precision="fp64_tc", **kw)
    E64 = ref.run()[1]
    mix = ccsd.ccsd(s, precision="mixed", **kw)
    Emx = mix.run()[1]
    assert mix.converged and ref.converged
    assert mix.phases[0][0] == 3 and mix.phases[-1][0] == 7
    assert mix.iterations_refine >= 2
    assert abs(Emx - E64) < 1e-9
    assert abs(mix.omega_low - E64) < 1e-6 * s.N


def test_ueg19_mixed_within_tolerance(tc_ctx):
    """Mixed form (5 digit levels): |dOmega| <= 1e-6 Ha per electron."""
    s = systems.UEGSystem(0.1, 2 * numpy.pi, 1.2, mu=0.1, norb=19)
    cc = ccsd.ccsd(s, T=0.1, mu=0.1, max_iter=50, damp=0.2, ngrid=10, precision="mixed",
                   digits=5, ctx=tc_ctx)
    Et, Ecc = cc.run()
    assert abs(Ecc - (-0.015646626108)) < 1e-6 * s.N
