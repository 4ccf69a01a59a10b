"""GPU parity of the libkvft kernels against Kelvin's outputs (golden
fixtures) and the oracle.  FP64 tolerances: 1e-12 absolute on O(0.1-1)
quantities unless stated."""
import numpy
import pytest

from conftest import golden, random_system, random_T, unpack_blocks
from kelvin_gb300 import _lib, ft_cc_energy, ft_cc_equations, quadrature
from oracle import cc_equations as occ
from oracle import ft_ccsd as oft
from oracle import quadrature as oq

pytestmark = pytest.mark.gpu


def close(a, b, rtol=1e-13):
    """max |a - b| <= rtol * max(1, max |b|): random denominators make
    exp(dt D) reach e^12, so the quadrature bound is relative."""
    return abs(a - b).max() <= rtol * max(1.0, abs(b).max())


@pytest.mark.parametrize("tag", ["sq", "rect", "mid"])
def test_int_tbar_vs_kelvin(ctx, tag):
    d = golden("int_tbar.npz")
    ti, G = d[tag + "_ti"], d[tag + "_G"]
    ng = ti.shape[0]
    T1 = quadrature.int_tbar1(ng, d[tag + "_t1bar"], ti, d[tag + "_D1"], G)
    T2 = quadrature.int_tbar2(ng, d[tag + "_t2bar"], ti, d[tag + "_D2"], G)
    assert close(T1, d[tag + "_T1"])
    assert close(T2, d[tag + "_T2"])
    ig = ng - 2
    s1 = quadrature.int_tbar1_single(ng, ig, d[tag + "_t1bar"], ti, d[tag + "_D1"], G)
    s2 = quadrature.int_tbar2_single(ng, ig, d[tag + "_t2bar"], ti, d[tag + "_D2"], G)
    assert close(s1, d[tag + "_T1single"])
    assert close(s2, d[tag + "_T2single"])


@pytest.mark.parametrize("rule,ng", [("lin", 10), ("lin", 11), ("ln", 8), ("sin", 9),
                                     ("exp", 6), ("quad", 7), ("mid", 12), ("L", 9)])
def test_int_tbar_rules_vs_oracle(ctx, rule, ng):
    """Every Kelvin rule (uniform and mapped grids, step-1/step-2 chains)."""
    rng = numpy.random.default_rng(ng)
    nv, no = 4, 3
    ti, g, G = quadrature.ft_quad(ng, 4.0, rule)
    ev, eo = rng.standard_normal(nv) * 2, rng.standard_normal(no) * 2
    D2 = (ev[:, None, None, None] + ev[None, :, None, None]
          - eo[None, None, :, None] - eo[None, None, None, :])
    t2b = rng.standard_normal((ng, nv, nv, no, no))
    ref = oq.int_tbar2(ng, t2b, ti, D2, G)
    out = quadrature.int_tbar2(ng, t2b, ti, D2, G)
    assert abs(out - ref).max() <= 1e-12 * max(1.0, abs(ref).max())


def test_int_tbar_dense_gl_full(ctx):
    ng = 8
    rng = numpy.random.default_rng(5)
    ti, g, G = quadrature.ft_quad(ng, 2.0, "gl")
    D1 = rng.standard_normal((3, 4)) * 0.5
    t1b = rng.standard_normal((ng, 3, 4))
    for full in (False, True):
        ref = oq.int_tbar1(ng, t1b, ti, D1, G, full=full)
        out = quadrature.int_tbar1(ng, t1b, ti, D1, G, full=full)
        assert close(out, ref, 1e-12)


def test_int_tbar_large_properties(ctx):
    """n=24, ng=16: linearity and the D = 0 limit (T = G tbar), on sizes the
    oracle would take long on."""
    ng, n = 16, 24
    rng = numpy.random.default_rng(11)
    ti, g, G = quadrature.ft_quad(ng, 5.0, "lin")
    x = rng.standard_normal((ng, n, n, n, n))
    y = rng.standard_normal((ng, n, n, n, n))
    D = rng.standard_normal((n, n, n, n))
    a, b = 0.75, -1.5
    lhs = quadrature.int_tbar2(ng, a * x + b * y, ti, D, G)
    rhs = a * quadrature.int_tbar2(ng, x, ti, D, G) + b * quadrature.int_tbar2(ng, y, ti, D, G)
    assert abs(lhs - rhs).max() < 1e-11 * abs(lhs).max()
    z = quadrature.int_tbar2(ng, x, ti, numpy.zeros_like(D), G)
    assert close(z, numpy.einsum('yx,xp->yp', G, x.reshape(ng, -1)).reshape(x.shape), 1e-13)


def test_energy_vs_kelvin(ctx):
    d = golden("energy.npz")
    for q, key in ((True, "E_q"), (False, "E_noq")):
        E = ft_cc_energy.ft_cc_energy(d["T1"], d["T2"], d["f"], d["eri"], d["g"],
                                      float(d["beta"]), q)
        assert abs(E - float(d[key])) < 1e-12


@pytest.mark.parametrize("no,nv,seed", [(3, 3, 0), (3, 5, 1), (5, 2, 2), (6, 6, 3)])
def test_stanton_residual_vs_oracle(ctx, no, nv, seed):
    rng = numpy.random.default_rng(seed)
    F, I = random_system(rng, no, nv)
    t1, t2 = random_T(rng, 1, nv, no, 0.2)
    R1, R2 = occ.residual(F, I, t1[0], t2[0])
    T1 = numpy.full((nv, no), 0.5)
    T2 = numpy.full((nv, nv, no, no), -0.25)
    ft_cc_equations.stanton_residual(T1, T2, F, I, t1[0], t2[0], fac=-1.0)
    assert abs(T1 - (0.5 - R1)).max() < 1e-12
    assert abs(T2 - (-0.25 - R2)).max() < 1e-12


@pytest.mark.parametrize("prefix", ["ft_", "rb_"])
def test_ccsd_stanton_vs_kelvin(ctx, prefix):
    d = golden("stanton.npz")
    F, I = unpack_blocks(d, prefix)
    ti, G = d[prefix + "ti"], d[prefix + "G"]
    T1, T2 = ft_cc_equations.ccsd_stanton(F, I, d[prefix + "t1"], d[prefix + "t2"],
                                          d[prefix + "D1"], d[prefix + "D2"], ti,
                                          ti.shape[0], G)
    assert close(T1, d[prefix + "T1"], 1e-12)
    assert close(T2, d[prefix + "T2"], 1e-12)


def test_ccsd_stanton_batched_vs_oracle(ctx):
    """n = 10 spin orbitals, ng = 6 tau points: every GEMM path incl. split-K."""
    rng = numpy.random.default_rng(7)
    n, ng = 10, 6
    F, I = random_system(rng, n, n, 0.1, 0.05)
    t1, t2 = random_T(rng, ng, n, n, 0.05)
    ti, g, G = quadrature.ft_quad(ng, 2.0, "lin")
    e = numpy.sort(rng.standard_normal(n))
    D1 = e[:, None] - e[None, :]
    D2 = (e[:, None, None, None] + e[None, :, None, None]
          - e[None, None, :, None] - e[None, None, None, :])
    r1, r2 = oft.ccsd_stanton(F, I, t1, t2, D1, D2, ti, ng, G)
    o1, o2 = ft_cc_equations.ccsd_stanton(F, I, t1, t2, D1, D2, ti, ng, G)
    assert close(o1, r1, 1e-12)
    assert close(o2, r2, 1e-12)


def test_bad_arguments_raise(ctx):
    with pytest.raises(Exception):
        quadrature.int_tbar1(3, numpy.zeros((2, 2, 2)), numpy.zeros(3), numpy.zeros((2, 2)),
                             numpy.zeros((3, 3)))
    with pytest.raises(_lib.KvftError):
        ctx.set_precision(9)
