"""Tau grids and the exp-weighted time integrals, drop-in for
kelvin/quadrature.py.

Grid construction (``ft_quad``/``d_ft_quad`` and the named rules) is O(ng^2)
host arithmetic, as in Kelvin.  The integrals ``int_tbar1/int_tbar2`` and
their single-point forms run on the GPU through libkvft; they accept numpy
arrays (copied in and out) or ``DeviceArray`` inputs (results stay on the
device).
"""
import numpy

from . import _lib


# ---------------------------------------------------------------------------
# weights (quadrature.py:17-75)
# ---------------------------------------------------------------------------
def get_G(ng, delta):
    """Cumulative Simpson weights with a trapezoid first panel
    (quadrature.py:32-42): row y integrates [0, ti[y]]."""
    G = numpy.zeros((ng, ng))
    simpson = numpy.array([1.0, 4.0, 1.0]) * (delta / 3.0)
    for y in range(1, ng):
        if y == 1:
            G[1, :2] = 0.5 * delta
        else:
            G[y] = G[y - 2]
            G[y, y - 2:y + 1] += simpson
    return G


def get_gint(ng, delta):
    """Simpson weights over [0, beta] (quadrature.py:45-60); an even ng puts
    a trapezoid on the first panel."""
    g = numpy.zeros(ng)
    first = 1 if ng % 2 == 0 else 0
    if first:
        g[:2] += 0.5 * delta
    for y in range(first, ng - 2, 2):
        g[y:y + 3] += numpy.array([1.0, 4.0, 1.0]) * (delta / 3.0)
    return g


def get_G_midpoint(ng, delta):
    return numpy.tril(numpy.full((ng, ng), float(delta)))


def get_g_midpoint(ng, delta):
    return numpy.full(ng, float(delta))


def get_gL(ng, delta):
    g = numpy.full(ng, float(delta))
    g[-1] = 0.0
    return g


def get_GL(ng, delta):
    return numpy.tril(numpy.full((ng, ng), float(delta)), k=-2)


# ---------------------------------------------------------------------------
# rules (quadrature.py:78-256)
# ---------------------------------------------------------------------------
def _uniform(ng, beta):
    delta = beta / (ng - 1.0)
    return numpy.arange(ng) * delta, delta


def simpsons(ng, beta):
    ti, delta = _uniform(ng, beta)
    return ti, get_gint(ng, delta), get_G(ng, delta)


def d_simpsons(ng, beta):
    ddelta = 1.0 / (ng - 1.0)
    return get_gint(ng, ddelta), get_G(ng, ddelta)


def left(ng, beta):
    ti, delta = _uniform(ng, beta)
    return ti, get_gL(ng, delta), get_GL(ng, delta)


def d_left(ng, beta):
    ddelta = 1.0 / (ng - 1.0)
    return get_gL(ng, ddelta), get_GL(ng, ddelta)


def midpoint(ng, beta):
    delta = beta / ng
    ti = numpy.arange(ng) * delta + delta / 2
    return ti, get_g_midpoint(ng, delta), get_G_midpoint(ng, delta)


# mapped Simpson rules: t = beta * m(s) on a uniform s-grid; the weights pick
# up the jacobian beta * m'(s) column-wise (quadrature.py:118-212)
_MAPS = {
    'ln': (lambda ng: (numpy.exp(1) - 1.0) / (ng - 1.0), 1.0,
           numpy.log, lambda s: 1.0 / s),
    'sin': (lambda ng: numpy.pi / (ng - 1.0), -numpy.pi / 2,
            lambda s: (numpy.sin(s) + 1.0) / 2.0, lambda s: numpy.cos(s) / 2.0),
    'exp': (lambda ng: numpy.log(2.0) / (ng - 1.0), 0.0,
            lambda s: numpy.exp(s) - 1.0, numpy.exp),
}


def _power_map(n):
    return (lambda ng: 1.0 / (ng - 1.0), 0.0,
            lambda s: (numpy.power(s, n) + s) / 2.0,
            lambda s: (numpy.power(s, n - 1) * float(n) + 1.0) / 2.0)


def _mapped_rule(ng, beta, rule, deriv=False):
    step, s0, m, dm = rule
    delta = step(ng)
    si = numpy.arange(ng) * delta + s0
    jac = dm(si) if deriv else beta * dm(si)
    g = get_gint(ng, delta) * jac
    G = get_G(ng, delta) * jac[None, :]
    if deriv:
        return g, G
    return beta * m(si), g, G


def gauss_legendre(ng, beta):
    """Gauss-Legendre nodes/weights on [0, beta]; G[y,x] integrates the
    Lagrange polynomial of node x over [0, ti[y]] (dense; use full=True).
    Kelvin has no such rule."""
    x, w = numpy.polynomial.legendre.leggauss(ng)
    ti = 0.5 * beta * (x + 1.0)
    g = 0.5 * beta * w
    xq, wq = numpy.polynomial.legendre.leggauss(ng + 2)
    Vinv = numpy.linalg.inv(numpy.polynomial.legendre.legvander(x, ng - 1))
    tq = 0.5 * ti[:, None] * (xq[None, :] + 1.0)                 # [y, q]
    P = numpy.polynomial.legendre.legvander(2.0 * tq / beta - 1.0, ng - 1)
    G = 0.5 * ti[:, None] * numpy.einsum('q,yqd,dx->yx', wq, P, Vinv)
    return ti, g, G


def ft_quad(ng, beta, quad):
    """(ti, g, G) for a named rule (quadrature.py:215-235) plus 'gl'."""
    if quad == 'lin':
        return simpsons(ng, beta)
    if quad in _MAPS:
        return _mapped_rule(ng, beta, _MAPS[quad])
    if quad in ('quad', 'cub', 'quar'):
        return _mapped_rule(ng, beta, _power_map({'quad': 2, 'cub': 3, 'quar': 4}[quad]))
    if quad == 'mid':
        return midpoint(ng, beta)
    if quad == 'L':
        return left(ng, beta)
    if quad == 'gl':
        return gauss_legendre(ng, beta)
    raise Exception("Unrecognized quadrature rule: {}".format(quad))


def d_ft_quad(ng, beta, quad):
    """d/dbeta of (g, G) (quadrature.py:238-256)."""
    if quad == 'lin':
        return d_simpsons(ng, beta)
    if quad in _MAPS:
        return _mapped_rule(ng, beta, _MAPS[quad], deriv=True)
    if quad in ('quad', 'cub', 'quar'):
        return _mapped_rule(ng, beta, _power_map({'quad': 2, 'cub': 3, 'quar': 4}[quad]),
                            deriv=True)
    if quad == 'L':
        return d_left(ng, beta)
    raise Exception("Unrecognized quadrature rule: {}".format(quad))


# ---------------------------------------------------------------------------
# GPU integrals (quadrature.py:292-317, 348-369)
# ---------------------------------------------------------------------------
def _int_tbar(rank, ng, tbar, ti, D, G, full, ctx):
    ctx = ctx or _lib.context()
    host = not isinstance(tbar, _lib.DeviceArray)
    shape = tbar.shape
    nv, no = shape[1], shape[-1]
    if len(shape) != (3 if rank == 1 else 5) or shape[0] != ng:
        raise Exception("int_tbar%d: bad amplitude shape %s" % (rank, shape))
    dt = _lib.as_device(ctx, tbar)
    dti = _lib.as_device(ctx, ti)
    dD = _lib.as_device(ctx, D)
    dG = _lib.as_device(ctx, G)
    out = _lib.DeviceArray(ctx, shape)
    fn = ctx.L.kvft_int_tbar1 if rank == 1 else ctx.L.kvft_int_tbar2
    ctx.check(fn(ctx.h, ng, nv, no, dt.ptr, dti.ptr, dD.ptr, dG.ptr, int(bool(full)), out.ptr),
              "int_tbar%d" % rank)
    return out.to_host() if host else out


def int_tbar1(ng, t1bar, ti, D1, G, full=False, ctx=None):
    """T1(ti[y]) = sum_x G[y,x] exp(dt D1) t1bar[x] (quadrature.py:292-303)."""
    return _int_tbar(1, ng, t1bar, ti, D1, G, full, ctx)


def int_tbar2(ng, t2bar, ti, D2, G, full=False, ctx=None):
    """T2(ti[y]) = sum_x G[y,x] exp(dt D2) t2bar[x] (quadrature.py:306-317)."""
    return _int_tbar(2, ng, t2bar, ti, D2, G, full, ctx)


def _int_single(rank, ng, ig, tbar, ti, D, G, ctx):
    ctx = ctx or _lib.context()
    host = not isinstance(tbar, _lib.DeviceArray)
    shape = tbar.shape
    nv, no = shape[1], shape[-1]
    dt = _lib.as_device(ctx, tbar)
    out = _lib.DeviceArray(ctx, shape[1:])
    dti, dD, dG = (_lib.as_device(ctx, a) for a in (ti, D, G))
    fn = ctx.L.kvft_int_tbar1_single if rank == 1 else ctx.L.kvft_int_tbar2_single
    ctx.check(fn(ctx.h, ng, ig, nv, no, dt.ptr, dti.ptr, dD.ptr, dG.ptr, out.ptr),
              "int_tbar%d_single" % rank)
    return out.to_host() if host else out


def int_tbar1_single(ng, ig, t1bar, ti, D1, G, ctx=None):
    """One grid point of int_tbar1 (quadrature.py:348-357)."""
    return _int_single(1, ng, ig, t1bar, ti, D1, G, ctx)


def int_tbar2_single(ng, ig, t2bar, ti, D2, G, ctx=None):
    """One grid point of int_tbar2 (quadrature.py:360-369)."""
    return _int_single(2, ng, ig, t2bar, ti, D2, G, ctx)
