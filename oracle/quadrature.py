"""Imaginary-time grids and exp-weighted integrals (oracle; test infrastructure).

Restates kelvin/quadrature.py.  Every rule returns ``(ti, g, G)``:

* ``ti[y]``   -- the tau grid on [0, beta];
* ``g[y]``    -- weights of the integral over [0, beta];
* ``G[y, x]`` -- weights of the cumulative integral over [0, ti[y]].

``int_tbar1/int_tbar2`` (quadrature.py:292-317) evaluate

    T(ti[y]) = sum_x G[y,x] exp(dt_x D) Tbar(ti[x]),
    dt_x = ti[x] - ti[y] for x < y and 0 for x >= y,

which is what Kelvin's loops compute (their ``dt`` array is only written for
x < y and starts at zero).  ``gauss_legendre`` is a rule the reference does not
have: its G is dense, and ``int_tbar*(..., full=True)`` applies the
exponential for every x.
"""
import numpy


def get_G(ng, delta):
    """Simpson cumulative weights, trapezoid first panel (quadrature.py:32-42)."""
    G = numpy.zeros((ng, ng))
    if ng > 1:
        G[1, 0] = G[1, 1] = 0.5 * delta
    for y in range(2, ng):
        G[y] = G[y - 2]
        G[y, y - 2] += delta / 3.0
        G[y, y - 1] += 4.0 * delta / 3.0
        G[y, y] += delta / 3.0
    return G


def get_gint(ng, delta):
    """Simpson weights over the whole interval (quadrature.py:45-60)."""
    g = numpy.zeros(ng)
    if ng % 2 == 0:
        g[0] += 0.5 * delta
        g[1] += 0.5 * delta
        start = 3
    else:
        start = 2
    for y in range(start, ng, 2):
        g[y - 2] += delta / 3.0
        g[y - 1] += 4.0 * delta / 3.0
        g[y] += delta / 3.0
    return g


def get_G_midpoint(ng, delta):
    """Cumulative midpoint weights (quadrature.py:17-23)."""
    return numpy.tril(numpy.full((ng, ng), delta))


def get_g_midpoint(ng, delta):
    """Midpoint weights (quadrature.py:26-29)."""
    return numpy.full(ng, delta)


def get_gL(ng, delta):
    """Left-rectangle weights (quadrature.py:63-67)."""
    g = numpy.full(ng, delta)
    g[ng - 1] = 0.0
    return g


def get_GL(ng, delta):
    """Cumulative left-rectangle weights, G[i,j] = delta for j < i-1
    (quadrature.py:70-75)."""
    G = numpy.zeros((ng, ng))
    for i in range(ng):
        G[i, :max(i - 1, 0)] = delta
    return G


def simpsons(ng, beta):
    """Uniform grid, Simpson weights (quadrature.py:102-107)."""
    delta = beta / (ng - 1.0)
    ti = numpy.arange(ng, dtype=float) * delta
    return ti, get_gint(ng, delta), get_G(ng, delta)


def d_simpsons(ng, beta):
    """d/dbeta of the Simpson weights (quadrature.py:110-115)."""
    ddelta = (beta / (ng - 1.0)) / beta
    return get_gint(ng, ddelta), get_G(ng, ddelta)


def _mapped(ng, beta, delta, si, ti_of, jac_of):
    """Simpson rule on a uniform s-grid mapped by t = ti_of(s) with
    jacobian jac_of(s): g -> g*jac, G[i] -> G[i]*jac (row-wise broadcast
    of the jacobian over the columns, as quadrature.py:126-127 does)."""
    ti = ti_of(si)
    g = get_gint(ng, delta) * jac_of(si)
    G = get_G(ng, delta) * jac_of(si)[None, :]
    return ti, g, G


def simpsons_ln(ng, beta):
    """t = beta ln(s), s in [1, e] (quadrature.py:118-128)."""
    delta = (numpy.exp(1) - 1.0) / (ng - 1.0)
    si = numpy.arange(ng, dtype=float) * delta + 1.0
    return _mapped(ng, beta, delta, si, lambda s: beta * numpy.log(s),
                   lambda s: beta / s)


def simpsons_sin(ng, beta):
    """t = beta (sin(s) + 1)/2, s in [-pi/2, pi/2] (quadrature.py:144-153)."""
    delta = numpy.pi / (ng - 1.0)
    si = numpy.arange(ng, dtype=float) * delta - numpy.pi / 2
    return _mapped(ng, beta, delta, si,
                   lambda s: beta * (numpy.sin(s) + 1.0) / 2.0,
                   lambda s: beta * numpy.cos(s) / 2.0)


def simpsons_exp(ng, beta):
    """t = beta (e^s - 1), s in [0, ln 2] (quadrature.py:167-177)."""
    delta = numpy.log(2.0) / (ng - 1.0)
    si = numpy.arange(ng, dtype=float) * delta
    return _mapped(ng, beta, delta, si,
                   lambda s: beta * (numpy.exp(s) - 1.0),
                   lambda s: beta * numpy.exp(s))


def simpsons_p(ng, beta, n=2):
    """t = beta (s^n + s)/2, s in [0, 1] (quadrature.py:192-201)."""
    delta = 1.0 / (ng - 1.0)
    si = numpy.arange(ng, dtype=float) * delta
    return _mapped(ng, beta, delta, si,
                   lambda s: beta * (numpy.power(s, n) + s) / 2.0,
                   lambda s: beta * (numpy.power(s, n - 1) * float(n) + 1.0) / 2.0)


def midpoint(ng, beta):
    """Midpoint grid (quadrature.py:94-99)."""
    delta = beta / ng
    ti = numpy.arange(ng, dtype=float) * delta + delta / 2
    return ti, get_g_midpoint(ng, delta), get_G_midpoint(ng, delta)


def left(ng, beta):
    """Left-rectangle grid (quadrature.py:78-83)."""
    delta = beta / (ng - 1.0)
    ti = numpy.arange(ng, dtype=float) * delta
    return ti, get_gL(ng, delta), get_GL(ng, delta)


def gauss_legendre(ng, beta):
    """Gauss-Legendre nodes and weights on [0, beta] (no reference rule).

    G[y, x] = int_0^{ti[y]} l_x(t) dt with l_x the Lagrange polynomial of
    node x; G is dense, so int_tbar must be called with ``full=True``.
    """
    x, w = numpy.polynomial.legendre.leggauss(ng)
    ti = 0.5 * beta * (x + 1.0)
    g = 0.5 * beta * w
    # integrate Lagrange basis polynomials exactly with a higher-order GL rule
    xq, wq = numpy.polynomial.legendre.leggauss(ng + 2)
    G = numpy.zeros((ng, ng))
    V = numpy.polynomial.legendre.legvander(x, ng - 1)      # [node, deg]
    Vinv = numpy.linalg.inv(V)                               # coeffs of l_x
    for y in range(ng):
        half = 0.5 * ti[y]
        tq = half * (xq + 1.0)                               # points in [0, ti[y]]
        sq = 2.0 * tq / beta - 1.0                           # back to [-1, 1]
        P = numpy.polynomial.legendre.legvander(sq, ng - 1)  # [q, deg]
        L = P @ Vinv                                         # l_x(t_q)
        G[y] = half * (wq @ L)
    return ti, g, G


def ft_quad(ng, beta, quad):
    """Rule dispatch (quadrature.py:215-235); 'gl' is an added rule."""
    rules = {
        'lin': simpsons, 'ln': simpsons_ln, 'sin': simpsons_sin,
        'exp': simpsons_exp, 'mid': midpoint, 'L': left,
        'gl': gauss_legendre,
    }
    if quad in rules:
        return rules[quad](ng, beta)
    if quad == 'quad':
        return simpsons_p(ng, beta, 2)
    if quad == 'cub':
        return simpsons_p(ng, beta, 3)
    if quad == 'quar':
        return simpsons_p(ng, beta, 4)
    raise Exception("Unrecognized quadrature rule: {}".format(quad))


def _dt_matrix(ti, full=False):
    """dt[y, x] = ti[x] - ti[y] for x < y (all x if full), else 0."""
    ng = ti.shape[0]
    dt = ti[None, :] - ti[:, None]
    if not full:
        dt = numpy.where(numpy.arange(ng)[None, :] < numpy.arange(ng)[:, None],
                         dt, 0.0)
    return dt


def int_tbar1(ng, t1bar, ti, D1, G, full=False):
    """Integrate t1bar with exp(dt D1) factors (quadrature.py:292-303)."""
    dt = _dt_matrix(ti, full)
    out = numpy.zeros(t1bar.shape, dtype=t1bar.dtype)
    for y in range(ng):
        fac = numpy.exp(dt[y][:, None, None] * D1[None, :, :])
        out[y] = numpy.einsum('x,xai->ai', G[y], fac * t1bar)
    return out


def int_tbar2(ng, t2bar, ti, D2, G, full=False):
    """Integrate t2bar with exp(dt D2) factors (quadrature.py:306-317)."""
    dt = _dt_matrix(ti, full)
    out = numpy.zeros(t2bar.shape, dtype=t2bar.dtype)
    for y in range(ng):
        fac = numpy.exp(dt[y][:, None, None, None, None] * D2[None])
        out[y] = numpy.einsum('x,xabij->abij', G[y], fac * t2bar)
    return out


def int_tbar1_single(ng, ig, t1bar, ti, D1, G):
    """One grid point of int_tbar1 (quadrature.py:348-357)."""
    dt = _dt_matrix(ti)[ig]
    fac = numpy.exp(dt[:, None, None] * D1[None])
    return numpy.einsum('x,xai->ai', G[ig], fac * t1bar)


def int_tbar2_single(ng, ig, t2bar, ti, D2, G):
    """One grid point of int_tbar2 (quadrature.py:360-369)."""
    dt = _dt_matrix(ti)[ig]
    fac = numpy.exp(dt[:, None, None, None, None] * D2[None])
    return numpy.einsum('x,xabij->abij', G[ig], fac * t2bar)


def int_L1(ng, L1old, ti, D1, g, G):
    """Backward-in-tau integral for lambda-1 (quadrature.py:320-331)."""
    out = numpy.zeros(L1old.shape, dtype=L1old.dtype)
    for s in range(ng):
        dt = numpy.zeros(ng)
        dt[s:] = ti[s] - ti[s:]
        fac = numpy.exp(dt[:, None, None] * D1[None])          # [y, a, i]
        Lt = fac.transpose(0, 2, 1) * L1old                      # [y, i, a]
        out[s] = numpy.einsum('y,yia,y->ia', g, Lt, G[:, s]) / g[s]
    return out


def int_L2(ng, L2old, ti, D2, g, G):
    """Backward-in-tau integral for lambda-2 (quadrature.py:334-345)."""
    out = numpy.zeros(L2old.shape, dtype=L2old.dtype)
    for s in range(ng):
        dt = numpy.zeros(ng)
        dt[s:] = ti[s] - ti[s:]
        fac = numpy.exp(dt[:, None, None, None, None] * D2[None])
        Lt = fac.transpose(0, 3, 4, 1, 2) * L2old
        out[s] = numpy.einsum('y,yijab,y->ijab', g, Lt, G[:, s]) / g[s]
    return out
