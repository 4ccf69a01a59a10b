"""Fermi-Dirac helpers used on the FT-CCSD path (oracle; test infrastructure).

Kelvin imports these from the external, un-vendored ``cqcpy`` package
(``cqcpy.ft_utils.ff/ffv/GP0``, ``cqcpy.utils.D1/D2``), called at
kelvin/ccsd.py:628-638 and kelvin/cc_utils.py:571-572.  They are restated here
from their definitions:

    f_p   = 1 / (1 + exp(beta (e_p - mu)))          occupation
    1-f_p = 1 / (1 + exp(-beta (e_p - mu)))         vacancy
    g0_p  = -(1/beta) ln(1 + exp(-beta (e_p - mu)))  orbital grand potential
    D1[a,i]     = e_a - e_i
    D2[a,b,i,j] = e_a + e_b - e_i - e_j
"""
import numpy


def ff(beta, e, mu):
    """Fermi-Dirac occupation f_p (cqcpy.ft_utils.ff, used at ccsd.py:628)."""
    x = beta * (numpy.asarray(e, dtype=float) - mu)
    # 1/(1+e^x) written through e^{-|x|} so that neither branch overflows
    ex = numpy.exp(-numpy.abs(x))
    return numpy.where(x > 0, ex / (1.0 + ex), 1.0 / (1.0 + ex))


def ffv(beta, e, mu):
    """Vacancy 1 - f_p (cqcpy.ft_utils.ffv, used at ccsd.py:629)."""
    return ff(beta, -numpy.asarray(e, dtype=float), -mu)


def GP0(beta, e, mu):
    """Orbital grand potentials (cqcpy.ft_utils.GP0, used at ccsd.py:638)."""
    x = -beta * (numpy.asarray(e, dtype=float) - mu)
    # ln(1+e^x) = max(x,0) + ln(1+e^{-|x|})
    return -(numpy.maximum(x, 0.0) + numpy.log1p(numpy.exp(-numpy.abs(x)))) / beta


def D1(ev, eo):
    """D1[a,i] = e_a - e_i (cqcpy.utils.D1, used at ccsd.py:633)."""
    return numpy.asarray(ev)[:, None] - numpy.asarray(eo)[None, :]


def D2(ev, eo):
    """D2[a,b,i,j] = e_a + e_b - e_i - e_j (cqcpy.utils.D2, ccsd.py:634)."""
    ev = numpy.asarray(ev)
    eo = numpy.asarray(eo)
    return (ev[:, None, None, None] + ev[None, :, None, None]
            - eo[None, None, :, None] - eo[None, None, None, :])


def HtoK(T):
    """Hartree to Kelvin (cqcpy.ft_utils.HtoK, logging only)."""
    return T * 315775.13


class one_e_blocks(object):
    """Attribute container .oo .ov .vo .vv (cqcpy.ov_blocks.one_e_blocks)."""

    def __init__(self, oo, ov, vo, vv):
        self.oo = oo
        self.ov = ov
        self.vo = vo
        self.vv = vv


class two_e_blocks(object):
    """Attribute container for the nine ERI blocks
    (cqcpy.ov_blocks.two_e_blocks, used at cc_utils.py:599-601)."""

    NAMES = ("vvvv", "vvvo", "vovv", "vvoo", "vovo",
             "oovv", "vooo", "ooov", "oooo")

    def __init__(self, vvvv=None, vvvo=None, vovv=None, vvoo=None, vovo=None,
                 oovv=None, vooo=None, ooov=None, oooo=None):
        self.vvvv = vvvv
        self.vvvo = vvvo
        self.vovv = vovv
        self.vvoo = vvoo
        self.vovo = vovo
        self.oovv = oovv
        self.vooo = vooo
        self.ooov = ooov
        self.oooo = oooo
