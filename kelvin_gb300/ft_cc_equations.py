"""FT-CCSD amplitude update on the GPU, drop-in for kelvin/ft_cc_equations.py.

``ccsd_stanton(F, I, T1old, T2old, D1, D2, ti, ng, G)`` has Kelvin's signature
and semantics (ft_cc_equations.py:96-113): for every tau point the CCSD
residual with Stanton-Gauss intermediates gives tbar = -F.vo - R1(t),
-I.vvoo - R2(t); the result is integrated in imaginary time.  Inputs are
never modified; new arrays are returned.  numpy inputs give numpy outputs;
``DeviceArray`` amplitudes give device outputs.
"""
import numpy

from . import _lib

F_ORDER = ("oo", "ov", "vo", "vv")
I_ORDER = ("vvvv", "vvvo", "vovv", "vvoo", "vovo", "oovv", "vooo", "ooov", "oooo")


class DeviceBlocks(object):
    """Device copies of Kelvin's one_e_blocks / two_e_blocks containers."""

    def __init__(self, ctx, F, I):
        self.F = [_lib.as_device(ctx, getattr(F, b)) for b in F_ORDER]
        self.I = [_lib.as_device(ctx, getattr(I, b)) for b in I_ORDER]
        nv, no = self.F[2].shape
        self.nv, self.no = nv, no
        self.Fp = _lib.ptr_array(self.F)
        self.Ip = _lib.ptr_array(self.I)


_cache = {}


def device_blocks(ctx, F, I):
    """Device blocks for (F, I), reused while the same objects are passed."""
    key = (id(F), id(I), ctx.device)
    hit = _cache.get(key)
    if hit is not None and hit[0] is F and hit[1] is I:
        return hit[2]
    blk = DeviceBlocks(ctx, F, I)
    _cache.clear()
    _cache[key] = (F, I, blk)
    return blk


def ccsd_stanton(F, I, T1old, T2old, D1, D2, ti, ng, G, full=False, ctx=None,
                 precision=None):
    """Time-dependent CCSD iteration with Stanton-Gauss intermediates."""
    ctx = ctx or _lib.context()
    if precision is not None:
        ctx.set_precision(*precision) if isinstance(precision, tuple) \
            else ctx.set_precision(precision)
    host = not isinstance(T1old, _lib.DeviceArray)
    blk = device_blocks(ctx, F, I)
    nv, no = blk.nv, blk.no
    if tuple(T1old.shape) != (ng, nv, no) or tuple(T2old.shape) != (ng, nv, nv, no, no):
        raise Exception("ccsd_stanton: amplitude shapes do not match F.vo / ng")
    d1, d2 = _lib.as_device(ctx, T1old), _lib.as_device(ctx, T2old)
    dD1, dD2, dti, dG = (_lib.as_device(ctx, a) for a in (D1, D2, ti, G))
    o1 = _lib.DeviceArray(ctx, (ng, nv, no))
    o2 = _lib.DeviceArray(ctx, (ng, nv, nv, no, no))
    ctx.check(ctx.L.kvft_ccsd_stanton(ctx.h, ng, nv, no, blk.Fp, blk.Ip, d1.ptr, d2.ptr,
                                      dD1.ptr, dD2.ptr, dti.ptr, dG.ptr, int(bool(full)),
                                      o1.ptr, o2.ptr), "ccsd_stanton")
    if host:
        return o1.to_host(), o2.to_host()
    return o1, o2


def stanton_residual(T1, T2, F, I, t1, t2, fac=1.0, ctx=None):
    """In-place T1 += fac R1(t1,t2), T2 += fac R2 for one tau point: the
    contract of cqcpy.cc_equations._Stanton called at ft_cc_equations.py:106."""
    ctx = ctx or _lib.context()
    blk = device_blocks(ctx, F, I)
    nv, no = blk.nv, blk.no
    dT1, dT2 = _lib.as_device(ctx, T1), _lib.as_device(ctx, T2)
    dt1, dt2 = _lib.as_device(ctx, t1), _lib.as_device(ctx, t2)
    ctx.check(ctx.L.kvft_stanton_residual(ctx.h, 1, nv, no, blk.Fp, blk.Ip, dt1.ptr, dt2.ptr,
                                          float(fac), dT1.ptr, dT2.ptr), "stanton_residual")
    if isinstance(T1, numpy.ndarray):
        dT1.to_host(T1)
        dT2.to_host(T2)
