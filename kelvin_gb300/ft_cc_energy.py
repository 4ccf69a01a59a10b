"""FT-CC grand potential on the GPU, drop-in for kelvin/ft_cc_energy.py.

Omega_cc = (1/beta) [ sum_ai t1n f_ia + sum_abij t2n I_ijab ],
t1n = sum_y g_y T1_y, t2n = sum_y g_y (T2_y/4 + [Qterm] T1_y T1_y / 2)
(ft_cc_energy.py:7-32), reduced in a fixed order on the device.
"""
import ctypes

from . import _lib


def ft_cc_energy(T1, T2, f, eri, g, beta, Qterm=True, ctx=None):
    """Return the FT-CC free-energy correction (a Python float)."""
    ctx = ctx or _lib.context()
    ng, nv, no = T1.shape
    if tuple(T2.shape) != (ng, nv, nv, no, no):
        raise Exception("ft_cc_energy: T2 shape does not match T1")
    d1, d2, df, de, dg = (_lib.as_device(ctx, a) for a in (T1, T2, f, eri, g))
    out = ctypes.c_double()
    ctx.check(ctx.L.kvft_ft_cc_energy(ctx.h, ng, nv, no, d1.ptr, d2.ptr, df.ptr, de.ptr,
                                      dg.ptr, float(beta), int(bool(Qterm)),
                                      ctypes.byref(out)), "ft_cc_energy")
    return float(out.value)
