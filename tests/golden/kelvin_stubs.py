"""Stand-ins that let Kelvin's own modules import in a container without its
external dependencies (pyscf, cqcpy).  Used only by make_golden.py, which runs
Kelvin's unmodified Python to produce the fixtures in this folder.

* ``pyscf.lib.einsum``  -> ``numpy.einsum`` (the only pyscf use on the path);
* ``cqcpy.ft_utils``, ``cqcpy.utils``, ``cqcpy.ov_blocks`` -> the oracle's
  restatements from their definitions;
* ``cqcpy.cc_equations._Stanton`` -> the oracle's restated Stanton-Gauss
  residual (checked separately against an exact Fock-space projection).
"""
import sys
import types

import numpy


def install(reference_root):
    from oracle import cc_equations, ft_utils

    def mod(name, **attrs):
        m = types.ModuleType(name)
        for k, v in attrs.items():
            setattr(m, k, v)
        sys.modules[name] = m
        return m

    lib = mod("pyscf.lib", einsum=numpy.einsum)
    mod("pyscf", lib=lib)

    def block_diag(A, B):
        out = numpy.zeros((A.shape[0] + B.shape[0], A.shape[1] + B.shape[1]))
        out[:A.shape[0], :A.shape[1]] = A
        out[A.shape[0]:, A.shape[1]:] = B
        return out

    def _unused(*a, **k):
        raise NotImplementedError("not on the FT-CCSD path")

    ftu = mod("cqcpy.ft_utils", ff=ft_utils.ff, ffv=ft_utils.ffv,
              GP0=ft_utils.GP0, HtoK=ft_utils.HtoK, dGP0=_unused, uGP0=_unused)
    utl = mod("cqcpy.utils", D1=ft_utils.D1, D2=ft_utils.D2,
              block_diag=block_diag)
    ovb = mod("cqcpy.ov_blocks", one_e_blocks=ft_utils.one_e_blocks,
              two_e_blocks=ft_utils.two_e_blocks,
              two_e_blocks_full=ft_utils.two_e_blocks)
    cce = mod("cqcpy.cc_equations", _Stanton=cc_equations.stanton)
    cen = mod("cqcpy.cc_energy", cc_energy_d=_unused, cc_energy_s1=_unused)
    mod("cqcpy", ft_utils=ftu, utils=utl, ov_blocks=ovb, cc_equations=cce,
        cc_energy=cen)
    if reference_root not in sys.path:
        sys.path.insert(0, reference_root)
