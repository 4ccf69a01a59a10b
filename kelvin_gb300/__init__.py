"""kelvin_gb300 -- GB300-native finite-temperature CCSD amplitude iteration.

Drop-in GPU versions of Kelvin's hot-path modules:

    kelvin_gb300.quadrature      (kelvin/quadrature.py)
    kelvin_gb300.ft_cc_equations (kelvin/ft_cc_equations.py: ccsd_stanton)
    kelvin_gb300.ft_cc_energy    (kelvin/ft_cc_energy.py)
    kelvin_gb300.cc_utils        (kelvin/cc_utils.py: ft_integrals, ft_cc_iter)
    kelvin_gb300.ccsd            (kelvin/ccsd.py: the FT driver)

All arithmetic on the path runs in libkvft.so (hand-written sm_103a CUDA,
C ABI in include/kvft.h).  Importing the package does not need a GPU; the
first call does, and fails loudly without the library or a device.
"""
__all__ = ["quadrature", "ft_cc_equations", "ft_cc_energy", "cc_utils", "ccsd",
           "systems"]
