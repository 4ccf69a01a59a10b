"""CPU oracle for the FT-CCSD amplitude iteration (TEST INFRASTRUCTURE ONLY).

This package is a plain numpy (FP64) restatement of Kelvin's finite-temperature
CCSD hot path (awhite862/kelvin):

* ``quadrature``   -- kelvin/quadrature.py: tau grids, weights and the
                      exp-weighted cumulative time integrals;
* ``ft_utils``     -- the Fermi-Dirac helpers Kelvin imports from cqcpy
                      (restated from their textbook definitions);
* ``cc_equations`` -- the Stanton-Gauss spin-orbital CCSD residual Kelvin
                      imports as ``cqcpy.cc_equations._Stanton`` (restated from
                      J. F. Stanton, J. Gauss, J. D. Watts, R. J. Bartlett,
                      J. Chem. Phys. 94, 4334 (1991));
* ``ft_ccsd``      -- kelvin/ft_cc_equations.py, kelvin/ft_cc_energy.py,
                      kelvin/cc_utils.py and kelvin/ccsd.py (FT general-spin
                      driver);
* ``ft_lambda``    -- the Lambda iteration (kelvin/ft_cc_equations.py:385-512,
                      kelvin/cc_utils.py:414-560), E, S, N
                      (kelvin/ccsd.py:167-214, 1075-1148) and the response
                      densities / normal-ordered RDMs
                      (kelvin/ft_cc_equations.py:704-753,
                      kelvin/cc_utils.py:1449-1466); the Lambda terms cqcpy
                      supplies are restated as the exact transpose of the
                      residual's Jacobian;
* ``systems``      -- kelvin/ueg_utils.py, kelvin/ueg_system.py,
                      kelvin/ueg_scf_system.py (loop builders, small n) and a
                      Hubbard-ring model in the momentum basis.

Only ``tests/``, ``__graft_entry__.smoke()`` and ``bench.py``'s CPU-baseline
leg may import it, and only as the checker or the timed CPU reference.  The
product package ``kelvin_gb300`` never imports it.

Parity pins: the restatement reproduces Kelvin's golden grand potentials
(kelvin/tests/test_ft_ccsd.py:23 -- UEG, 7 plane waves, -0.010750238811 --
and examples/ueg_ft_ccsd2.out:25 -- 19 plane waves, -0.015646626108), and the
Stanton residual equals the exact projection <mu| exp(-T) H exp(T) |0> built
from second-quantised operators in a small Fock space (tests/test_oracle.py).
The Lambda restatement reproduces Kelvin's published Lambda run for 19 plane
waves (examples/ueg_ft_ccsd_ESN.out: all 14 printed residuals to their last
digit, E, S and N to 3e-14) and finite differences of the grand potential
(tests/test_lambda.py).
"""
