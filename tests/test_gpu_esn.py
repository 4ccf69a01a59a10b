"""Energy, entropy and particle number (ccsd.compute_ESN) from central finite
differences of the converged grand potential, against Kelvin's own output
for the 19-plane-wave UEG (examples/ueg_ft_ccsd_ESN.out:43-45; Kelvin takes
them from its Lambda equations, converged there to a residual of ~1e-5)."""
import numpy
import pytest

from kelvin_gb300 import _lib, ccsd, systems

pytestmark = pytest.mark.gpu


def test_esn_ueg19_vs_kelvin(ctx):
    s = systems.UEGSystem(0.1, 2 * numpy.pi, 1.2, mu=0.1, norb=19)
    cc = ccsd.ccsd(s, T=0.1, mu=0.1, max_iter=100, damp=0.2, ngrid=10, econv=1e-11,
                   precision="fp64_tc", ctx=ctx)
    try:
        cc.run()
        E, S, N = cc.compute_ESN()
    finally:
        ctx.set_precision(_lib.PREC_FP64, 7)      # the context is shared by the tests
    assert abs(E - 0.16054077292256178) < 2e-5
    assert abs(S - 2.7712932131425982) < 2e-4
    assert abs(N - 1.9206450717478192) < 2e-5
    # thermodynamic consistency of the three with Omega
    assert abs(cc.Gtot - (E - 0.1 * S - 0.1 * N)) < 1e-6
