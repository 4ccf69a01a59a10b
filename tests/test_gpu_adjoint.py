"""dOmega/dbeta and dOmega/dmu through torch.autograd (kelvin_gb300.adjoint):
the backward pass is the Lambda equations on the device.  Checked against
central differences of Omega (dbeta = 1e-4 beta, dmu = 1e-5) and, through
E, S, N, against Kelvin's published Lambda-based properties of the
19-plane-wave UEG (examples/ueg_ft_ccsd_ESN.out:43-45)."""
import json
import os

import numpy
import pytest

from conftest import GOLDEN
from kelvin_gb300 import _lib, systems

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


def _ueg(norb):
    return lambda T, mu: systems.UEGSystem(T, 2 * numpy.pi, 1.2, mu=mu, norb=norb)


def test_adjoint_vs_central_differences(ctx):
    from kelvin_gb300 import adjoint
    T, mu = 0.1, 0.1
    beta = 1.0 / T
    opts = dict(ngrid=10, damp=0.2, econv=1e-12, max_iter=200, precision="fp64_tc", ctx=ctx)
    try:
        b = torch.tensor(beta, dtype=torch.float64, requires_grad=True)
        m = torch.tensor(mu, dtype=torch.float64, requires_grad=True)
        om = adjoint.grand_potential(b, m, _ueg(7), **opts)
        om.backward()
        db, dm = 1e-4 * beta, 1e-5

        def f(bb, mm):
            return float(adjoint.grand_potential(bb, mm, _ueg(7), **opts).detach())
        fd_b = (f(beta + db, mu) - f(beta - db, mu)) / (2 * db)
        fd_m = (f(beta, mu + dm) - f(beta, mu - dm)) / (2 * dm)
    finally:
        ctx.set_precision(_lib.PREC_FP64, 7)
    assert abs(float(b.grad) - fd_b) < 1e-7 * max(1.0, abs(fd_b))
    assert abs(float(m.grad) - fd_m) < 1e-7 * max(1.0, abs(fd_m))


def test_adjoint_ueg19_vs_kelvin(ctx):
    from kelvin_gb300 import adjoint
    meta = json.load(open(os.path.join(GOLDEN, "ueg19_esn.json")))
    T, mu = meta["T"], meta["mu"]
    try:
        Om, E, S, N = adjoint.thermodynamics(
            1.0 / T, mu, _ueg(meta["norb"]), ngrid=meta["ngrid"], damp=meta["damp"],
            econv=1e-11, max_iter=100, precision="fp64_tc", ctx=ctx)
    finally:
        ctx.set_precision(_lib.PREC_FP64, 7)
    # Kelvin converged T to 1e-8 and Lambda to 1e-5
    assert abs(E - meta["E"]) < 2e-6
    assert abs(S - meta["S"]) < 2e-5
    assert abs(N - meta["N"]) < 2e-6
    assert abs(Om - (E - T * S - mu * N)) < 1e-9
