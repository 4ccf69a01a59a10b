"""Host logic of the autograd adjoint (kelvin_gb300.adjoint) with a fake
driver: the gradient it returns is assembled from E, S, N as
dOmega/dmu = -N and dOmega/dbeta = (E - Omega - mu N) / beta."""
import pytest

torch = pytest.importorskip("torch")


class FakeCC(object):
    """Omega(beta, mu) = beta^2 mu + 3 mu + 1 / beta, with the E, S, N that
    Kelvin's relations give for it."""
    released = 0

    def __init__(self, sys, T, mu, **kw):
        self.b, self.m = 1.0 / T, mu

    def omega(self):
        b, m = self.b, self.m
        return b * b * m + 3.0 * m + 1.0 / b

    def run(self):
        return self.omega(), 0.0

    def compute_ESN(self, method='fd'):
        assert method == 'lambda'
        b, m = self.b, self.m
        dOb, dOm = 2.0 * b * m - 1.0 / (b * b), b * b + 3.0
        N = -dOm
        E = self.omega() + b * dOb + m * N
        S = b * (E - self.omega() - m * N)
        return E, S, N

    def release(self):
        FakeCC.released += 1


def test_gradient_from_esn(monkeypatch):
    from kelvin_gb300 import adjoint
    monkeypatch.setattr(adjoint, "ccsd", FakeCC)
    b = torch.tensor(2.0, dtype=torch.float64, requires_grad=True)
    m = torch.tensor(0.3, dtype=torch.float64, requires_grad=True)
    om = adjoint.grand_potential(b, m, lambda T, mu: None)
    (2.0 * om).backward()
    assert abs(float(om.detach()) - (4.0 * 0.3 + 0.9 + 0.5)) < 1e-14
    assert abs(float(b.grad) - 2.0 * (2.0 * 2.0 * 0.3 - 0.25)) < 1e-13
    assert abs(float(m.grad) - 2.0 * (4.0 + 3.0)) < 1e-13
    assert FakeCC.released == 1
    Om, E, S, N = adjoint.thermodynamics(2.0, 0.3, lambda T, mu: None)
    ref = FakeCC(None, 0.5, 0.3)
    E0, S0, N0 = ref.compute_ESN('lambda')
    assert abs(E - E0) < 1e-13 and abs(S - S0) < 1e-12 and abs(N - N0) < 1e-13
