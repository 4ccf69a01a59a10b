"""The grand potential as a differentiable function of (beta, mu).

``grand_potential(beta, mu, make_system, **options)`` returns Omega(beta, mu)
of the finite-temperature CCSD solve as a 0-dim float64 torch tensor; its
backward pass is the adjoint of the amplitude iteration -- Kelvin's Lambda
equations, the transposed contractions of the residual (kvft_ccsd_lambda),
solved on the device on the forward solve's resident integrals and
amplitudes -- followed by the Lagrangian's explicit derivative
(kelvin/ccsd.py:128-214 compute_ESN with the grid derivative of
1075-1148).  So

    beta = torch.tensor(b, dtype=torch.float64, requires_grad=True)
    mu = torch.tensor(m, dtype=torch.float64, requires_grad=True)
    om = grand_potential(beta, mu, lambda T, mu: systems.ueg_recipe(...), ngrid=16)
    om.backward()
    N = -mu.grad;  E = om + beta dOmega/dbeta + mu N;  S = beta (E - Omega - mu N)

``thermodynamics(...)`` does exactly that and returns (Omega, E, S, N).

Omega(beta, mu) is the function Kelvin differentiates: the orbital energies
stay fixed and the mean-field Fock matrix follows the occupations f(beta, mu)
(the system factory builds the system at T = 1 / beta and mu).  The forward
solve keeps T at every tau point resident in HBM until the backward pass
(2.4 GB of T2 for 66 spin orbitals and 16 points, 27 GB for 114 and 20), so
no tau checkpointing is needed on these configurations; a solve whose
amplitudes do not fit fails at creation with KVFT_ENOMEM.
"""
import torch

from .ccsd import ccsd


class GrandPotential(torch.autograd.Function):
    """Omega(beta, mu); backward by the Lambda (adjoint) equations."""

    @staticmethod
    def forward(ctx, beta, mu, make_system, options):
        b, m = float(beta), float(mu)
        sys = make_system(1.0 / b, m)
        cc = ccsd(sys, T=1.0 / b, mu=m, **options)
        omega = cc.run()[0]
        if any(ctx.needs_input_grad[:2]):
            ctx.cc = cc             # T stays resident until the backward pass
        else:
            cc.release()
            ctx.cc = None
        ctx.omega = omega
        ctx.point = (b, m)
        return torch.tensor(omega, dtype=torch.float64)

    @staticmethod
    def backward(ctx, grad):
        cc = ctx.cc
        b, m = ctx.point
        try:
            dbeta, dmu = omega_gradient(cc, ctx.omega, b, m)
        finally:
            cc.release()
            ctx.cc = None
        g = grad.to(torch.float64)
        return g * dbeta, g * dmu, None, None


def omega_gradient(cc, omega, beta, mu):
    """(dOmega/dbeta, dOmega/dmu) of a solved driver from its Lambda
    equations: compute_ESN(method='lambda') gives N = -dOmega/dmu and
    E = Omega + beta dOmega/dbeta + mu N."""
    E, S, N = cc.compute_ESN(method='lambda')
    return (E - omega - mu * N) / beta, -N


def grand_potential(beta, mu, make_system, **options):
    """Omega(beta, mu) as a differentiable torch scalar (float64).

    beta, mu: 0-dim tensors (or floats); make_system(T, mu) builds the
    system; options are ccsd keywords (ngrid, damp, econv, max_iter,
    precision, ...)."""
    if not torch.is_tensor(beta):
        beta = torch.tensor(float(beta), dtype=torch.float64)
    if not torch.is_tensor(mu):
        mu = torch.tensor(float(mu), dtype=torch.float64)
    return GrandPotential.apply(beta, mu, make_system, options)


def thermodynamics(beta, mu, make_system, **options):
    """(Omega, E, S, N) from one forward solve and its adjoint."""
    b = torch.tensor(float(beta), dtype=torch.float64, requires_grad=True)
    m = torch.tensor(float(mu), dtype=torch.float64, requires_grad=True)
    om = grand_potential(b, m, make_system, **options)
    om.backward()
    Om = float(om.detach())
    N = -float(m.grad)
    E = Om + float(beta) * float(b.grad) + float(mu) * N
    S = float(beta) * (E - Om - float(mu) * N)
    return Om, E, S, N
