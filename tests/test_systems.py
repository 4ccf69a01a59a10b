"""Model-system builders: the closed forms used with device-built integrals
(Fock matrix, first-order energy, exchange shift) against the dense n^4
host formulas, and the device tensors against the host tensors."""
import numpy
import pytest

from kelvin_gb300 import systems

CASES = [
    lambda d: systems.ueg_recipe(14, 4.0, 19, 0.5, device_build=d),
    lambda d: systems.UEGSystem(0.1, 2 * numpy.pi, 1.2, mu=0.1, norb=7, device_build=d),
    lambda d: systems.hubbard_recipe(8, 1.0, 4.0, 2.0, device_build=d),
    lambda d: systems.HubbardRing(0.3, 6, t=1.0, U=2.0, mu=0.4, device_build=d),
]


@pytest.mark.parametrize("make", CASES)
def test_closed_forms_match_dense(make):
    host, dev = make(False), make(True)
    assert numpy.allclose(host.g_energies_tot(), dev.g_energies_tot(), rtol=0, atol=1e-14)
    assert abs(host.mu - dev.mu) < 1e-14 and abs(host.N - dev.N) < 1e-12
    assert abs(host.g_fock_tot() - dev.g_fock_tot()).max() < 1e-14
    assert abs(host.get_mp1() - dev.get_mp1()) < 1e-13 * max(1.0, abs(host.get_mp1()))


@pytest.mark.gpu
@pytest.mark.parametrize("make", CASES)
def test_device_integrals_bit_identical(ctx, make):
    host, dev = make(False), make(True)
    eri = dev.device_aint_tot(ctx).to_host()
    assert numpy.array_equal(eri, host.g_aint_tot())


@pytest.mark.gpu
def test_device_built_solve_matches_host_built(ctx):
    from kelvin_gb300 import ccsd
    kw = dict(max_iter=60, damp=0.5, ngrid=10, econv=1e-11)
    res = []
    for d in (False, True):
        s = systems.ueg_recipe(14, 4.0, 19, 0.5, device_build=d)
        cc = ccsd.ccsd(s, T=s.T, mu=s.mu, ctx=ctx, **kw)
        res.append(cc.run())
        cc.release()
    assert abs(res[0][1] - res[1][1]) < 1e-12
    assert abs(res[0][0] - res[1][0]) < 1e-11


@pytest.mark.parametrize("make", CASES)
def test_builders_are_spin_blocked(make):
    """The solver's spin-block path needs alpha spin orbitals first and every
    integral zero outside the spin-conserving blocks (s_p + s_q = s_r + s_s);
    the UEG and Hubbard builders give exactly that."""
    s = make(False)
    eri, fock = s.g_aint_tot(), s.g_fock_tot()
    n = eri.shape[0]
    assert n % 2 == 0
    sp = (numpy.arange(n) >= n // 2).astype(int)
    cons = (sp[:, None, None, None] + sp[None, :, None, None]
            == sp[None, None, :, None] + sp[None, None, None, :])
    assert not eri[~cons].any()
    assert not fock[sp[:, None] != sp[None, :]].any()
    assert eri[cons].any()
