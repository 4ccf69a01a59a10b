"""The CPU oracle against Kelvin's own outputs (golden fixtures) and an exact
second-quantised residual.  CPU only."""
import json
import os

import numpy
import pytest

from conftest import GOLDEN, golden, random_system, random_T, unpack_blocks
from oracle import cc_equations, fock_space, ft_ccsd, quadrature, systems


def test_grids_match_kelvin():
    d = golden("quad_grids.npz")
    for k in d.files:
        if not k.endswith("_ti"):
            continue
        base = k[:-3]
        rule, ng, beta = base.split("_")
        ti, g, G = quadrature.ft_quad(int(ng), float(beta), rule)
        assert numpy.allclose(ti, d[base + "_ti"], rtol=0, atol=1e-13), base
        assert numpy.allclose(g, d[base + "_g"], rtol=0, atol=1e-13), base
        assert numpy.allclose(G, d[base + "_G"], rtol=0, atol=1e-13), base


@pytest.mark.parametrize("tag", ["sq", "rect", "mid"])
def test_int_tbar_match_kelvin(tag):
    d = golden("int_tbar.npz")
    ti, G = d[tag + "_ti"], d[tag + "_G"]
    ng = ti.shape[0]
    T1 = quadrature.int_tbar1(ng, d[tag + "_t1bar"], ti, d[tag + "_D1"], G)
    T2 = quadrature.int_tbar2(ng, d[tag + "_t2bar"], ti, d[tag + "_D2"], G)
    assert abs(T1 - d[tag + "_T1"]).max() < 1e-14
    assert abs(T2 - d[tag + "_T2"]).max() < 1e-14
    ig = ng - 2
    s1 = quadrature.int_tbar1_single(ng, ig, d[tag + "_t1bar"], ti, d[tag + "_D1"], G)
    assert abs(s1 - d[tag + "_T1single"]).max() < 1e-14
    L1 = quadrature.int_L1(ng, d[tag + "_L1old"], ti, d[tag + "_D1"], d[tag + "_g"], G)
    L2 = quadrature.int_L2(ng, d[tag + "_L2old"], ti, d[tag + "_D2"], d[tag + "_g"], G)
    assert abs(L1 - d[tag + "_L1"]).max() < 1e-13
    assert abs(L2 - d[tag + "_L2"]).max() < 1e-13


def test_energy_match_kelvin():
    d = golden("energy.npz")
    for q, key in ((True, "E_q"), (False, "E_noq")):
        E = ft_ccsd.ft_cc_energy(d["T1"], d["T2"], d["f"], d["eri"], d["g"], float(d["beta"]), q)
        assert abs(E - float(d[key])) < 1e-13


@pytest.mark.parametrize("prefix", ["ft_", "rb_"])
def test_ccsd_stanton_match_kelvin(prefix):
    d = golden("stanton.npz")
    F, I = unpack_blocks(d, prefix)
    ti, G = d[prefix + "ti"], d[prefix + "G"]
    T1, T2 = ft_ccsd.ccsd_stanton(F, I, d[prefix + "t1"], d[prefix + "t2"], d[prefix + "D1"],
                                  d[prefix + "D2"], ti, ti.shape[0], G)
    assert abs(T1 - d[prefix + "T1"]).max() < 1e-13
    assert abs(T2 - d[prefix + "T2"]).max() < 1e-13


@pytest.mark.parametrize("no,nv,seed", [(2, 3, 1), (3, 4, 2), (4, 3, 3)])
def test_stanton_equals_exact_projection(no, nv, seed):
    """The restated Stanton-Gauss residual equals <mu|exp(-T) H exp(T)|0>."""
    rng = numpy.random.default_rng(seed)
    F, I = random_system(rng, no, nv)
    t1, t2 = random_T(rng, 1, nv, no, 0.2)
    R1e, R2e = fock_space.exact_residual(F, I, t1[0], t2[0])
    R1, R2 = cc_equations.residual(F, I, t1[0], t2[0])
    assert abs(R1 + F.vo - R1e).max() < 1e-12
    assert abs(R2 + I.vvoo - R2e).max() < 1e-12


def test_ueg_golden_omega():
    """Kelvin test_ft_ccsd.py:119-133: UEG, 7 plane waves, -0.010750238811."""
    meta = json.load(open(os.path.join(GOLDEN, "ueg7.json")))
    b = systems.UEGBasis(meta["L"], meta["cutoff"], norb=meta["norb"])
    eri = systems.g2e_loop(b)
    en = systems.ueg_g_energies(b)
    fock = systems.g_fock_tot(b, eri, en, meta["T"], meta["mu"])
    E1 = systems.get_mp1(eri, en, meta["T"], meta["mu"])
    d = golden("ueg7.npz")
    assert abs(eri - d["eri"]).max() == 0.0
    hist = []
    Et, Ecc = ft_ccsd.ft_ccsd(en, fock, eri, meta["T"], meta["mu"], ngrid=10,
                              damp=meta["damp"], max_iter=50, E1=E1, history=hist)
    assert abs(Ecc - meta["kelvin_test_golden"]) < 1e-9
    assert abs(Ecc - meta["Omega_cc"]) < 1e-12
    assert abs(Et - meta["Omega_total"]) < 1e-12
    assert len(hist) == len(meta["iterations"])


def _hubbard_atom(eps=0.0, U=1.0):
    """One site, two spin orbitals: h = eps, <01||01> = U."""
    h = numpy.diag([eps, eps])
    eri = numpy.zeros((2, 2, 2, 2))
    eri[0, 1, 0, 1] = eri[1, 0, 1, 0] = U
    eri[0, 1, 1, 0] = eri[1, 0, 0, 1] = -U
    return h, eri


def test_ft_ccsd_exact_for_two_spin_orbitals():
    """FT-CCSD is exact for two spin orbitals as the grid is refined
    (kelvin/tests/test_ft_ccsd.py:26-47 compares with FT-FCI at ng = 200 to
    1e-9).  The exact grand potential comes from diagonalising H - mu N in the
    Fock space and equals the Hubbard atom's closed form."""
    from oracle import ft_lambda, ft_utils
    eps, U, T, mu = 0.0, 1.0, 1.0, 0.3
    h, eri = _hubbard_atom(eps, U)
    exact = fock_space.grand_potential(h, eri, T, mu)
    b = 1.0 / T
    closed = -T * numpy.log(1 + 2 * numpy.exp(-b * (eps - mu))
                            + numpy.exp(-b * (2 * eps + U - 2 * mu)))
    assert abs(exact - closed) < 1e-14
    err = {}
    for label, en in (("bare", numpy.diag(h).copy()), ("shifted", numpy.diag(h) + 0.5 * U)):
        fock = ft_lambda.mean_field(h, eri, ft_utils.ff(b, en, mu))
        E1 = ft_lambda.omega_ref(en, h, eri, b, mu)[1]
        for ng in (100, 200):
            Et = ft_ccsd.ft_ccsd(en, fock, eri, T, mu, ngrid=ng, econv=1e-11, max_iter=24,
                                 E1=E1)[0]
            err[label, ng] = abs(Et - exact)
    assert err["shifted", 200] < 1e-10 and err["bare", 200] < 2e-9
    # third-order convergence in the grid spacing (Simpson weights)
    assert 6.0 < err["bare", 100] / err["bare", 200] < 10.0
