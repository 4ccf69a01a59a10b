"""Host-side logic of the product (no GPU): tau grids, system builders, the
C ABI of libkvft.so (it loads and exports every symbol include/kvft.h
declares)."""
import ctypes
import json
import os
import re

import numpy
import pytest

from conftest import GOLDEN, ROOT, golden
from kelvin_gb300 import quadrature, systems
from oracle import quadrature as oq
from oracle import systems as osys


def test_grids_match_kelvin():
    d = golden("quad_grids.npz")
    for k in d.files:
        if not k.endswith("_ti"):
            continue
        base = k[:-3]
        rule, ng, beta = base.split("_")
        ti, g, G = quadrature.ft_quad(int(ng), float(beta), rule)
        assert abs(ti - d[base + "_ti"]).max() < 1e-13, base
        assert abs(g - d[base + "_g"]).max() < 1e-13, base
        assert abs(G - d[base + "_G"]).max() < 1e-13, base
        if base + "_gd" in d.files:
            gd, Gd = quadrature.d_ft_quad(int(ng), float(beta), rule)
            assert abs(gd - d[base + "_gd"]).max() < 1e-13, base
            assert abs(Gd - d[base + "_Gd"]).max() < 1e-13, base


def test_unknown_rule_raises():
    with pytest.raises(Exception):
        quadrature.ft_quad(10, 1.0, "nope")


@pytest.mark.parametrize("ng", [4, 7, 10])
def test_gauss_legendre_rule(ng):
    beta = 3.0
    ti, g, G = quadrature.ft_quad(ng, beta, "gl")
    ti2, g2, G2 = oq.gauss_legendre(ng, beta)
    assert abs(G - G2).max() < 1e-13
    # exact for polynomials of degree < ng: cumulative integral of t^k
    for k in range(ng):
        assert abs(G @ ti ** k - ti ** (k + 1) / (k + 1)).max() < 1e-11 * beta ** (k + 1)
    assert abs(g.sum() - beta) < 1e-13


def test_ueg_builders_match_kelvin():
    d = golden("ueg7.npz")
    s = systems.UEGSystem(0.1, 2 * numpy.pi, 1.2, mu=0.1, norb=7)
    assert abs(s.g_aint_tot() - d["eri"]).max() == 0.0
    assert abs(s.g_energies_tot() - d["eps"]).max() == 0.0
    assert abs(s.g_fock_tot() - d["fock"]).max() < 1e-15
    d = golden("uegscf7.npz")
    s = systems.UEGSystem(0.1, 2 * numpy.pi, 1.2, mu=0.1182817, norb=7, hf_shift=True)
    assert abs(s.g_aint_tot() - d["eri"]).max() == 0.0
    assert abs(s.g_energies_tot() - d["eps"]).max() < 1e-15
    assert abs(s.g_fock_tot() - d["fock"]).max() < 1e-15


def test_ueg_builder_matches_loop_builder():
    L = 2 * numpy.pi
    b = osys.UEGBasis(L, 3.0, norb=11)
    s = systems.UEGSystem(0.1, L, 3.0, mu=0.1, norb=11)
    assert numpy.array_equal(numpy.array(b.basis), s.nvec)
    assert abs(osys.g2e_loop(b) - s.g_aint_tot()).max() == 0.0


@pytest.mark.parametrize("args", [(14, 4.0, 19, 0.5), (38, 1.0, 57, 0.25), (14, 2.0, 33, 0.5)])
def test_ueg_recipe_fills_N(args):
    s = systems.ueg_recipe(*args)
    assert s.nb == args[2]
    assert abs(s.N - args[0]) < 1e-9


def test_hubbard_ring_integrals():
    h = systems.hubbard_recipe(6, 1.0, 4.0, 2.0)
    g = h.g_aint_tot()
    assert abs(g + g.transpose(1, 0, 2, 3)).max() == 0.0
    assert abs(g + g.transpose(0, 1, 3, 2)).max() == 0.0
    assert abs(g - g.transpose(2, 3, 0, 1)).max() == 0.0
    assert abs(h.N - 6.0) < 1e-12          # half filling at mu = 0
    # site-basis check: the momentum integrals are the Fourier transform of U n_up n_dn
    L, U = 6, 4.0
    k = numpy.arange(L)
    phi = numpy.exp(2j * numpy.pi * numpy.outer(numpy.arange(L), k) / L) / numpy.sqrt(L)
    Vk = U * numpy.einsum('ja,jb,jc,jd->abcd', phi.conj(), phi.conj(), phi, phi)
    assert abs(Vk.imag).max() < 1e-12
    assert abs(g[:L, L:, :L, L:] - Vk.real).max() < 1e-12


def _declared_symbols():
    txt = open(os.path.join(ROOT, "include", "kvft.h")).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    return sorted(set(re.findall(r"\b(kvft_[a-z0-9_]+)\s*\(", txt)))


def test_library_exports_declared_symbols():
    from kelvin_gb300 import _lib
    L = _lib.lib()
    declared = _declared_symbols()
    assert len(declared) >= 30
    for name in declared:
        assert hasattr(L, name), name
    # every declared entry point has a ctypes signature in the binding
    assert set(declared) <= set(_lib.exported_symbols())


def test_library_status_strings_without_gpu():
    from kelvin_gb300 import _lib
    L = _lib.lib()
    assert L.kvft_status_string(0) == b"ok"
    assert L.kvft_status_string(6) == b"not converged"
    assert L.kvft_solver_footprint(38, 10, 0) > 8 * 38 ** 4 * 10


@pytest.mark.parametrize("device_build", [False, True])
def test_hf_shifted_first_order_energy(device_build):
    """With HF-shifted orbital energies the first-order grand potential has
    Kelvin's sum_i (h_ii - e_i) f_i term (ueg_scf_system.py:146-157): E1 and
    Omega equal the UEGSCFSystem values of examples/ueg_ft_cc_compare."""
    meta = json.load(open(os.path.join(GOLDEN, "uegscf7.json")))
    s = systems.UEGSystem(meta["T"], meta["L"], meta["cutoff"], mu=meta["mu"], norb=7,
                          hf_shift=True, device_build=device_build)
    E0 = systems.grand_potential0(1.0 / meta["T"], s.g_energies_tot(), meta["mu"]) \
        + s.const_energy()
    assert abs(s.get_mp1() - meta["G1"]) < 1e-15
    assert abs(E0 + s.get_mp1() + meta["Omega_cc"] - meta["Omega_total"]) < 1e-14
