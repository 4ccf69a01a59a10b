"""Oracle values of the benchmark configurations that the GPU tests compare
against (tests/test_gpu_configs.py), written to configs.json beside this file.

    python tests/golden/make_config_golden.py [ueg38_gl] [hubbard16]

Kelvin has neither a Gauss-Legendre rule nor the Hubbard ring's lattice
package here, so these values come from the oracle (oracle/ft_ccsd.py, a
restatement of Kelvin's FT-CCSD path pinned to Kelvin's own fixtures and
published numbers) on the systems that kelvin_gb300.systems builds:

* ueg38_gl: UEG, 14 electrons, rs = 4, the 19 lowest plane waves (38 spin
  orbitals), Theta = 0.5, ng = 10 Gauss-Legendre points, damping 0.5, econv
  1e-10: Omega_cc and Omega;
* hubbard16: the half-filled 16-site ring, t = 1, U = 4, mean-field momentum
  basis (e_k = -2 cos(2 pi k / 16) + U/2, mu = U/2), ng = 40, beta = 1:
  Omega_cc and Omega, and E, S, N from the oracle's Lambda equations.  At
  beta = 4 and 10 the damped iteration of this ring diverges (damping 0.5,
  0.8 and 0.9 alike), so there is no value to record.

CPU only; minutes per entry.
"""
import json
import os
import sys
import time

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

OUT = os.path.join(HERE, "configs.json")

HUBBARD = {"ngrid": 40, "damp": 0.5, "max_iter": 200, "econv": 1e-10}


def ueg38_gl():
    from kelvin_gb300 import systems
    from oracle import ft_ccsd
    s = systems.ueg_recipe(14, 4.0, 19, 0.5)
    t0 = time.time()
    om, occ = ft_ccsd.ft_ccsd(s.g_energies_tot(), s.g_fock_tot(), s.g_aint_tot(), s.T, s.mu,
                              ngrid=10, quad='gl', econv=1e-10, max_iter=100, damp=0.5,
                              E_const=s.const_energy(), E1=s.get_mp1())
    return {"ngrid": 10, "damp": 0.5, "econv": 1e-10, "omega_cc": float(occ),
            "omega": float(om), "cpu_s": time.time() - t0}


def hubbard16(beta):
    import numpy
    from kelvin_gb300 import systems
    from oracle import ft_lambda
    h = systems.hubbard_mf_recipe(16, 1.0, 4.0, beta)
    en, eri = h.g_energies_tot(), h.g_aint_tot()
    hcore = numpy.diag(numpy.hstack((h.ek, h.ek)))
    t0 = time.time()
    hist = []
    E, S, N, Om, T1, T2, L1, L2 = ft_lambda.solve(
        en, hcore, eri, h.T, h.mu, ngrid=HUBBARD["ngrid"], damp=HUBBARD["damp"],
        econv=HUBBARD["econv"], max_iter=HUBBARD["max_iter"], lconv=1e-9, history=hist)
    from oracle import ft_ccsd, quadrature
    beta_ = 1.0 / h.T
    ti, g, G = quadrature.ft_quad(HUBBARD["ngrid"], beta_, 'lin')
    F, I = ft_ccsd.ft_integrals(h.g_fock_tot(), eri, en, beta_, h.mu)
    occ = ft_ccsd.ft_cc_energy(T1, T2, F.ov, I.oovv, g, beta_)
    return dict(HUBBARD, beta=beta, omega_cc=float(occ), omega=float(Om), E=float(E),
                S=float(S), N=float(N), lambda_iterations=len(hist), cpu_s=time.time() - t0)


def main():
    want = sys.argv[1:] or ["ueg38_gl", "hubbard16"]
    out = json.load(open(OUT)) if os.path.exists(OUT) else {}
    if "ueg38_gl" in want:
        out["ueg38_gl"] = ueg38_gl()
        print("ueg38_gl", out["ueg38_gl"], flush=True)
    if "hubbard16" in want:
        out.setdefault("hubbard16", {})
        for beta in (1.0,):
            out["hubbard16"]["%g" % beta] = hubbard16(beta)
            print("hubbard16", beta, out["hubbard16"]["%g" % beta], flush=True)
            json.dump(out, open(OUT, "w"), indent=1, sort_keys=True)
    json.dump(out, open(OUT, "w"), indent=1, sort_keys=True)


if __name__ == "__main__":
    main()
