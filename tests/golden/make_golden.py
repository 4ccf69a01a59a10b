"""Generate the golden fixtures in this folder by running Kelvin's own code.

Usage (needs a read-only Kelvin checkout; never run on the GPU host):

    python tests/golden/make_golden.py <path of the Kelvin checkout>

Kelvin's modules are imported unmodified; its absent dependencies are
replaced by ``kelvin_stubs`` (numpy einsum for pyscf, the oracle's
restatements for cqcpy).  Outputs (all small, seeded):

* quad_grids.npz   -- quadrature.ft_quad / d_ft_quad for every rule
* int_tbar.npz     -- quadrature.int_tbar1/2, *_single and int_L1/L2 on
                      seeded random inputs (square and non-square blocks)
* energy.npz       -- ft_cc_energy.ft_cc_energy (Qterm on/off)
* stanton.npz      -- ft_cc_equations.ccsd_stanton on two seeded inputs
* ueg7.npz / ueg7.json -- UEGSystem(T=0.1, L=2pi, cutoff 1.2, mu=0.1,
                      norb=7, 'g') integrals and the full ccsd(...).run()
                      (Kelvin test_ft_ccsd.py:119-133 golden -0.010750238811)
* uegscf7.json     -- UEGSCFSystem at ng=40 (examples/ueg_ft_cc_compare.py)
* ueg19_esn.json   -- Kelvin's published Lambda run, read from the text of
                      examples/ueg_ft_ccsd_ESN.py (settings) and
                      examples/ueg_ft_ccsd_ESN.out (Omega, the Lambda
                      residual per iteration, E, S, N); nothing is executed
                      (``--esn-only`` writes just this file)
"""
import json
import logging
import os
import sys

import numpy

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, HERE)


def rand_antisym(rng, n, scale):
    g = rng.standard_normal((n, n, n, n)) * scale
    g = g - g.transpose(1, 0, 2, 3)
    return g - g.transpose(0, 1, 3, 2)


def blocks_from_full(f, g, no, nv):
    from oracle.ft_utils import one_e_blocks, two_e_blocks
    o, v = slice(0, no), slice(no, no + nv)
    F = one_e_blocks(f[o, o], f[o, v], f[v, o], f[v, v])
    sl = {'o': o, 'v': v}
    I = two_e_blocks(**{nm: g[tuple(sl[c] for c in nm)].copy()
                        for nm in two_e_blocks.NAMES})
    return F, I


def rand_T(rng, ng, nv, no, scale):
    T1 = rng.standard_normal((ng, nv, no)) * scale
    T2 = rng.standard_normal((ng, nv, nv, no, no)) * scale
    T2 = T2 - T2.transpose(0, 2, 1, 3, 4)
    T2 = T2 - T2.transpose(0, 1, 2, 4, 3)
    return T1, T2


def pack_blocks(prefix, F, I):
    out = {}
    for b in ('oo', 'ov', 'vo', 'vv'):
        out[prefix + 'F_' + b] = getattr(F, b)
    for b in I.NAMES:
        out[prefix + 'I_' + b] = getattr(I, b)
    return out


def main(ref_root):
    import kelvin_stubs
    kelvin_stubs.install(ref_root)
    from kelvin import quadrature, ft_cc_energy, ft_cc_equations
    from kelvin.ccsd import ccsd
    from kelvin.ueg_system import UEGSystem
    from kelvin.ueg_scf_system import UEGSCFSystem
    from oracle import ft_ccsd as oft

    # ---- quadrature grids -------------------------------------------------
    grids = {}
    for rule in ('lin', 'ln', 'sin', 'exp', 'quad', 'cub', 'quar', 'mid', 'L'):
        for ng in (5, 10, 11):
            for beta in (2.0, 10.0):
                ti, g, G = quadrature.ft_quad(ng, beta, rule)
                key = "%s_%d_%g" % (rule, ng, beta)
                grids[key + "_ti"] = ti
                grids[key + "_g"] = g
                grids[key + "_G"] = G
                if rule != 'mid':
                    gd, Gd = quadrature.d_ft_quad(ng, beta, rule)
                    grids[key + "_gd"] = gd
                    grids[key + "_Gd"] = Gd
    numpy.savez_compressed(os.path.join(HERE, "quad_grids.npz"), **grids)

    # ---- int_tbar / int_L -------------------------------------------------
    rng = numpy.random.default_rng(20240601)
    it = {}
    for tag, (nv, no, ng, beta, rule) in {
            'sq': (5, 5, 6, 2.0, 'lin'), 'rect': (4, 3, 7, 3.0, 'sin'),
            'mid': (3, 3, 5, 1.5, 'mid')}.items():
        ti, g, G = quadrature.ft_quad(ng, beta, rule)
        ev = rng.standard_normal(nv)
        eo = rng.standard_normal(no)
        D1 = ev[:, None] - eo[None, :]
        D2 = (ev[:, None, None, None] + ev[None, :, None, None]
              - eo[None, None, :, None] - eo[None, None, None, :])
        t1b, t2b = rand_T(rng, ng, nv, no, 0.1)
        L1o = rng.standard_normal((ng, no, nv)) * 0.1
        L2o = rng.standard_normal((ng, no, no, nv, nv)) * 0.1
        it.update({tag + "_ti": ti, tag + "_g": g, tag + "_G": G,
                   tag + "_D1": D1, tag + "_D2": D2,
                   tag + "_t1bar": t1b, tag + "_t2bar": t2b,
                   tag + "_L1old": L1o, tag + "_L2old": L2o})
        it[tag + "_T1"] = quadrature.int_tbar1(ng, t1b, ti, D1, G)
        it[tag + "_T2"] = quadrature.int_tbar2(ng, t2b, ti, D2, G)
        ig = ng - 2
        it[tag + "_T1single"] = quadrature.int_tbar1_single(ng, ig, t1b, ti, D1, G)
        it[tag + "_T2single"] = quadrature.int_tbar2_single(ng, ig, t2b, ti, D2, G)
        it[tag + "_L1"] = quadrature.int_L1(ng, L1o, ti, D1, g, G)
        it[tag + "_L2"] = quadrature.int_L2(ng, L2o, ti, D2, g, G)
    numpy.savez_compressed(os.path.join(HERE, "int_tbar.npz"), **it)

    # ---- ft_cc_energy -----------------------------------------------------
    en = {}
    nv, no, ng = 5, 4, 6
    T1, T2 = rand_T(rng, ng, nv, no, 0.1)
    f = rng.standard_normal((no, nv))
    eri = rng.standard_normal((no, no, nv, nv))
    ti, g, G = quadrature.simpsons(ng, 2.5)
    en.update(T1=T1, T2=T2, f=f, eri=eri, g=g, beta=2.5)
    en["E_q"] = ft_cc_energy.ft_cc_energy(T1, T2, f, eri, g, 2.5, Qterm=True)
    en["E_noq"] = ft_cc_energy.ft_cc_energy(T1, T2, f, eri, g, 2.5, Qterm=False)
    numpy.savez_compressed(os.path.join(HERE, "energy.npz"), **en)

    # ---- ccsd_stanton -----------------------------------------------------
    st = {}
    # (a) FT-structured: one n-orbital system scaled by Fermi factors
    n, ng, beta, mu = 6, 5, 2.0, 0.1
    e = numpy.sort(rng.standard_normal(n))
    h = rng.standard_normal((n, n)) * 0.1
    fock = numpy.diag(e) + 0.5 * (h + h.T)
    g4 = rand_antisym(rng, n, 0.1)
    g4 = 0.5 * (g4 + g4.transpose(2, 3, 0, 1))
    F, I = oft.ft_integrals(fock, g4, e, beta, mu)
    ti, g, G = quadrature.simpsons(ng, beta)
    D1 = e[:, None] - e[None, :]
    D2 = (e[:, None, None, None] + e[None, :, None, None]
          - e[None, None, :, None] - e[None, None, None, :])
    t1, t2 = rand_T(rng, ng, n, n, 0.05)
    T1n, T2n = ft_cc_equations.ccsd_stanton(F, I, t1, t2, D1, D2, ti, ng, G)
    st.update(pack_blocks("ft_", F, I))
    st.update(ft_t1=t1, ft_t2=t2, ft_D1=D1, ft_D2=D2, ft_ti=ti, ft_G=G,
              ft_T1=T1n, ft_T2=T2n, ft_eps=e, ft_fock=fock, ft_eri=g4,
              ft_beta=beta, ft_mu=mu)
    # (b) independent random blocks, no != nv
    no, nv, ng = 3, 5, 4
    nt = no + nv
    fr = rng.standard_normal((nt, nt)) * 0.2
    gr = rand_antisym(rng, nt, 0.1)
    F, I = blocks_from_full(fr, gr, no, nv)
    ti, g, G = quadrature.simpsons(ng, 2.0)
    ev = rng.standard_normal(nv)
    eo = rng.standard_normal(no)
    D1 = ev[:, None] - eo[None, :]
    D2 = (ev[:, None, None, None] + ev[None, :, None, None]
          - eo[None, None, :, None] - eo[None, None, None, :])
    t1, t2 = rand_T(rng, ng, nv, no, 0.05)
    T1n, T2n = ft_cc_equations.ccsd_stanton(F, I, t1, t2, D1, D2, ti, ng, G)
    st.update(pack_blocks("rb_", F, I))
    st.update(rb_t1=t1, rb_t2=t2, rb_D1=D1, rb_D2=D2, rb_ti=ti, rb_G=G,
              rb_T1=T1n, rb_T2=T2n)
    numpy.savez_compressed(os.path.join(HERE, "stanton.npz"), **st)

    # ---- UEG end to end through Kelvin's ccsd driver ----------------------
    class Grab(logging.Handler):
        def __init__(self):
            super().__init__()
            self.lines = []

        def emit(self, record):
            self.lines.append(record.getMessage())

    def run(system, **kw):
        grab = Grab()
        root = logging.getLogger()
        root.addHandler(grab)
        root.setLevel(logging.INFO)
        cc = ccsd(system, **kw)
        Etot, Ecc = cc.run()
        root.removeHandler(grab)
        iters = []
        for ln in grab.lines:
            p = ln.split()
            if len(p) == 3 and p[0].isdigit():
                iters.append([float(p[1]), float(p[2])])
        return cc, Etot, Ecc, iters

    T, mu, L = 0.1, 0.1, 2 * numpy.pi
    ueg = UEGSystem(T, L, 1.2, mu=mu, norb=7, orbtype='g')
    cc, Etot, Ecc, iters = run(ueg, T=T, mu=mu, iprint=0, max_iter=50,
                               damp=0.2, ngrid=10)
    en = ueg.g_energies_tot()
    sel = numpy.random.default_rng(7).integers(0, cc.T2.size, 4096)
    numpy.savez_compressed(
        os.path.join(HERE, "ueg7.npz"), eps=en, fock=ueg.g_fock_tot(),
        eri=ueg.g_aint_tot(), T1=cc.T1, T2_sample_idx=sel,
        T2_sample=cc.T2.reshape(-1)[sel])
    json.dump({"T": T, "mu": mu, "L": L, "cutoff": 1.2, "norb": 7, "ngrid": 10,
               "damp": 0.2, "max_iter": 50, "econv": 1e-8,
               "Omega_total": Etot, "Omega_cc": Ecc, "G0": cc.G0, "G1": cc.G1,
               "iterations": iters, "T2_norm": float(numpy.linalg.norm(cc.T2)),
               "kelvin_test_golden": -0.010750238811},
              open(os.path.join(HERE, "ueg7.json"), "w"), indent=1)

    T, mu = 0.1, 0.1182817
    ueg = UEGSCFSystem(T, L, 1.2, mu=mu, norb=7, orbtype='g')
    cc, Etot, Ecc, iters = run(ueg, T=T, mu=mu, iprint=0, max_iter=50,
                               damp=0.1, ngrid=40, tconv=1e-8)
    numpy.savez_compressed(os.path.join(HERE, "uegscf7.npz"),
                           eps=ueg.g_energies_tot(), fock=ueg.g_fock_tot(),
                           eri=ueg.g_aint_tot())
    json.dump({"T": T, "mu": mu, "L": L, "cutoff": 1.2, "norb": 7, "ngrid": 40,
               "damp": 0.1, "max_iter": 50, "econv": 1e-8, "tconv": 1e-8,
               "Omega_total": Etot, "Omega_cc": Ecc, "G1": cc.G1,
               "iterations": iters,
               "kelvin_example_golden_u": -0.009757267319},
              open(os.path.join(HERE, "uegscf7.json"), "w"), indent=1)
    print("UEG7", Ecc, "UEGSCF7", Ecc)


def esn_example(ref_root):
    """ueg19_esn.json from the example script and its recorded output."""
    import re
    ex = os.path.join(ref_root, "examples")
    src = open(os.path.join(ex, "ueg_ft_ccsd_ESN.py")).read()
    out = open(os.path.join(ex, "ueg_ft_ccsd_ESN.out")).read().splitlines()

    def setting(name):
        return float(re.search(r"^%s = ([0-9.eE+-]+)$" % name, src, re.M).group(1))
    meta = {"T": setting("T"), "mu": setting("mu"), "norb": int(setting("norb")),
            "cutoff": setting("cut"), "damp": setting("damp"),
            "max_iter": int(setting("mi")),
            "ngrid": int(re.search(r"ngrid=(\d+)", src).group(1)),
            "econv": 1e-8,                      # ccsd() default; tconv = 1000 econv
            "source": "examples/ueg_ft_ccsd_ESN.py, examples/ueg_ft_ccsd_ESN.out"}
    start = [i for i, l in enumerate(out) if l.startswith("OmegaC:")][0]
    stop = [i for i, l in enumerate(out) if l.startswith("Total CCSD Lambda time")][0]
    meta["Omega"] = float([l for l in out if l.startswith("Omega:")][0].split()[1])
    meta["Omega_cc"] = float(out[start].split()[1])
    meta["lambda_residuals"] = [float(l.split()[1]) for l in out[start + 1:stop]]
    for key in ("E", "S", "N"):
        meta[key] = float([l for l in out if l.startswith(key + ": ")][0].split()[1])
    with open(os.path.join(HERE, "ueg19_esn.json"), "w") as f:
        json.dump(meta, f, indent=1)


if __name__ == "__main__":
    args = [a for a in sys.argv[1:] if not a.startswith("--")]
    root = args[0] if args else "/root/reference"
    esn_example(root)
    if "--esn-only" not in sys.argv:
        main(root)
