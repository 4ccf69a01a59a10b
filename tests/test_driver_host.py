"""The ccsd driver's host logic with a fake device solver.

compute_ESN: with the correlated part of Omega replaced by zero, E, S and N
must be those of Omega0 + Omega1 with the mean-field Fock matrix following
the occupations, whose derivatives are known in closed form.  Unrestricted
systems: amplitudes are returned and accepted per spin case."""
import numpy

from kelvin_gb300 import ccsd as ccsd_mod
from kelvin_gb300.systems import fermi


class FakeCtx(object):
    def __init__(self):
        self._precision = (0, 7)

    def set_precision(self, prec, digits=7):
        self._precision = (prec, digits)


class FakeSystem(object):
    """n orbitals with fixed energies and a symmetric <ij||ij> matrix."""

    def __init__(self, rng, n, T, mu):
        self.T, self.mu = T, mu
        self.en = numpy.sort(rng.standard_normal(n))
        g = rng.standard_normal((n, n, n, n)) * 0.05
        g = g - g.transpose(1, 0, 2, 3)
        g = g - g.transpose(0, 1, 3, 2)
        self.eri = 0.5 * (g + g.transpose(2, 3, 0, 1))

    def verify(self, T, mu):
        return T == self.T and mu == self.mu

    def g_energies_tot(self):
        return self.en

    def g_fock_tot(self):
        fo = fermi(1.0 / self.T, self.en, self.mu)
        return numpy.diag(self.en) + numpy.einsum('prqr,r->pq', self.eri, fo)

    def g_aint_tot(self):
        return self.eri

    def const_energy(self):
        return 0.0


class FakeSolver(object):
    calls = []

    @classmethod
    def from_system(cls, ctx, en, fock, eri, beta, mu, ti, g, G):
        cls.calls.append((beta, mu, fock.copy()))
        return cls()

    def set_amplitudes(self, T1, T2):
        pass

    def guess(self, kind):
        return 0.0

    def prepare_amplitudes(self):
        return lambda: None

    def close(self):
        pass


def test_esn_of_the_mean_field_part(monkeypatch):
    rng = numpy.random.default_rng(4)
    T, mu = 0.3, 0.1
    s = FakeSystem(rng, 6, T, mu)
    monkeypatch.setattr(ccsd_mod, "DeviceSolver", FakeSolver)
    monkeypatch.setattr(ccsd_mod, "converge", lambda *a, **k: (0.0, {}))
    FakeSolver.calls = []
    cc = ccsd_mod.ccsd(s, T=T, mu=mu, ngrid=4, ctx=FakeCtx(), precision='mixed')
    cc.T1, cc.T2 = numpy.zeros(1), numpy.zeros(1)
    E, S, N = cc.compute_ESN()
    assert cc.ctx._precision == (0, 7)                    # restored

    beta, en = 1.0 / T, s.en
    W = numpy.einsum('ijij->ij', s.eri)
    f = fermi(beta, en, mu)
    df_dmu = beta * f * (1 - f)
    df_dbeta = -(en - mu) * f * (1 - f)
    Om1 = 0.5 * f @ W @ f
    Om0 = ccsd_mod.grand_potential0(beta, en, mu)
    N_ref = f.sum() - f @ W @ df_dmu
    E_ref = (f * (en - mu)).sum() + Om1 + beta * (f @ W @ df_dbeta) + mu * N_ref
    S_ref = beta * (E_ref - mu * N_ref - Om0 - Om1)
    assert abs(N - N_ref) < 1e-8
    assert abs(E - E_ref) < 1e-8
    assert abs(S - S_ref) < 1e-7
    # Kelvin's split: with no correlation the CC parts vanish
    assert abs(cc.N0 - f.sum()) < 1e-14
    assert abs(cc.Ncc) < 1e-8 and abs(cc.Ecc) < 1e-8 and abs(cc.Scc) < 1e-7
    assert abs(cc.E0 + cc.E1 + cc.Ecc - E) < 1e-14
    # five solves; the Fock matrix of each follows its occupations
    assert len(FakeSolver.calls) == 5
    for b, m, fock in FakeSolver.calls:
        fo = fermi(b, en, m)
        assert numpy.allclose(fock, numpy.diag(en) + numpy.einsum('prqr,r->pq', s.eri, fo),
                              rtol=0, atol=1e-13)


class USystem(FakeSystem):
    """The same system offered in Kelvin's unrestricted form (has_u)."""

    def has_u(self):
        return True

    def u_energies_tot(self):
        n = self.en.shape[0] // 2
        return self.en[:n], self.en[n:]

    def get_mp1(self):
        f = fermi(1.0 / self.T, self.en, self.mu)
        return 0.5 * numpy.einsum('ijij,i,j->', self.eri, f, f)


def test_unrestricted_system_amplitudes(monkeypatch):
    """Amplitudes of an unrestricted system come back per spin case and are
    accepted per spin case (kelvin/ccsd.py:714-880)."""
    rng = numpy.random.default_rng(5)
    T, mu, ng = 0.3, 0.1, 4
    s = USystem(rng, 6, T, mu)
    n, na = 6, 3
    sp = (numpy.arange(n) >= na).astype(int)
    cons = (sp[:, None, None, None] + sp[None, :, None, None]
            == sp[None, None, :, None] + sp[None, None, None, :])
    T1 = rng.standard_normal((ng, n, n)) * (sp[:, None] == sp[None, :])
    T2 = rng.standard_normal((ng, n, n, n, n))
    T2 = (T2 - T2.transpose(0, 2, 1, 3, 4))
    T2 = (T2 - T2.transpose(0, 1, 2, 4, 3)) * cons
    seen = {}

    class Solver(FakeSolver):
        def amplitudes(self, out=None):
            return T1.copy(), T2.copy()

        def set_amplitudes(self, a, b):
            seen["T1"], seen["T2"] = a, b

    monkeypatch.setattr(ccsd_mod, "DeviceSolver", Solver)
    monkeypatch.setattr(ccsd_mod, "converge", lambda *a, **k: (
        -0.01, {"iterations": 3, "iterations_refine": 0, "converged": True,
                "omega_low": None}))
    cc = ccsd_mod.ccsd(s, T=T, mu=mu, ngrid=ng, ctx=FakeCtx())
    cc.run()
    (t1a, t1b), (t2aa, t2ab, t2bb) = cc.T1, cc.T2
    assert numpy.array_equal(t1a, T1[:, :na, :na]) and numpy.array_equal(t1b, T1[:, na:, na:])
    assert numpy.array_equal(t2ab, T2[:, :na, na:, :na, na:])
    assert numpy.array_equal(t2aa, T2[:, :na, :na, :na, :na])
    assert numpy.array_equal(t2bb, T2[:, na:, na:, na:, na:])
    cc.run(T1=cc.T1, T2=cc.T2)
    assert numpy.array_equal(seen["T1"], T1) and numpy.array_equal(seen["T2"], T2)


def test_unrestricted_lambda_driver(monkeypatch):
    """_ft_ccsd_lambda on a system in the unrestricted form: Kelvin's
    unrestricted guess and residual measure, the general-spin Lambda returned
    per spin case (kelvin/ccsd.py:963-1073)."""
    from kelvin_gb300 import ft_cc_equations as fe
    from kelvin_gb300.cc_utils import one_e_blocks, two_e_blocks
    rng = numpy.random.default_rng(9)
    T, mu, ng, n, na = 0.3, 0.1, 4, 6, 3
    s = USystem(rng, n, T, mu)
    sp = (numpy.arange(n) >= na).astype(int)
    same = sp[:, None] == sp[None, :]
    cons = (sp[:, None, None, None] + sp[None, :, None, None]
            == sp[None, None, :, None] + sp[None, None, None, :])
    T1 = rng.standard_normal((ng, n, n)) * 0.05 * same
    Lg = (rng.standard_normal((ng, n, n)) * same, rng.standard_normal((ng,) + (n,) * 4) * cons)
    F = one_e_blocks(*[rng.standard_normal((n, n)) * same for _ in range(4)])
    I = two_e_blocks(**{k: rng.standard_normal((n,) * 4) * cons for k in fe.I_ORDER})
    seen = {}

    def fake_iter(method, L1, L2, T1_, T2_, F_, I_, D1, D2, g, G, beta, ng_, ti, iprint, conv,
                  ctx=None, spin_half=None):
        seen.update(L1=L1, L2=L2, spin_half=spin_half)
        return Lg
    monkeypatch.setattr(ccsd_mod, "ft_integrals", lambda *a, **k: (F, I))
    monkeypatch.setattr(ccsd_mod, "ft_lambda_iter", fake_iter)
    cc = ccsd_mod.ccsd(s, T=T, mu=mu, ngrid=ng, ctx=FakeCtx())
    cc._Tg = (T1, numpy.zeros((ng,) + (n,) * 4))
    cc.T1 = fe.g_to_u_t(T1, cc._Tg[1], na)[0]
    cc._ft_ccsd_lambda()
    assert seen["spin_half"] == na
    g1, g2 = fe.ccsd_lambda_guess(F, I, T1, cc.beta_max, ng, unrestricted=True)
    assert abs(seen["L1"] - g1).max() == 0.0 and abs(seen["L2"] - g2).max() == 0.0
    (l1a, l1b), (l2aa, l2ab, l2bb) = cc.L1, cc.L2
    assert numpy.array_equal(l1b, Lg[0][:, na:, na:])
    assert numpy.array_equal(l2ab, Lg[1][:, :na, na:, :na, na:])
    assert cc._Lg is Lg


def test_full_rdms_of_the_reference():
    """With no correlation (zero normal-ordered parts) the full RDMs are the
    grand-canonical mean-field ones: gamma = diag(f), and
    sum_pq Gamma[p,q,p,q] = (sum f)^2 - sum f^2 (kelvin/cc_utils.py:2018-2024)."""
    rng = numpy.random.default_rng(6)
    T, mu = 0.3, 0.1
    s = FakeSystem(rng, 6, T, mu)
    cc = ccsd_mod.ccsd(s, T=T, mu=mu, ngrid=4, ctx=FakeCtx())
    n = s.en.shape[0]
    cc.n1rdm, cc.n2rdm = numpy.zeros((n, n)), numpy.zeros((n,) * 4)
    f = fermi(1.0 / T, s.en, mu)
    assert numpy.allclose(cc.full_1rdm(), numpy.diag(f), rtol=0, atol=1e-15)
    g2 = cc.full_2rdm()
    assert abs(numpy.einsum('pqpq->', g2) - (f.sum() ** 2 - (f * f).sum())) < 1e-13
    assert abs(g2 + g2.transpose(1, 0, 2, 3)).max() < 1e-15


def test_lambda_on_the_resident_solver():
    """After a solve the Lambda equations run on the solver's resident
    integrals and amplitudes, with Kelvin's unrestricted guess and measure for
    a system in the unrestricted form."""
    from kelvin_gb300 import ft_cc_equations as fe
    rng = numpy.random.default_rng(10)
    T, mu, ng, n, na = 0.3, 0.1, 3, 6, 3
    s = USystem(rng, n, T, mu)
    Lg = (rng.standard_normal((ng, n, n)), rng.standard_normal((ng,) + (n,) * 4))
    seen = {}

    class Solver(object):
        def lambda_solve(self, conv, guess=1, L1=None, L2=None, measure_half=None,
                         history=None):
            seen.update(conv=conv, guess=guess, measure_half=measure_half)
            return Lg
    cc = ccsd_mod.ccsd(s, T=T, mu=mu, ngrid=ng, ctx=FakeCtx(), damp=0.3, max_iter=17)
    cc._Tg = (numpy.zeros((ng, n, n)), numpy.zeros((ng,) + (n,) * 4))
    cc.T1 = "set"
    cc.solver = Solver()
    cc._ft_ccsd_lambda()
    assert seen["guess"] == 2 and seen["measure_half"] == na
    assert seen["conv"]["damp"] == 0.3 and seen["conv"]["max_iter"] == 17
    assert cc._Lg is Lg
    assert numpy.array_equal(cc.L2[1], Lg[1][:, :na, na:, :na, na:])
    assert cc.ctx._precision == (0, 7)


class ScriptSolver(object):
    """Steps through scripted (E, res) pairs per digit-level setting and
    records the mixing factor each step was given."""

    def __init__(self, ctx, script):
        self.ctx, self.script, self.pos, self.damps = ctx, script, {}, []

    def step(self, damp):
        lv = self.ctx._precision[1]
        k = self.pos.get(lv, 0)
        self.pos[lv] = k + 1
        self.damps.append(damp)
        seq = self.script[lv]
        return seq[min(k, len(seq) - 1)]


def test_converge_phases_and_residual_cut():
    """Few-digit phases end at their noise floor (three sweeps without a new
    best below 0.9 of it) or, with low_tconv, once the residual is below it;
    the ladder continues after a cut; only the refinement's Kelvin test
    counts as convergence."""
    three = [(-1.0, 1e-1), (-0.9, 1e-2), (-0.95, 5e-5), (-0.95, 8e-5), (-0.95, 6e-5),
             (-0.95, 7e-5), (-0.95, 9e-5)]
    five = [(-0.95, 1e-4), (-0.95, 4e-5), (-0.95, 5e-5), (-0.95, 6e-5), (-0.95, 7e-5)]
    seven = [(-0.9500001, 1e-5), (-0.95000001, 1e-6), (-0.950000010001, 1e-8)]
    conv = {"econv": 1e-10, "tconv": 1e-7, "max_iter": 50, "damp": 0.3}

    ctx = FakeCtx()
    s = ScriptSolver(ctx, {3: three, 5: five, 7: seven})
    E, info = ccsd_mod.converge(s, ctx, conv, 'mixed', 3, ladder=(5,))
    assert info["phases"] == [(3, 6, True), (5, 5, True), (7, 3, False)]
    assert info["converged"] and abs(E + 0.950000010001) < 1e-15

    ctx = FakeCtx()
    s = ScriptSolver(ctx, {3: three, 5: five, 7: seven})
    E, info = ccsd_mod.converge(s, ctx, conv, 'mixed', 3, ladder=(5,), low_tconv=1e-4)
    # 3 levels: cut at the third sweep; 5 levels: 1e-4 is not below the cut,
    # 4e-5 is; then the refinement
    assert info["phases"] == [(3, 3, False), (5, 2, False), (7, 3, False)]
    assert info["iterations"] == 5 and info["iterations_refine"] == 3
    assert info["converged"]
    assert set(s.damps) == {0.3}
    assert ctx._precision == (0, 7)           # the caller's setting is restored

    # a refinement that never meets Kelvin's test is not converged, even when
    # every few-digit phase met its cut
    ctx = FakeCtx()
    s = ScriptSolver(ctx, {3: three, 7: [(-0.95, 1e-5), (-0.96, 1e-5)]})
    E, info = ccsd_mod.converge(s, ctx, dict(conv, max_iter=4), 'mixed', 3, ladder=(),
                                low_tconv=1e-4)
    assert not info["converged"] and info["iterations_refine"] == 4


def test_prepared_amplitude_arrays():
    """DeviceSolver.prepare_amplitudes: the host thread returns zeroed arrays
    of the amplitude shapes (the read-back writes only the spin-conserving
    blocks into them)."""
    from kelvin_gb300.cc_utils import DeviceSolver
    for h in (0, 2):
        sv = DeviceSolver.__new__(DeviceSolver)
        sv.ng, sv.nv, sv.no = 3, 4, 4
        sv.spin_blocks = lambda on=None, h=h: h
        T1, T2 = sv.prepare_amplitudes()()
        assert T1.shape == (3, 4, 4) and T2.shape == (3, 4, 4, 4, 4)
        assert T2.flags.c_contiguous and not T2.any()
