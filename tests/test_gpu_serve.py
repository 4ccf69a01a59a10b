"""Continuous batching on the GPU (kelvin_gb300.serve): requests that overlap
on the device give the grand potential each gives alone, within the mixed
form's stated tolerance (1e-6 Ha per electron)."""
import pytest

from kelvin_gb300 import serve

pytestmark = pytest.mark.gpu


def _requests():
    R = serve.Request
    return [R(0, 0.00, 'ueg', (14, 19, 4.0), 0.5, 10),
            R(1, 0.00, 'hubbard', (12, 2.0), 0.8, 20),
            R(2, 0.01, 'ueg', (14, 27, 2.0), 1.0, 10),
            R(3, 0.02, 'hubbard', (8, 2.0), 1.0, 10),
            R(4, 0.03, 'ueg', (14, 19, 1.5), 2.0, 20)]


@pytest.mark.parametrize("accel", [0, 3])
def test_results_alone_and_in_the_mix(accel):
    """Kelvin's damped update with CUDA-graph replay, and the accelerated
    scheme (depth 3, mixing factor 0.7, residual cut 1e-4) whose split step
    keeps the solves overlapped."""
    kw = dict(accel=accel, mix=0.7, low_tconv=1e-4) if accel else {}
    mix = serve.Server(precision='mixed', slots=3, warm=False, workspace_bytes=4 << 30, **kw)
    rep = mix.serve(_requests())
    assert rep["solves"] == 5 and rep["rejected"] == 0
    assert rep["max_active"] >= 2                    # their iterations overlapped
    by_mix = {d["rid"]: d for d in rep["requests"]}
    alone = serve.Server(precision='mixed', slots=1, warm=False, workspace_bytes=4 << 30,
                         **kw)
    for r in _requests():
        one = alone.serve([serve.Request(r.rid, 0.0, r.kind, r.params, r.theta, r.ng)])
        d = one["requests"][0]
        m = by_mix[r.rid]
        assert d["ok"] and m["ok"] and d["converged"] and m["converged"]
        N = r.system().N
        assert abs(d["omega"] - m["omega"]) < 1e-6 * N, (r.rid, d["omega"], m["omega"])
        # the same arithmetic in the same order: far below the bar
        assert abs(d["omega"] - m["omega"]) < 1e-9, (r.rid, d["omega"], m["omega"])


def test_graph_replay_matches_eager(ctx):
    """A solve whose iterations are replayed as a CUDA graph gives the eager
    solve's grand potential, and the graph is in use."""
    from kelvin_gb300 import _lib, systems
    from kelvin_gb300.cc_utils import DeviceSolver, iterate
    from kelvin_gb300.quadrature import ft_quad
    s = systems.ueg_recipe(14, 4.0, 19, 0.5)
    beta = 1.0 / s.T
    ti, g, G = ft_quad(10, beta, 'lin')
    conv = {"econv": 1e-10, "tconv": 1e-7, "max_iter": 100, "damp": 0.5}
    out = {}
    for graph in (False, True):
        ctx.set_precision(_lib.PREC_FP64_TC, 7)
        sv = DeviceSolver.from_system(ctx, s.g_energies_tot(), s.g_fock_tot(), s.g_aint_tot(),
                                      beta, s.mu, ti, g, G)
        try:
            sv.guess(1)
            sv.set_graph(graph)
            out[graph] = (iterate(sv, conv), sv.iterations, sv.set_graph())
        finally:
            sv.close()
            ctx.set_precision(_lib.PREC_FP64, 7)
    assert out[True][2] == 2 and out[False][2] == 0
    assert out[True][1] == out[False][1]
    assert abs(out[True][0] - out[False][0]) < 1e-12
