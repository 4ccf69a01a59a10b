"""bench.py's JSON line on the CPU, with a fake context, solver and driver in
place of the device: the keys and units of the line, the roofline fraction
against the measured peaks, the end-to-end byte counts and the CPU baseline
entry."""
import json

import numpy
import pytest

import conftest  # noqa: F401  (puts the repository root on the path)

bench = pytest.importorskip("bench")
from kelvin_gb300 import _lib, cc_utils, ccsd   # noqa: E402


class FakeCtx(object):
    device = 0

    def __init__(self):
        self._precision = (0, 7)

    def set_precision(self, p, d=None):
        self._precision = (p, d)

    def sync(self):
        pass

    def record(self, k):
        pass

    def elapsed_ms(self, a, b):
        return 100.0

    def profile_begin(self):
        pass

    def profile_end(self):
        # (launches, ms, work) per category: the n^5 class dominates by time
        return {c: (10, 300.0 if c == "gemm" else 10.0, 1e12 if c == "gemm6" else 1e9)
                for c in _lib.PROFILE_CATEGORIES}

    def launches(self):
        return 5


class FakeSolver(object):
    full = False

    @classmethod
    def from_system(cls, *a, **k):
        return cls()

    def set_acceleration(self, m):
        pass

    def guess(self, k):
        return 0.0

    def step(self, d):
        return -0.9, 1e-3

    def close(self):
        pass


class FakeCC(object):
    def __init__(self, s, **kw):
        self.Gcc, self.Gtot = -0.95, -3.0
        self.iterations, self.iterations_refine = 7, 7
        self.phases = [(3, 7, False), (6, 7, False)]
        self.converged = True

    def run(self):
        return (-3.0, -0.95)

    def compute_ESN(self, method='fd'):
        return (1.0, 2.0, 3.0)

    def release(self):
        pass


class FakeSystem(object):
    T, mu = 0.25, 0.1

    def g_energies_tot(self):
        return numpy.zeros(114)

    def g_fock_tot(self):
        return None

    def g_aint_tot(self):
        return None


class Args(object):
    precision, digits, quad = "mixed", 0, "gl"
    accel, mix, low_tconv = 3, 0.7, 3e-4
    steps, warmup, workload = 3, 1, "ueg114"


def test_bench_line_contract(monkeypatch, capsys):
    monkeypatch.setattr(bench, "dist_setup", lambda: (1, 0, 0))
    monkeypatch.setattr(_lib, "context", lambda d=0: FakeCtx())
    monkeypatch.setattr(cc_utils, "DeviceSolver", FakeSolver)
    monkeypatch.setattr(ccsd, "ccsd", FakeCC)
    monkeypatch.setattr(bench, "oracle_c1_iterations",
                        lambda q, n, until_converged: (1.0, [3.0, 3.1, 3.2], None, -0.1))
    monkeypatch.setattr(bench, "build_system", lambda w: FakeSystem())
    monkeypatch.setattr(bench.ClockSampler, "start", lambda self: None)
    monkeypatch.setattr(bench.ClockSampler, "stop", lambda self: None)
    bench.run_gpu(Args(), bench.WORKLOADS["ueg114"])
    line = [ln for ln in capsys.readouterr().out.splitlines() if ln.startswith("{")][-1]
    d = json.loads(line)
    for k in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step",
              "higher_is_better", "scaling", "vs_baseline", "dtype", "data", "config",
              "roofline", "cpu_baseline", "e2e", "gpu_launches"):
        assert k in d, k
    assert d["unit"] == "solves/s" and d["higher_is_better"] is True
    assert (d["n_gpus"], d["steps"], d["warmup"]) == (1, 3, 1)
    assert d["value"] > 0 and abs(d["ms_per_step"] - 100.0 / 3) < 1e-9
    assert "114 spin orbitals" in d["config"]["workload"]
    # the end-to-end figure: same metric, the step's host <-> device bytes
    e = d["e2e"]
    assert e["unit"] == d["unit"] and e["value"] > 0
    assert e["h2d_bytes_per_step"] > 0 and e["d2h_bytes_per_step"] > 0
    # the dominant category by time, against the measured peak of its bound
    r = d["roofline"]
    peaks, _ = bench.load_peaks()          # the measured file, else the fallback
    assert r["category"] == "gemm" and r["bound"] == "hbm" and r["unit"] == "GB/s"
    assert r["peak"] == peaks["hbm_gbs"]
    assert abs(r["frac"] - r["achieved"] / r["peak"]) < 1e-12
    assert set(r["categories"]) == set(_lib.PROFILE_CATEGORIES)
    c = d["cpu_baseline"]
    assert c["kind"] in ("port", "reference") and c["cores"] >= 1 and c["value"] > 0
    assert c["unit"] == d["unit"] and c["sample"]
    assert isinstance(d["gpu_launches"], int) and d["gpu_launches"] >= 0


def test_reference_arm_contract(monkeypatch, capsys):
    """--impl reference: rank 0 times the oracle's complete solve of the
    38-spin-orbital workload and prints the same metric with impl, its CPU
    baseline (the line's own value) and an e2e entry with no device bytes;
    other ranks print nothing."""
    monkeypatch.setattr(bench, "oracle_c1_iterations",
                        lambda q, n, until_converged: (1.0, [3.0, 3.1, 3.2, 3.3], 3, -0.127))

    class A(Args):
        gpus = 1
    monkeypatch.setattr(bench, "dist_setup", lambda: (2, 1, 1))
    assert bench.run_reference(A(), bench.WORKLOADS["ueg38"]) == 0
    assert not [ln for ln in capsys.readouterr().out.splitlines() if ln.startswith("{")]
    monkeypatch.setattr(bench, "dist_setup", lambda: (1, 0, 0))
    assert bench.run_reference(A(), bench.WORKLOADS["ueg38"]) == 0
    d = json.loads([ln for ln in capsys.readouterr().out.splitlines() if ln.startswith("{")][-1])
    assert d["impl"] == "reference" and d["metric"] == bench.METRIC and d["unit"] == "solves/s"
    # guess 1 s + the three iterations to convergence
    assert abs(d["value"] - 1.0 / (1.0 + 3.0 + 3.1 + 3.2)) < 1e-12
    assert d["cpu_baseline"]["value"] == d["value"] and d["cpu_baseline"]["kind"] == "port"
    assert d["e2e"] == {"value": d["value"], "unit": "solves/s", "h2d_bytes_per_step": 0,
                        "d2h_bytes_per_step": 0}
    assert "38 spin orbitals" in d["config"]["workload"]
