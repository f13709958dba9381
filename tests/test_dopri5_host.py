"""The GPU's dopri5 arithmetic on the CPU: the engine's own solver code
(dust2_gb300/csrc/engine/dopri5.cuh, compiled for the host with nvcc from
tests/dopri5_host.cu) against the oracle's restatement of dust2's solver
and against dust2's own fixtures.  The engine evaluates the stage sums as
fused multiply-add chains, the step-size controller's powers through its
own exp and log and the error norm's divisions through its reciprocal,
so it rounds differently from dust2; the contract is
agreement within the solver's tolerance (rtol = atol = 1e-6).  Observed:
within 4e-13 relative, with the same step counts."""

import ctypes
import shutil
import subprocess

import numpy as np
import pytest

from conftest import ROOT, golden
from dust2_gb300 import workloads

CSRC = ROOT / "dust2_gb300" / "csrc"


@pytest.fixture(scope="module")
def host(tmp_path_factory):
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not shutil.which(nvcc):
        pytest.skip("nvcc not available")
    lib = tmp_path_factory.mktemp("dopri5") / "libdopri5_host.so"
    subprocess.run(
        [nvcc, "-std=c++17", "-O2", "-shared", "-Xcompiler",
         "-fPIC,-ffp-contract=off", "-I", str(CSRC),
         "-gencode", "arch=compute_103a,code=sm_103a",
         str(ROOT / "tests" / "dopri5_host.cu"), "-o", str(lib)],
        check=True, capture_output=True)
    so = ctypes.CDLL(str(lib))
    so.host_div_period.restype = ctypes.c_double
    so.host_div_period.argtypes = [ctypes.c_double, ctypes.c_double]
    so.host_recip.restype = ctypes.c_double
    so.host_recip.argtypes = [ctypes.c_double]
    d = ctypes.POINTER(ctypes.c_double)

    def run(name, flat, n, times, n_state, critical=()):
        flat = np.ascontiguousarray(flat, dtype=np.float64)
        times = np.ascontiguousarray(times, dtype=np.float64)
        crit = np.ascontiguousarray(critical, dtype=np.float64)
        out = np.empty(times.size * n * n_state)
        stats = np.empty(3 * n, dtype=np.int64)
        rc = so.host_ode(
            name.encode(), flat.ctypes.data_as(d), flat.size // n, n,
            times.ctypes.data_as(d), times.size, out.ctypes.data_as(d),
            stats.ctypes.data_as(ctypes.POINTER(ctypes.c_int64)),
            ctypes.c_double(np.finfo(float).eps), ctypes.c_double(np.inf),
            crit.ctypes.data_as(d) if crit.size else None, crit.size)
        assert rc == 0
        return out, stats.reshape(n, 3)
    run.lib = so
    return run


def sirode_row(p):
    return np.array([p["I0"], p["N"], p["beta"], p["gamma"]])


def test_dopri5_workload_matches_oracle(host, port):
    n = 2048
    w = workloads.sirode_batched(n_instances=n)
    got, stats = host("sirode", w["pars"], n, w["times"], 5)
    want, want_stats = port.ode_simulate("sirode", w["pars"], n, 1, 0.0,
                                         w["times"], 5)
    np.testing.assert_allclose(got, want, rtol=1e-6, atol=1e-6)
    rel = np.abs(got - want) / np.maximum(1, np.abs(want))
    assert rel.max() < 1e-11
    assert np.mean(stats[:, 0] == want_stats[:, 0]) > 0.99


def test_dopri5_matches_reference_fixture(host):
    g = golden("ode_sirode")
    pars = [{"beta": 0.2, "gamma": 0.1, "N": 1000, "I0": 10},
            {"beta": 0.4, "gamma": 0.05, "N": 1e6, "I0": 50}]
    flat = np.concatenate([sirode_row(p) for p in pars for _ in range(2)])
    got, stats = host("sirode", flat, 4, g["times"], 5)
    np.testing.assert_allclose(got, g["out"], rtol=1e-12, atol=1e-12)
    np.testing.assert_array_equal(stats, g["stats"])


def test_dopri5_critical_times_fixture(host):
    g = golden("ode_sirode_critical")
    flat = sirode_row({"beta": 0.2, "gamma": 0.1, "N": 1000, "I0": 10})
    got, _ = host("sirode", flat, 1, np.array([50.0]), 5,
                  critical=[10, 20, 30])
    np.testing.assert_allclose(got, g["out"][-5:], rtol=1e-12)


def test_period_division_is_exact(host):
    # the zero_every check's t / period: a multiplication by the exact
    # reciprocal for powers of two, a division otherwise -- always the
    # correctly rounded quotient
    rs = np.random.default_rng(5)
    ts = np.concatenate([rs.uniform(0, 400, 20000), np.arange(0, 401.0),
                         rs.uniform(-50, 50, 2000), [0.0, -0.0, 1e-310]])
    for period in (1.0, 0.5, 0.25, 2.0, 7.0, 2.0 ** -30, 2.0 ** 40, 0.1, 3.0,
                   -1.0):
        got = np.array([host.lib.host_div_period(t, period) for t in ts])
        np.testing.assert_array_equal(got.view(np.uint64),
                                      (ts / period).view(np.uint64))


def test_reciprocal_within_an_ulp(host):
    rs = np.random.default_rng(6)
    xs = np.concatenate([10.0 ** rs.uniform(-29, 29, 20000),
                         -(10.0 ** rs.uniform(-5, 5, 100)),
                         [1e-300, 1e300, 3.0, 0.1]])
    got = np.array([host.lib.host_recip(x) for x in xs])
    want = 1.0 / xs
    ulp = np.spacing(np.abs(want))
    assert np.all(np.abs(got - want) <= ulp)
