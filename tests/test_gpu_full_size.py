"""Parity at the benchmark sizes.  Each benchmark workload runs in full
on the GPU; the CPU oracle then computes a few of its groups (or
instances).  Groups and instances are independent, so those must agree:
log-likelihoods to 1e-12 relative (parallel vs serial weight sums),
dopri5 outputs within the solver's tolerance (the step controller's pow
is each platform's own).  Slower than the other tests (about a minute)."""

import ctypes

import numpy as np
import pytest

import bench
import dust2_gb300 as d
from dust2_gb300 import _lib, workloads

pytestmark = pytest.mark.gpu


def filter_full_vs_oracle(port, w, gen, pick, n_state):
    npg = w["n_particles"]
    G = len(npg)
    obj = d.dust_filter_create(gen, 0, bench.data_columns(w),
                               n_particles=npg, dt=w["dt"], seed=w["seed"])
    ll = d.dust_likelihood_run(obj, w["plist"])
    rng = np.frombuffer(d.rng_streams(sum(n + 2 for n in npg), w["seed"]),
                        dtype="<u8")
    want, _, _ = port.filter_run(
        gen.name, w["pars"], npg, 0.0, w["times"],
        np.asarray(w["data"]).ravel(), G, w["dt"], rng, index_group=pick,
        n_state=n_state, n_threads=port.max_threads())
    np.testing.assert_allclose(ll[pick], want[0][pick], rtol=1e-12, atol=0)


def test_batched_sir_full_size(port):
    # 64 groups, 514,064 particles, 200 observations
    w = workloads.sir_batched(bench.gpu_simulate_factory())
    assert sum(w["n_particles"]) == 514064
    filter_full_vs_oracle(port, w, d.sir_cases(), [0, 31, 63], 4)


def test_age_seir_full_size(port):
    # 32 groups x 8192 particles, 365 observations
    w = workloads.seir_batched(bench.gpu_simulate_factory())
    filter_full_vs_oracle(port, w, d.seir_age(), [0, 17], 96)


def test_dopri5_full_size(port):
    # 262,144 instances, 201 outputs
    w = workloads.sirode_batched()
    G = w["n_groups"]
    times = _lib.as_f64(w["times"])
    h = bench.ode_alloc(w)
    try:
        _lib.check(_lib.lib().dust2_gb300_system_set_state_initial(h))
        out = np.empty(times.size * G * 5)
        _lib.check(_lib.lib().dust2_gb300_system_simulate(
            h, _lib.dptr(times), times.size, None, 0, _lib.dptr(out)))
        n = G
        ns = np.zeros(n, dtype=np.int64)
        na = np.zeros(n, dtype=np.int64)
        nr = np.zeros(n, dtype=np.int64)
        ss = np.zeros(n)
        er = np.zeros(n)
        _lib.check(_lib.lib().dust2_gb300_system_internals(
            h, _lib.dptr(ss), _lib.dptr(er),
            ns.ctypes.data_as(_lib.c_i64_p), na.ctypes.data_as(_lib.c_i64_p),
            nr.ctypes.data_as(_lib.c_i64_p)))
    finally:
        _lib.lib().dust2_gb300_system_free(h)
    k = 2048
    pars = np.asarray(w["pars"]).reshape(G, 4)[:k].ravel()
    want, stats = port.ode_simulate("sirode", pars, k, 1, 0.0, times, 5,
                                    n_threads=port.max_threads())
    got = out.reshape(times.size, G, 5)[:, :k, :]
    np.testing.assert_allclose(got.ravel(), want, rtol=1e-9, atol=1e-9)
    assert np.mean(ns[:k] == stats[:, 0]) > 0.99
