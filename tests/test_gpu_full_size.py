"""Parity at the benchmark sizes.  Each benchmark workload runs in full
on the GPU; the CPU oracle then computes groups (or instances, or
requests) of it.  Groups, instances and sessions are independent, so
those must agree: log-likelihoods to 1e-12 relative (parallel vs serial
weight sums), final state and generator words exactly, dopri5 outputs
within the solver's tolerance (the GPU solver fuses its stage sums and
evaluates the controller's powers with the engine's exp and log, so
its rounding differs from the CPU's).  Slower than the other tests (a minute or two)."""

import ctypes

import numpy as np
import pytest

import bench
import dust2_gb300 as d
from dust2_gb300 import _lib, workloads

pytestmark = pytest.mark.gpu


def filter_full_vs_oracle(port, w, gen, pick_ll, pick_state, n_state):
    """Run the whole workload on the GPU; the oracle runs the groups of
    pick_ll and pick_state.  Log-likelihoods of pick_ll agree to 1e-12
    relative; final state, particle generators and filter generators of
    pick_state agree exactly."""
    npg = w["n_particles"]
    G = len(npg)
    obj = d.dust_filter_create(gen, 0, bench.data_columns(w),
                               n_particles=npg, dt=w["dt"], seed=w["seed"])
    words0 = np.frombuffer(d.dust_likelihood_rng_state(obj), dtype="<u8")
    ll = d.dust_likelihood_run(obj, w["plist"])
    state = d.dust_likelihood_last_state(obj)
    if obj.n_particles_per_group is None:
        state = np.asarray(state).transpose(2, 1, 0)
    state = np.asarray(state).ravel()  # [group][particle][state]
    words = np.frombuffer(d.dust_likelihood_rng_state(obj), dtype="<u8")
    pick = sorted(set(pick_ll) | set(pick_state))
    want, want_state, want_rng = port.filter_run(
        gen.name, w["pars"], npg, 0.0, w["times"],
        np.asarray(w["data"]).ravel(), G, w["dt"], words0,
        index_group=pick, n_state=n_state, n_threads=port.max_threads())
    np.testing.assert_allclose(ll[pick_ll], want[0][pick_ll], rtol=1e-12,
                               atol=0)
    off = np.concatenate([[0], np.cumsum(npg)])
    soff = np.concatenate([[0], np.cumsum([n + 2 for n in npg])])
    for g in pick_state:
        a, b = off[g] * n_state, off[g + 1] * n_state
        np.testing.assert_array_equal(state[a:b], want_state[a:b])
        a, b = 4 * soff[g], 4 * soff[g + 1]
        np.testing.assert_array_equal(words[a:b], want_rng[a:b])


def test_batched_sir_full_size(port):
    # 64 groups, 514,064 particles, 200 observations: every group's
    # log-likelihood, and the final state and generators of four
    w = workloads.sir_batched(bench.gpu_simulate_factory())
    assert sum(w["n_particles"]) == 514064
    filter_full_vs_oracle(port, w, d.sir_cases(), list(range(64)),
                          [0, 21, 42, 63], 4)


def test_age_seir_full_size(port):
    # 32 groups x 8192 particles, 365 observations: eight groups'
    # log-likelihoods, the state and generators of two
    w = workloads.seir_batched(bench.gpu_simulate_factory())
    filter_full_vs_oracle(port, w, d.seir_age(), list(range(0, 32, 4)),
                          [0, 20], 96)


def test_serving_stream_requests_match_oracle(port):
    # requests of the serving workload (its sessions, parameters and
    # data), served two in a row per session among the other sessions of
    # the stream, against the oracle running each session's filter alone
    # from the same streams: the second request continues from the
    # generators the first left
    w = bench.serve_workload(bench.gpu_simulate_factory(), 8)
    assert min(w["counts"]) == 2  # two requests per session
    clients = w["clients"]
    sizes = [c["n_particles"] for c in clients]
    picks = [int(np.argmin(sizes)), int(np.argsort(sizes)[32]),
             int(np.argmax(sizes))]
    server = d.dust_likelihood_server(d.seir_age(), hbm_budget=8e9,
                                      max_sessions=64)
    try:
        ids = [server.open(c["pars"][0], c["data"], c["n_particles"],
                           dt=w["dt"], seed=c["seed"]) for c in clients]
        tickets = [[server.submit(ids[i], c["pars"][0])]
                   for i, c in enumerate(clients)]
        got = {}
        for i in picks:
            got[i] = [server.wait(tickets[i][0])[0]]
            tickets[i].append(server.submit(ids[i], clients[i]["pars"][1]))
        for i, c in enumerate(clients):
            if i not in picks:
                server.wait(tickets[i][0])
        for i in picks:
            got[i].append(server.wait(tickets[i][1])[0])
    finally:
        server.free()
    for i in picks:
        c = clients[i]
        n = c["n_particles"]
        rng = np.frombuffer(d.rng_streams(n + 2, c["seed"]), dtype="<u8")
        data = np.asarray(c["data"]["incidence"], dtype=float)
        for r in range(2):
            pars = d.seir_age().pack_pars(c["pars"][r])
            want, _, rng = port.filter_run(
                "seir_age", pars, [n], 0.0, c["data"]["time"], data, 1,
                w["dt"], rng, n_state=96, n_threads=port.max_threads())
            np.testing.assert_allclose(got[i][r], want[0][0], rtol=1e-12,
                                       atol=0)


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
