"""The likelihood server against the plain filter.

A session of the server is a one-group likelihood object; every request
must give exactly the log-likelihood (and leave exactly the generator
state) that the same sequence of dust_likelihood_run calls gives on a
plain filter created with the same parameters, data and seed, whatever
else the server is running at the time.  The plain filter is itself
checked against the reference engine and the oracle in
test_gpu_filter.py.  Tolerance: exact (same kernels, same tiles, same
arithmetic)."""

import numpy as np
import pytest

import dust2_gb300 as d

pytestmark = pytest.mark.gpu

DT = 0.25


def sir_data(rs, n_obs, scale=1.0):
    times = np.arange(1, n_obs + 1, dtype=float)
    inc = rs.poisson(scale * (5 + 20 * np.sin(times / 7) ** 2)).astype(float)
    return {"time": times, "incidence": inc}


def sir_pars(rs):
    return {"N": 1e5, "I0": float(rs.integers(1, 50)),
            "beta": float(rs.uniform(0.15, 0.5)),
            "gamma": float(rs.uniform(0.05, 0.2))}


def sir_update(rs):
    return {"beta": float(rs.uniform(0.15, 0.5)),
            "gamma": float(rs.uniform(0.05, 0.2))}


def plain_runs(gen, data, n_particles, seed, pars_seq):
    obj = d.dust_filter_create(gen, 0, data, n_particles=n_particles, dt=DT,
                               seed=seed)
    ll = [float(np.ravel(d.dust_likelihood_run(obj, p))[0])
          for p in pars_seq]
    return ll, d.dust_likelihood_rng_state(obj)


def make_sessions(rs, k, n_choices, obs_range):
    out = []
    for i in range(k):
        n = int(rs.choice(n_choices))
        n_obs = int(rs.integers(*obs_range))
        p0 = sir_pars(rs)
        seq = [p0] + [dict(p0, **sir_update(rs)) for _ in range(2)]
        out.append({"n": n, "data": sir_data(rs, n_obs), "seed": 1000 + i,
                    "pars": seq})
    return out


def serve(server, sessions, order="interleaved"):
    """Submit every session's requests, interleaved across sessions;
    returns per session the list of log-likelihoods and its ids."""
    ids = [server.open(s["pars"][0], s["data"], s["n"], dt=DT,
                       seed=s["seed"]) for s in sessions]
    tickets = [[] for _ in sessions]
    n_req = max(len(s["pars"]) for s in sessions)
    for r in range(n_req):
        for i, s in enumerate(sessions):
            if r < len(s["pars"]):
                tickets[i].append(server.submit(ids[i], s["pars"][r]))
    ll = [[server.wait(t)[0] for t in ts] for ts in tickets]
    return ll, ids


def test_server_matches_plain_filter(built):
    gen = d.sir_cases()
    rs = np.random.default_rng(11)
    sessions = make_sessions(rs, 9, [1, 7, 64, 100, 129, 513, 2000],
                             (5, 40))
    server = d.dust_likelihood_server(gen, hbm_budget=2e8, max_sessions=16)
    ll, ids = serve(server, sessions)
    for s, got, sid in zip(sessions, ll, ids):
        want, rng = plain_runs(gen, s["data"], s["n"], s["seed"], s["pars"])
        np.testing.assert_array_equal(np.array(got), np.array(want))
        assert server.rng_state(sid, s["n"]) == rng
    st = server.stats()
    assert st["requests_done"] == sum(len(s["pars"]) for s in sessions)
    assert st["max_running"] > 1  # requests did overlap on the device
    server.free()


def test_server_alone_equals_mix(built):
    gen = d.sir_cases()
    rs = np.random.default_rng(12)
    sessions = make_sessions(rs, 6, [50, 300, 1000], (10, 30))
    alone = []
    for s in sessions:
        server = d.dust_likelihood_server(gen, hbm_budget=1e8,
                                          max_sessions=2)
        ll, _ = serve(server, [s])
        alone.append(ll[0])
        server.free()
    server = d.dust_likelihood_server(gen, hbm_budget=1e8, max_sessions=8)
    mixed, _ = serve(server, sessions)
    server.free()
    for a, m in zip(alone, mixed):
        np.testing.assert_array_equal(np.array(a), np.array(m))


def test_server_admits_as_memory_frees(built):
    gen = d.sir_cases()
    rs = np.random.default_rng(13)
    server = d.dust_likelihood_server(gen, hbm_budget=1.2e6, max_sessions=4)
    cap = server.capacity()["n_particles"]
    n = cap // 2 - 40  # two sessions fit at a time
    assert n > 64
    sessions = []
    for i in range(5):
        p0 = sir_pars(rs)
        sessions.append({"n": n, "data": sir_data(rs, 12), "seed": 77 + i,
                         "pars": [p0, dict(p0, **sir_update(rs))]})
    assert 5 * n > cap
    ids = [server.open(s["pars"][0], s["data"], s["n"], dt=DT,
                       seed=s["seed"]) for s in sessions]
    tickets = [[server.submit(i, p) for p in s["pars"]]
               for i, s in zip(ids, sessions)]
    # a session's memory is released when it is closed after its requests
    for i in ids:
        server.close(i)
    for s, ts in zip(sessions, tickets):
        got = [server.wait(t)[0] for t in ts]
        want, _ = plain_runs(gen, s["data"], s["n"], s["seed"], s["pars"])
        np.testing.assert_array_equal(np.array(got), np.array(want))
    st = server.stats()
    assert st["resident_sessions"] == 0 and st["particles_in_use"] == 0
    server.free()


def test_server_seir_matches_plain(built):
    from dust2_gb300 import workloads
    gen = d.seir_age()
    rs = np.random.default_rng(3)
    plist = workloads.seir_plist(rs.uniform(1.2, 3.0, 3))
    sessions = []
    for i, (p, n) in enumerate(zip(plist, [37, 128, 300])):
        n_obs = 15 + 5 * i
        times = np.arange(1, n_obs + 1, dtype=float)
        data = {"time": times,
                "incidence": rs.poisson(3.0, n_obs).astype(float)}
        seq = [p, dict(p, R0=float(rs.uniform(1.2, 3.0)))]
        sessions.append({"n": n, "data": data, "seed": 5 + i, "pars": seq})
    server = d.dust_likelihood_server(gen, hbm_budget=5e8, max_sessions=8)
    ll, ids = serve(server, sessions)
    for s, got, sid in zip(sessions, ll, ids):
        want, rng = plain_runs(gen, s["data"], s["n"], s["seed"], s["pars"])
        np.testing.assert_array_equal(np.array(got), np.array(want))
        assert server.rng_state(sid, s["n"]) == rng
    server.free()


def test_server_request_errors(built):
    gen = d.sir_cases()
    rs = np.random.default_rng(14)
    p0 = sir_pars(rs)
    data = sir_data(rs, 8)
    bad = dict(p0, beta=-1.0)
    good = dict(p0, beta=0.3)
    obj = d.dust_filter_create(gen, 0, data, n_particles=50, dt=DT, seed=9)
    d.dust_likelihood_run(obj, p0)
    with pytest.raises(d.DustError) as plain_err:
        d.dust_likelihood_run(obj, bad)
    want_good = float(np.ravel(d.dust_likelihood_run(obj, good))[0])

    server = d.dust_likelihood_server(gen, hbm_budget=1e8, max_sessions=4)
    sid = server.open(p0, data, 50, dt=DT, seed=9)
    server.likelihood(sid, p0)
    with pytest.raises(d.DustError) as served_err:
        server.likelihood(sid, bad)
    assert str(served_err.value) == str(plain_err.value)
    # the session carries on, as the plain object does
    assert server.likelihood(sid, good) == want_good
    server.free()


def test_server_handles(built):
    gen = d.sir_cases()
    rs = np.random.default_rng(15)
    server = d.dust_likelihood_server(gen, hbm_budget=1e8, max_sessions=2)
    with pytest.raises(d.DustError, match="Unknown or closed session"):
        server.submit(12345, None)
    sid = server.open(sir_pars(rs), sir_data(rs, 5), 10, dt=DT, seed=1)
    server.close(sid)
    with pytest.raises(d.DustError, match="Unknown or closed session"):
        server.submit(sid, None)
    with pytest.raises(d.DustError, match="Unknown request"):
        server.wait(999)
    with pytest.raises(d.DustError, match="more device memory"):
        server.open(sir_pars(rs), sir_data(rs, 5), 10**8, dt=DT, seed=1)
    # a pending request reports that it is pending
    sid = server.open(sir_pars(rs), sir_data(rs, 200), 5000, dt=DT, seed=2)
    t = server.submit(sid, None)
    res = server.wait(t, timeout=0.0)
    assert res is None or np.isfinite(res[0])
    if res is None:
        assert np.isfinite(server.wait(t)[0])
    server.free()
    with pytest.raises(d.DustError, match="Can't serve"):
        d.dust_likelihood_server(d.sirode())
