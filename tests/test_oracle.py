"""The CPU oracle pinned to dust2's own engine.

Where the reference sources are present, the CPU restatement
(oracle/port) is checked bit for bit against dust2's engine compiled from
those sources (oracle/ref_driver.cpp).  Everywhere, the restatement is
checked against the golden fixtures that engine produced
(tests/golden/make_golden.py)."""

import numpy as np
import pytest

import dust2_gb300
import xoshiro
import workload_data
from conftest import golden


def test_port_filter_matches_golden(port):
    for name in ("filter_sir_2groups", "filter_sir_missing"):
        g = golden(name)
        n = int(g["n_particles"])
        ll, state, rng = port.filter_run(
            "sir", g["pars"], [n, n], 0.0, g["times"], g["data"], 2,
            float(g["dt"]), g["rng"], n_runs=g["ll"].shape[0], n_state=5)
        np.testing.assert_array_equal(ll, g["ll"])
        np.testing.assert_array_equal(state[:2 * n * 5], g["state"])
        np.testing.assert_array_equal(rng, g["rng_out"])


def test_port_single_group_workload_matches_golden(port):
    g = golden("filter_sir_cases_1000")
    n = int(g["n_particles"])
    ll, state, rng = port.filter_run("sir_cases", g["pars"], [n], 0.0,
                                     g["times"], g["data"], 1, float(g["dt"]),
                                     g["rng"], n_runs=g["ll"].shape[0],
                                     n_state=4)
    np.testing.assert_array_equal(ll, g["ll"])
    np.testing.assert_array_equal(state[:n * 4], g["state"])
    np.testing.assert_array_equal(rng, g["rng_out"])


@pytest.mark.parametrize("name", ["sir", "walk", "seir_age"])
def test_port_simulate_matches_golden(port, name):
    g = golden(f"simulate_{name}")
    out, rng = port.discrete_simulate(name, g["pars"], int(g["n_groups"]),
                                      int(g["n_particles"]), 0.0,
                                      float(g["dt"]), g["rng"], g["times"])
    np.testing.assert_array_equal(out[:g["out"].size], g["out"])
    np.testing.assert_array_equal(rng, g["rng_out"])


def test_port_compare_matches_golden(port):
    g = golden("compare_sir")
    out, rng = port.compare("sir", g["pars"], 1, 10, 0.0, g["state"],
                            np.array([30.0]), 1, g["rng"])
    np.testing.assert_array_equal(out, g["out"])
    np.testing.assert_array_equal(rng, g["rng_out"])


def test_port_ode_matches_golden(port):
    g = golden("ode_sirode")
    out, stats = port.ode_simulate("sirode", g["pars"], 2, 2, 0.0,
                                   g["times"], 5)
    np.testing.assert_array_equal(out, g["out"])
    np.testing.assert_array_equal(stats, g["stats"])
    g = golden("ode_logistic")
    out, stats = port.ode_simulate("logistic", g["pars"], 1, 1, 0.0,
                                   g["times"], 4)
    np.testing.assert_array_equal(out, g["out"])
    g = golden("ode_sirode_critical")
    out, stats = port.ode_simulate(
        "sirode", workload_data.pack(
            "sirode", [{"beta": 0.2, "gamma": 0.1, "N": 1000, "I0": 10}]),
        1, 1, 0.0, np.array([0.0, 50.0]), 5, critical_times=[10, 20, 30])
    np.testing.assert_array_equal(out, g["out"])


def test_port_details_match_golden(port):
    g = golden("filter_details")
    for u, idx in zip(g["u"], g["idx"]):
        np.testing.assert_array_equal(port.resample_weight(g["w"], u), idx)
    r1, w1 = port.scale_log_weights(g["lw"])
    assert r1 == g["lw_ret"][0]
    np.testing.assert_array_equal(w1, g["lw_w1"])
    r2, w2 = port.scale_log_weights(np.full(5, -np.inf))
    assert r2 == g["lw_ret"][1] == -np.inf
    np.testing.assert_array_equal(w2, g["lw_w2"])
    r3, w3 = port.scale_log_weights(np.array([-3.5]))
    assert r3 == g["lw_ret"][2] == -3.5


def test_resample_matches_find_interval(port):
    """tests/testthat/test-filter-details.R:1-22: systematic resampling is
    findInterval(u/n + (i-1)/n, cumsum(w/sum(w)))."""
    rs = np.random.default_rng(1)
    w = np.abs(rs.standard_cauchy(20))
    for u in (rs.uniform(), 0.0, 1 - 1e-8):
        n = w.size
        uu = u / n + np.arange(n) / n
        cw = np.cumsum(w / w.sum())
        expect = np.searchsorted(cw, uu, side="right")
        np.testing.assert_array_equal(port.resample_weight(w, u), expect)


def test_scale_log_weights_semantics(port):
    """test-filter-details.R:55-64: NaN -> zero weight; all -Inf -> -Inf."""
    w = np.array([-1.0, np.nan, -2.0, -3.0])
    r, ww = port.scale_log_weights(w)
    m = -1.0
    expect = np.log(np.mean(np.exp(np.array([-1.0, -2, -3]) - m)
                            * np.array([1, 1, 1])) * 3 / 4) + m
    assert abs(r - expect) < 1e-14
    assert ww[1] == 0


# ---- the restatement against dust2's own engine (reference present) ----

def _uneven_inputs(seed, G, n, T):
    rs = np.random.default_rng(seed)
    plist = [{"N": 1e5, "I0": float(rs.integers(5, 50)),
              "beta": float(rs.uniform(0.15, 0.5)),
              "gamma": float(rs.uniform(0.05, 0.2))} for _ in range(G)]
    times = np.arange(1, T + 1, dtype=float)
    data = rs.poisson(20, size=(T, G)).astype(float)
    data[rs.uniform(size=data.shape) < 0.05] = np.nan
    return workload_data.pack("sir_cases", plist), times, data


@pytest.mark.parametrize("G,n,dt", [(1, 1, 1.0), (3, 257, 0.25),
                                    (2, 2000, 0.5)])
def test_port_filter_equals_reference_engine(port, ref, G, n, dt):
    pars, times, data = _uneven_inputs(G * n, G, n, 20)
    rng = xoshiro.streams(G + n, G * (n + 2))
    a = port.filter_run("sir_cases", pars, [n] * G, 0.0, times,
                        data.ravel(), G, dt, rng, n_runs=3, n_state=4)
    b = ref.filter_run("sir_cases", pars, [n] * G, 0.0, times, data.ravel(),
                       G, dt, rng, n_runs=3, n_state=4)
    np.testing.assert_array_equal(a[0], b[0])
    np.testing.assert_array_equal(a[1][:G * n * 4], b[1][:G * n * 4])
    np.testing.assert_array_equal(a[2], b[2])


def test_port_threads_do_not_change_results(port):
    pars, times, data = _uneven_inputs(4, 3, 500, 15)
    rng = xoshiro.streams(1, 3 * 502)
    a = port.filter_run("sir_cases", pars, [500] * 3, 0.0, times,
                        data.ravel(), 3, 0.25, rng, n_state=4, n_threads=1)
    b = port.filter_run("sir_cases", pars, [500] * 3, 0.0, times,
                        data.ravel(), 3, 0.25, rng, n_state=4,
                        n_threads=port.max_threads())
    for x, y in zip(a, b):
        np.testing.assert_array_equal(x, y)


def test_port_seir_equals_reference_engine(port, ref):
    from dust2_gb300 import workloads
    pars = workload_data.pack("seir_age", workloads.seir_plist([1.5, 2.5]))
    rng = xoshiro.streams(3, 2 * 5)
    tt = np.arange(0, 31, dtype=float)
    a = port.discrete_simulate("seir_age", pars, 2, 5, 0.0, 0.25, rng, tt)
    b = ref.discrete_simulate("seir_age", pars, 2, 5, 0.0, 0.25, rng, tt)
    np.testing.assert_array_equal(a[0][:tt.size * 10 * 96],
                                  b[0][:tt.size * 10 * 96])
    np.testing.assert_array_equal(a[1], b[1])


def test_port_ode_equals_reference_engine(port, ref):
    rs = np.random.default_rng(2)
    plist = [{"beta": float(rs.uniform(0.1, 0.5)),
              "gamma": float(rs.uniform(0.05, 0.2)), "N": 1e6,
              "I0": float(rs.uniform(1, 100))} for _ in range(20)]
    pars = workload_data.pack("sirode", plist)
    tt = np.arange(0, 201, dtype=float)
    a = port.ode_simulate("sirode", pars, 20, 1, 0.0, tt, 5)
    b = ref.ode_simulate("sirode", pars, 20, 1, 0.0, tt, 5)
    np.testing.assert_array_equal(a[0], b[0])
    np.testing.assert_array_equal(a[1], b[1])


def test_port_errors_match_reference_engine(port, ref):
    pars = workload_data.pack("sir", [{"gamma": -0.2}])
    rng = xoshiro.streams(42, 10)
    with pytest.raises(Exception) as e1:
        port.discrete_simulate("sir", pars, 1, 10, 0.0, 1.0, rng, [30.0])
    with pytest.raises(Exception) as e2:
        ref.discrete_simulate("sir", pars, 1, 10, 0.0, 1.0, rng, [30.0])
    assert str(e1.value) == str(e2.value)
    assert str(e1.value).startswith("10 particles reported errors.")
    assert "(and 6 more)" in str(e1.value)


@pytest.mark.parametrize("name", ["sir", "sirode"])
def test_port_unfilter_equals_reference_engine(port, name):
    g = golden(f"unfilter_{name}")
    n_particles = 3 if name == "sir" else 2
    ll, state = port.unfilter_run(name, g["pars"], 2, n_particles, 0.0,
                                  g["times"], g["data"], 2, 5, dt=0.25,
                                  n_runs=2, n_threads=2)
    np.testing.assert_array_equal(ll, g["ll"])
    np.testing.assert_array_equal(state, g["state"])


ADJOINT_LABELS = ["four_days", "odd_steps", "four_groups", "quarter_days",
                  "late_start"]


def _adjoint_case(g, label):
    n_groups, t0, dt, ngd = g[f"{label}__meta"]
    return (g[f"{label}__pars"], int(n_groups), float(t0),
            g[f"{label}__times"], g[f"{label}__data"], int(ngd), float(dt))


@pytest.mark.parametrize("label", ADJOINT_LABELS)
def test_port_adjoint_equals_reference_engine(port, label):
    g = golden("adjoint_sir")
    pars, G, t0, times, data, ngd, dt = _adjoint_case(g, label)
    ll, gr, state = port.unfilter_adjoint("sir", pars, G, 1, t0, times,
                                          data, ngd, 5, dt=dt)
    np.testing.assert_array_equal(ll, g[f"{label}__ll"])
    np.testing.assert_array_equal(gr, g[f"{label}__gradient"])
    np.testing.assert_array_equal(state, g[f"{label}__state"])
    # the adjoint run's log-likelihood is the plain run's
    ll_plain, _ = port.unfilter_run("sir", pars, G, 1, t0, times, data, ngd,
                                    5, dt=dt)
    np.testing.assert_array_equal(ll_plain[0], ll)


def test_reference_adjoint_reproduces_fixture(ref):
    g = golden("adjoint_sir")
    for label in ADJOINT_LABELS:
        pars, G, t0, times, data, ngd, dt = _adjoint_case(g, label)
        ll, gr, _ = ref.unfilter_adjoint("sir", pars, G, 1, t0, times, data,
                                         ngd, 5, dt=dt)
        np.testing.assert_array_equal(ll, g[f"{label}__ll"])
        np.testing.assert_array_equal(gr, g[f"{label}__gradient"])


@pytest.mark.parametrize("label", ["four_days", "odd_steps"])
def test_adjoint_gradient_matches_finite_differences(port, label):
    """test-unfilter-adjoint.R "can run the adjoint model": the gradient
    in (beta, gamma, I0) against central differences of the plain
    likelihood, compared as R's all.equal does (sum of absolute
    differences over sum of absolute values) to 1e-4.  At dt = 1 the
    model's adjoint is exact in beta and gamma; its I0 entry leaves out
    the S = N - I0 dependence, which this tolerance allows, as in the
    reference's own test."""
    g = golden("adjoint_sir")
    pars, G, t0, times, data, ngd, dt = _adjoint_case(g, label)
    names = [p["name"] for p in dust2_gb300.sir().parameters]
    idx = [names.index(n) for n in ("beta", "gamma", "I0")]
    _, gr, _ = port.unfilter_adjoint("sir", pars, G, 1, t0, times, data,
                                     ngd, 5, dt=dt)

    def f(x):
        p = np.array(pars, dtype=float)
        p[idx] = x
        ll, _ = port.unfilter_run("sir", p, 1, 1, t0, times, data, ngd, 5,
                                  dt=dt)
        return ll.ravel()[0]

    x0 = np.asarray(pars, dtype=float)[idx]
    num = np.empty(3)
    for i in range(3):
        h = 1e-5 * max(1.0, abs(x0[i]))
        e = np.zeros(3)
        e[i] = h
        num[i] = (f(x0 + e) - f(x0 - e)) / (2 * h)
    got = gr.ravel()
    assert np.sum(np.abs(num - got)) / np.sum(np.abs(num)) < 1e-4
    np.testing.assert_allclose(got[:2], num[:2], rtol=1e-6)


def test_port_adjoint_particles_agree(port):
    """Several particles per group (the engine's extension): each carries
    the one-particle gradient of its group."""
    g = golden("adjoint_sir")
    pars, G, t0, times, data, ngd, dt = _adjoint_case(g, "four_groups")
    ll1, gr1, _ = port.unfilter_adjoint("sir", pars, G, 1, t0, times, data,
                                        ngd, 5, dt=dt)
    ll5, gr5, _ = port.unfilter_adjoint("sir", pars, G, 5, t0, times, data,
                                        ngd, 5, dt=dt)
    np.testing.assert_array_equal(ll5, np.repeat(ll1, 5, axis=1))
    np.testing.assert_array_equal(gr5, np.repeat(gr1, 5, axis=1))


def test_port_unfilter_states_equal_reference_trajectories(port):
    """The deterministic run's state at each data time is what dust2's
    unfilter saves as trajectories and snapshots (run and run_adjoint
    alike)."""
    t = golden("unfilter_trajectories")
    g = golden("unfilter_sir")
    ll, states = port.unfilter_states("sir", g["pars"], 2, 3, 0.0,
                                      g["times"], g["data"], 2, 5, dt=0.25)
    np.testing.assert_array_equal(ll, t["ll"])
    np.testing.assert_array_equal(states, t["full"])
    np.testing.assert_array_equal(states[..., [1, 3]], t["sub"])
    snap_at = np.searchsorted(g["times"], t["snapshots"])
    np.testing.assert_array_equal(states[snap_at], t["snap"])
    np.testing.assert_array_equal(t["full_adjoint"], t["full"])
    np.testing.assert_array_equal(t["snap_adjoint"], t["snap"])
    np.testing.assert_array_equal(t["ll_adjoint"], t["ll"])
    g = golden("unfilter_sirode")
    ll, states = port.unfilter_states("sirode", g["pars"], 2, 2, 0.0,
                                      g["times"], g["data"], 2, 5)
    np.testing.assert_array_equal(ll, t["ll_ode"])
    np.testing.assert_array_equal(states, t["full_ode"])
    snap_at = np.searchsorted(g["times"], t["ode_snapshots"])
    np.testing.assert_array_equal(states[snap_at], t["snap_ode"])


@pytest.mark.parametrize("label,dt", [("ode_only", 0.0), ("daily", 1.0),
                                      ("coarse", 1.0), ("uneven", 2.0)])
def test_port_mixed_simulate_equals_reference_engine(port, label, dt):
    """Mixed time (continuous/system.hpp:544-585): the restatement against
    dust2's own dust_continuous, exactly (same arithmetic, same pow)."""
    g = golden("mixed_malaria")
    times = {"ode_only": np.arange(21.0), "daily": np.arange(21.0),
             "coarse": np.array([4.0, 8, 12, 16]),
             "uneven": np.array([3.0, 5, 9, 10, 16])}[label]
    y, stats = port.mixed_simulate("malaria", g["sim_pars"], 2, 4, 0.0, dt,
                                   g["sim_rng"], times, 20)
    np.testing.assert_array_equal(y, g[f"sim_{label}"])
    np.testing.assert_array_equal(stats, g[f"sim_{label}_stats"])


def test_reference_mixed_filter_reproduces_fixture(ref):
    g = golden("mixed_malaria")
    ll, state, rng_out = ref.mixed_filter_run(
        "malaria", g["f1_pars"], 1, 100, 0.0, g["f1_times"],
        g["f1_data"].ravel(), 1, 1.0, g["f1_rng"], 20, n_runs=5)
    np.testing.assert_array_equal(ll, g["f1_ll"])
    np.testing.assert_array_equal(rng_out, g["f1_rng_out"])


def test_port_trajectories_equal_reference_engine(port):
    g = golden("trajectories_sir")
    args = ("sir", g["pars"], 2, int(g["n_particles"]), 0.0, g["times"],
            g["data"], 2, 1.0, g["rng"])
    ll, full, _, snap = port.filter_trajectories(
        *args, 5, snapshots=g["snapshots"])
    np.testing.assert_array_equal(ll, g["ll"])
    np.testing.assert_array_equal(full, g["full"])
    np.testing.assert_array_equal(snap, g["snap"])
    _, sub, _, _ = port.filter_trajectories(*args, 2, index_state=[1, 3])
    np.testing.assert_array_equal(sub, g["sub"])
    _, one, _, snap_one = port.filter_trajectories(
        *args, 5, select=g["select"], snapshots=g["snapshots"])
    np.testing.assert_array_equal(one, g["one"])
    np.testing.assert_array_equal(snap_one, g["snap_one"])
