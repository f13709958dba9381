"""Mixed-time systems on the GPU (an ODE with a discrete-time update every
dt; continuous/system.hpp:80-106, 544-585) against dust2's own
dust_continuous and filter (golden fixtures from
tests/golden/make_golden.py, tests/testthat/test-malaria.R and
test-filter.R "can run filter on mixed time models" are the model).

Tolerance: 1e-9 relative.  The update and the compare are exact; the
GPU solver's stage sums are fused multiply-adds and its step-size
controller's powers come from the engine's exp and log, so its rounding
differs from the CPU's (as for the pure ODE systems, where agreement is
~1e-13).
Generator states are compared exactly."""

import numpy as np
import pytest

import dust2_gb300 as d
from conftest import golden

pytestmark = pytest.mark.gpu

CASES = [("ode_only", None), ("daily", 1.0), ("coarse", 1.0),
         ("uneven", 2.0)]
TIMES = {"ode_only": np.arange(21.0), "daily": np.arange(21.0),
         "coarse": np.array([4.0, 8, 12, 16]),
         "uneven": np.array([3.0, 5, 9, 10, 16])}


def plist(gen, flat, n_groups):
    out = []
    for row in np.asarray(flat).reshape(n_groups, gen.n_pars):
        p = {}
        off = 0
        for par in gen.parameters:
            v = row[off:off + par["length"]]
            if not np.isnan(v[0]):
                p[par["name"]] = float(v[0])
            off += par["length"]
        out.append(p)
    return out


@pytest.mark.parametrize("label,dt", CASES)
def test_mixed_simulate_matches_reference(built, label, dt):
    g = golden("mixed_malaria")
    gen = d.malaria()
    sys = d.dust_system_create(gen, plist(gen, g["sim_pars"], 2),
                               n_particles=4, n_groups=2, dt=dt, seed=13)
    assert d.dust_system_rng_state(sys) == g["sim_rng"].astype("<u8") \
        .tobytes()
    d.dust_system_set_state_initial(sys)
    res = d.dust_system_simulate(sys, TIMES[label])
    got = res.transpose(3, 2, 1, 0)
    want = g[f"sim_{label}"]
    np.testing.assert_allclose(got, want, rtol=1e-9, atol=1e-12)
    stats = d.dust_system_internals(sys)
    same = np.mean(stats["n_steps"] == g[f"sim_{label}_stats"][:, 0])
    assert same >= 0.75
    # the particles' generators never advance in a mixed-time run
    assert d.dust_system_rng_state(sys) == g["sim_rng"].astype("<u8") \
        .tobytes()


def test_mixed_without_dt_is_the_ode(built):
    """test-malaria.R "can run model without any stochastic updates":
    beta stays at -log(0.9) and all particles agree."""
    sys = d.dust_system_create(d.malaria(), {}, n_particles=10)
    d.dust_system_set_state_initial(sys)
    y = d.dust_system_simulate(sys, np.arange(21.0))
    assert y.shape == (20, 10, 21)
    np.testing.assert_array_equal(y, y[:, [0] * 10, :])
    yy = d.dust_unpack_state(sys, y)
    assert list(yy) == ["Sh", "Ih", "Sv", "Iv", "Ev", "beta"]
    assert yy["Ev"].shape == (15, 10, 21) and yy["beta"].shape == (10, 21)
    np.testing.assert_allclose(yy["beta"], np.log(10 / 9), rtol=1e-15)
    idx = d.dust_unpack_index(sys)
    assert list(idx["Ev"]) == list(range(5, 20)) and list(idx["beta"]) == [20]


def test_mixed_updates_between_runs_match_ode_segments(built):
    """test-malaria.R "can apply stochastic updates by setting dt": with
    dt = 1 and daily outputs, every day is the ODE from the last output."""
    sys = d.dust_system_create(d.malaria(), {}, n_particles=10, dt=1,
                               seed=3)
    d.dust_system_set_state_initial(sys)
    t = np.arange(21.0)
    y = d.dust_system_simulate(sys, t)
    sys0 = d.dust_system_create(d.malaria(), {}, n_particles=10)
    for i in range(t.size - 1):
        d.dust_system_set_state(sys0, y[:, :, i])
        d.dust_system_run_to_time(sys0, t[i + 1])
        y0 = d.dust_system_state(sys0)
        np.testing.assert_allclose(y0[:-1], y[:-1, :, i + 1], rtol=1e-9)


def test_mixed_compare_data(built):
    """test-malaria.R "Can compare to data": the binomial log density of
    the positives among the tested at the human prevalence."""
    from scipy.stats import binom
    sys = d.dust_system_create(d.malaria(), {}, n_particles=10, dt=1,
                               seed=1)
    d.dust_system_set_state_initial(sys)
    d.dust_system_run_to_time(sys, 10)
    s = d.dust_system_state(sys)
    got = d.dust_system_compare_data(sys, {"tested": 4, "positive": 2})
    np.testing.assert_allclose(got, binom.logpmf(2, 4, s[1]), rtol=1e-12)


def test_mixed_filter_matches_reference(built):
    g = golden("mixed_malaria")
    gen = d.malaria()
    data = {"time": g["f1_times"], "tested": g["f1_data"][:, 0],
            "positive": g["f1_data"][:, 1]}
    obj = d.dust_filter_create(gen, 0, data, n_particles=100, dt=1, seed=42)
    ll = [d.dust_likelihood_run(obj, {}) for _ in range(5)]
    np.testing.assert_allclose(np.ravel(ll), g["f1_ll"].ravel(), rtol=1e-9)
    assert d.dust_likelihood_rng_state(obj) == \
        g["f1_rng_out"].astype("<u8").tobytes()
    state = d.dust_likelihood_last_state(obj)
    np.testing.assert_allclose(state.T, g["f1_state"][0], rtol=1e-9,
                               atol=1e-12)


def test_mixed_filter_groups_match_reference(built):
    """3 groups x 40 particles, per-group data, dt = 0.5: resampling moves
    each particle's solver record with its state."""
    g = golden("mixed_malaria")
    gen = d.malaria()
    times = g["f3_times"]
    rows = g["f3_data"]
    data = {"time": np.repeat(times, 3),
            "tested": rows[:, :, 0].ravel(), "positive": rows[:, :, 1].ravel(),
            "group": np.tile([1, 2, 3], times.size)}
    obj = d.dust_filter_create(gen, 0, data, n_particles=40, dt=0.5, seed=5)
    pars = plist(gen, g["f3_pars"], 3)
    ll = [d.dust_likelihood_run(obj, pars if r == 0 else None)
          for r in range(3)]
    np.testing.assert_allclose(np.array(ll), g["f3_ll"], rtol=1e-9)
    assert d.dust_likelihood_rng_state(obj) == \
        g["f3_rng_out"].astype("<u8").tobytes()


def test_mixed_unfilter_matches_reference(built):
    g = golden("mixed_malaria")
    gen = d.malaria()
    times = g["u_times"]
    data = {"time": np.repeat(times, 2),
            "tested": np.repeat(g["u_data"][:, 0], 2),
            "positive": np.repeat(g["u_data"][:, 1], 2),
            "group": np.tile([1, 2], times.size)}
    obj = d.dust_unfilter_create(gen, 0, data, dt=1)
    ll = d.dust_likelihood_run(obj, plist(gen, g["sim_pars"], 2))
    np.testing.assert_allclose(np.ravel(ll), g["u_ll"].ravel(), rtol=1e-9)


def test_mixed_errors(built):
    with pytest.raises(d.DustError, match="continuous-time models"):
        d.dust_filter_create(d.sirode(), 0, {"time": [1.0, 2.0],
                                             "incidence": [1.0, 2.0]},
                             n_particles=10)
    with pytest.raises(d.DustError, match="'n_rates' must be an integer"):
        d.dust_system_create(d.malaria(), {"n_rates": 40}, n_particles=2)
