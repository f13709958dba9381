"""dopri5 on the GPU against dust2's own solver (fixtures), the analytic
logistic solution and the oracle (tests/testthat/test-logistic.R,
test-sirode.R).  Solutions agree within the solver tolerance: the GPU
solver evaluates its stage sums as fused multiply-adds and the step
controller's powers with the engine's exp and log, so it rounds
differently from the CPU; in practice they agree to ~1e-13 with the
same step counts."""

import numpy as np
import pytest

import dust2_gb300 as d
from conftest import golden

pytestmark = pytest.mark.gpu


def test_sirode_matches_reference_engine(built):
    g = golden("ode_sirode")
    gen = d.sirode()
    pars = [{"beta": 0.2, "gamma": 0.1, "N": 1000, "I0": 10},
            {"beta": 0.4, "gamma": 0.05, "N": 1e6, "I0": 50}]
    sys = d.dust_system_create(gen, pars, n_particles=2, n_groups=2,
                               deterministic=True)
    d.dust_system_set_state_initial(sys)
    res = d.dust_system_simulate(sys, g["times"])
    got = res.transpose(3, 2, 1, 0).ravel()
    np.testing.assert_allclose(got, g["out"], rtol=1e-6, atol=1e-6)
    # close to bit-identical in practice
    assert np.max(np.abs(got - g["out"]) / np.maximum(1, np.abs(g["out"]))) \
        < 1e-12
    stats = d.dust_system_internals(sys)
    np.testing.assert_array_equal(stats["n_steps"], g["stats"][:, 0])
    np.testing.assert_array_equal(stats["n_steps_accepted"], g["stats"][:, 1])
    np.testing.assert_array_equal(stats["n_steps_rejected"], g["stats"][:, 2])


def logistic_analytic(r, k, t, y0):
    y = k / (1 + (k / y0 - 1) * np.exp(-np.outer(t, r)))
    return np.column_stack([y, y.sum(axis=1)])


def test_logistic_analytic_and_reference(built):
    """test-logistic.R:1-25."""
    g = golden("ode_logistic")
    pars = {"n": 3, "r": [0.1, 0.2, 0.3], "K": [100, 100, 100]}
    sys = d.dust_system_create(d.logistic(), pars, n_particles=1,
                               preserve_particle_dimension=True,
                               deterministic=True)
    np.testing.assert_array_equal(d.dust_system_state(sys), np.zeros((4, 1)))
    d.dust_system_set_state_initial(sys)
    np.testing.assert_array_equal(d.dust_system_state(sys),
                                  np.array([[1.0], [1], [1], [3]]))
    d.dust_system_run_to_time(sys, 10)
    s = d.dust_system_state(sys)[:, 0]
    expect = logistic_analytic(np.array(pars["r"]), 100, np.array([10.0]),
                               1)[0]
    np.testing.assert_allclose(s, expect, rtol=1e-6)
    sys2 = d.dust_system_create(d.logistic(), pars, n_particles=1,
                                deterministic=True)
    d.dust_system_set_state_initial(sys2)
    res = d.dust_system_simulate(sys2, g["times"])
    np.testing.assert_allclose(res.T.ravel(), g["out"], rtol=1e-12, atol=0)


def test_critical_times(built):
    """test-sirode.R:119-142."""
    g = golden("ode_sirode_critical")
    pars = {"beta": 0.2, "gamma": 0.1, "N": 1000, "I0": 10}
    ctl1 = d.dust_ode_control(critical_times=[10, 20, 30],
                              debug_record_step_times=True)
    ctl2 = d.dust_ode_control(debug_record_step_times=True)
    s1 = d.dust_system_create(d.sirode(), pars, ode_control=ctl1,
                              deterministic=True)
    s2 = d.dust_system_create(d.sirode(), pars, ode_control=ctl2,
                              deterministic=True)
    for s in (s1, s2):
        d.dust_system_set_state_initial(s)
        d.dust_system_run_to_time(s, 50)
    t1 = d.dust_system_internals(s1)["step_times"][0]
    t2 = d.dust_system_internals(s2)["step_times"][0]
    assert all(x in t1 for x in (10, 20, 30))
    assert not all(x in t2 for x in (10, 20, 30))
    np.testing.assert_allclose(d.dust_system_state(s1),
                               d.dust_system_state(s2), rtol=1e-6)
    np.testing.assert_allclose(d.dust_system_state(s1),
                               g["out"][-5:], rtol=1e-12)


def test_too_many_steps_error(built):
    """test-sirode.R:67-102."""
    pars = {"beta": 0.2, "gamma": 0.1, "N": 1000, "I0": 10}
    sys = d.dust_system_create(d.sirode(), pars, n_particles=10,
                               ode_control=d.dust_ode_control(max_steps=5),
                               deterministic=True)
    d.dust_system_set_state_initial(sys)
    with pytest.raises(d.DustError, match="10 particles reported errors") as e:
        d.dust_system_run_to_time(sys, 30)
    assert "1: too many steps" in str(e.value)
    assert "- (and 6 more)" in str(e.value)
    with pytest.raises(d.DustError, match="errors are pending"):
        d.dust_system_run_to_time(sys, 30)
    d.dust_system_update_pars(sys, {"gamma": 0.2})
    d.dust_system_set_state_initial(sys)
    assert d.dust_system_time(sys) == 0


def test_incidence_is_daily(built):
    """test-sirode.R:1-16: cumulative cases equal summed daily incidence."""
    pars = {"beta": 0.2, "gamma": 0.1, "N": 1000, "I0": 10}
    sys = d.dust_system_create(d.sirode(), pars, n_particles=1,
                               preserve_particle_dimension=True,
                               ode_control=d.dust_ode_control(
                                   step_size_max=0.8), deterministic=True)
    d.dust_system_set_state_initial(sys)
    res = d.dust_system_simulate(sys, np.arange(0, 11))
    assert np.all(np.diff(res[3, 0]) >= 0)
    np.testing.assert_allclose(np.cumsum(res[4, 0]), res[3, 0], rtol=1e-10)


def test_many_instances_match_oracle(port):
    """A batch of instances with different parameters, as in the dopri5
    workload, against the CPU restatement."""
    rs = np.random.default_rng(3)
    n = 512
    plist = [{"beta": float(rs.uniform(0.1, 0.5)),
              "gamma": float(rs.uniform(0.05, 0.2)), "N": 1e6,
              "I0": float(rs.uniform(1, 100))} for _ in range(n)]
    gen = d.sirode()
    flat = np.concatenate([gen.pack_pars(p) for p in plist])
    times = np.arange(0, 201, dtype=float)
    sys = d.dust_system_create(gen, plist, n_particles=1, n_groups=n,
                               deterministic=True)
    d.dust_system_set_state_initial(sys)
    res = d.dust_system_simulate(sys, times)
    out, stats = port.ode_simulate("sirode", flat, n, 1, 0.0, times, 5,
                                   n_threads=port.max_threads())
    # ungrouped-particle layout: (state, group, time)
    got = res.reshape(5, n, times.size).transpose(2, 1, 0).ravel()
    np.testing.assert_allclose(got, out, rtol=1e-6, atol=1e-6)
    internals = d.dust_system_internals(sys)
    frac_same = np.mean(internals["n_steps"] == stats[:, 0])
    assert frac_same > 0.99
