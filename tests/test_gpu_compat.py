"""The sirs system, a class written in dust2's own shape (cpp11::list
readers, monty samplers, dust2::packing and zero_every_type) and adapted
by compat/plugin.hpp, runs on the GPU through the same verbs as the
native systems: simulate and the particle filter equal the CPU oracle
running the same class (state and generators exactly, log-likelihoods to
1e-12 relative), and its parameter reader keeps dust2's semantics."""

import numpy as np
import pytest

import dust2_gb300 as d

pytestmark = pytest.mark.gpu

PARS = {"N": 5000, "I0": 20, "beta": 0.4, "gamma": 0.1, "omega": 0.02,
        "kappa": 8}


def test_sirs_simulate_matches_oracle(port):
    gen = d.sirs()
    n, G = 300, 2
    plist = [PARS, dict(PARS, beta=0.25)]
    sys = d.dust_system_create(gen, plist, n_particles=n, n_groups=G,
                               dt=0.25, seed=9)
    words = np.frombuffer(d.dust_system_rng_state(sys), dtype="<u8")
    d.dust_system_set_state_initial(sys)
    times = np.arange(1, 41, dtype=float)
    got = d.dust_system_simulate(sys, times)  # [state, particle, group, time]
    flat = np.concatenate([gen.pack_pars(p) for p in plist])
    want, rng_out = port.discrete_simulate("sirs", flat, G, n, 0.0, 0.25,
                                           words, times)
    want = want[:times.size * G * n * 4].reshape(times.size, G, n, 4)
    np.testing.assert_array_equal(np.asarray(got).transpose(3, 2, 1, 0),
                                  want)
    np.testing.assert_array_equal(
        np.frombuffer(d.dust_system_rng_state(sys), dtype="<u8"), rng_out)


def test_sirs_filter_matches_oracle(port):
    gen = d.sirs()
    rs = np.random.default_rng(3)
    times = np.arange(1, 61, dtype=float)
    cases = rs.poisson(30, times.size).astype(float)
    cases[[4, 17]] = np.nan  # missing data compare to 0
    obj = d.dust_filter_create(gen, 0, {"time": times, "cases": cases},
                               n_particles=700, dt=0.25, seed=5)
    words = np.frombuffer(d.dust_likelihood_rng_state(obj), dtype="<u8")
    ll = d.dust_likelihood_run(obj, PARS)
    state = np.asarray(d.dust_likelihood_last_state(obj)).T.ravel()
    after = np.frombuffer(d.dust_likelihood_rng_state(obj), dtype="<u8")
    want, want_state, want_rng = port.filter_run(
        "sirs", gen.pack_pars(PARS), [700], 0.0, times, cases, 1, 0.25,
        words, n_state=4, n_threads=port.max_threads())
    np.testing.assert_allclose(ll, want[0][0], rtol=1e-12, atol=0)
    np.testing.assert_array_equal(state, want_state[:700 * 4])
    np.testing.assert_array_equal(after, want_rng)


def test_sirs_parameter_reader_semantics():
    gen = d.sirs()
    # beta has no default in the class (read_real without one)
    with pytest.raises(d.DustError, match="A value is expected for 'beta'"):
        d.dust_system_create(gen, {"N": 100}, n_particles=4, dt=1)
    sys = d.dust_system_create(gen, PARS, n_particles=4, dt=1, seed=1)
    d.dust_system_set_state_initial(sys)
    s0 = np.asarray(d.dust_system_state(sys))
    assert s0.shape[0] == 4
    np.testing.assert_array_equal(s0[:, 0], [4980, 20, 0, 0])
    # update_pars keeps what is not given (the class reads the current
    # value as the default)
    d.dust_system_update_pars(sys, {"I0": 50})
    d.dust_system_set_state_initial(sys)
    np.testing.assert_array_equal(np.asarray(d.dust_system_state(sys))[:, 0],
                                  [4950, 50, 0, 0])
