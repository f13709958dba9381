"""Batched stepping on the GPU against dust2's own engine (fixtures) and
the CPU oracle; behaviour of the system verbs as in
tests/testthat/test-sir.R and test-walk.R.  State and generator state are
compared exactly."""

import numpy as np
import pytest

import dust2_gb300 as d
import xoshiro
from conftest import golden

pytestmark = pytest.mark.gpu


def plist_from(gen, flat, n_groups):
    out = []
    for row in np.asarray(flat).reshape(n_groups, gen.n_pars):
        p = {}
        off = 0
        for par in gen.parameters:
            v = row[off:off + par["length"]]
            if not np.isnan(v[0]):
                p[par["name"]] = v[0] if par["length"] == 1 else v
            off += par["length"]
        out.append(p)
    return out


@pytest.mark.parametrize("name", ["sir", "walk", "seir_age"])
def test_simulate_matches_reference_engine(built, name):
    g = golden(f"simulate_{name}")
    gen = d.Generator(name)
    G, n = int(g["n_groups"]), int(g["n_particles"])
    sys = d.dust_system_create(gen, plist_from(gen, g["pars"], G),
                               n_particles=n, n_groups=G, dt=float(g["dt"]),
                               seed=g["rng"].astype("<u8").tobytes())
    d.dust_system_set_state_initial(sys)
    # the reference output starts after the first run_to_time (t = 0)
    res = d.dust_system_simulate(sys, g["times"])
    got = res.transpose(3, 2, 1, 0).ravel()
    np.testing.assert_array_equal(got, g["out"])
    rng = np.frombuffer(d.dust_system_rng_state(sys), dtype="<u8")
    np.testing.assert_array_equal(rng, g["rng_out"])


def test_run_to_time_matches_oracle(port):
    gen = d.sir_cases()
    plist = [{"beta": 0.3 + 0.05 * i, "gamma": 0.1, "N": 1e5, "I0": 20}
             for i in range(4)]
    flat = np.concatenate([gen.pack_pars(p) for p in plist])
    n = 3000
    sys = d.dust_system_create(gen, plist, n_particles=n, n_groups=4,
                               dt=0.25, seed=5)
    words = np.frombuffer(d.dust_system_rng_state(sys), dtype="<u8")
    d.dust_system_set_state_initial(sys)
    d.dust_system_run_to_time(sys, 40)
    got = d.dust_system_state(sys)
    out, rng_out = port.discrete_simulate("sir_cases", flat, 4, n, 0.0, 0.25,
                                          words, [40.0])
    np.testing.assert_array_equal(got.transpose(2, 1, 0).ravel(),
                                  out[:4 * n * 4])
    np.testing.assert_array_equal(
        np.frombuffer(d.dust_system_rng_state(sys), dtype="<u8"), rng_out)


def test_compare_matches_reference_engine(built):
    g = golden("compare_sir")
    sys = d.dust_system_create(d.sir(), {"exp_noise": 0.5}, n_particles=10,
                               seed=g["rng"].astype("<u8").tobytes())
    d.dust_system_set_state(sys, g["state"].reshape(10, 5).T)
    res = d.dust_system_compare_data(sys, {"incidence": 30})
    np.testing.assert_array_equal(res, g["out"])
    rng = np.frombuffer(d.dust_system_rng_state(sys), dtype="<u8")
    np.testing.assert_array_equal(rng, g["rng_out"])


def test_compare_missing_does_not_draw(built):
    """test-sir.R:49-62."""
    sys = d.dust_system_create(d.sir(), {"exp_noise": 0.5}, n_particles=10,
                               seed=42)
    s0 = d.dust_system_rng_state(sys)
    res = d.dust_system_compare_data(sys, {"incidence": np.nan})
    np.testing.assert_array_equal(res, np.zeros(10))
    assert d.dust_system_rng_state(sys) == s0


def test_sir_basics(built):
    """test-sir.R:1-28."""
    pars = {"beta": 0.1, "gamma": 0.2, "N": 1000, "I0": 10, "exp_noise": 1e6}
    sys = d.dust_system_create(d.sir(), pars, n_particles=10, seed=42)
    assert sys.n_state == 5
    assert len(d.dust_system_rng_state(sys)) == 32 * 10
    np.testing.assert_array_equal(d.dust_system_state(sys), np.zeros((5, 10)))
    assert d.dust_system_time(sys) == 0
    d.dust_system_set_state_initial(sys)
    np.testing.assert_array_equal(
        d.dust_system_state(sys),
        np.tile(np.array([[990.0], [10], [0], [0], [0]]), (1, 10)))
    d.dust_system_run_to_time(sys, 30)
    s1 = d.dust_system_state(sys)
    assert np.all(s1[0] < 990) and np.all(s1[2] > 0) and np.all(s1[3] > 0)


def test_incidence_resets_daily(built):
    """test-sir.R:103-120: cumulative cases equal summed daily incidence."""
    pars = {"beta": 1.0, "gamma": 0.5, "N": 1000, "I0": 10, "exp_noise": 1e6}
    sys = d.dust_system_create(d.sir(), pars, n_particles=100, seed=42)
    d.dust_system_set_state_initial(sys)
    res = d.dust_system_simulate(sys, np.arange(0, 6))
    assert np.all(np.diff(res[3], axis=1) >= 0)
    assert np.any(np.diff(res[4], axis=1) < 0)
    np.testing.assert_array_equal(np.cumsum(res[4], axis=1), res[3])


def test_errors_are_reported_and_gate_verbs(built):
    """test-sir.R:251-287."""
    pars = {"beta": 0.1, "gamma": -0.2, "N": 1000, "I0": 10, "exp_noise": 1e6}
    sys = d.dust_system_create(d.sir(), pars, n_particles=10, seed=42)
    d.dust_system_set_state_initial(sys)
    with pytest.raises(d.DustError, match="10 particles reported errors") as e:
        d.dust_system_run_to_time(sys, 30)
    assert "1: Invalid call to binomial with" in str(e.value)
    assert "- (and 6 more)" in str(e.value)
    for fn, msg in [
            (lambda: d.dust_system_run_to_time(sys, 30), "run"),
            (lambda: d.dust_system_time(sys), "get time from"),
            (lambda: d.dust_system_state(sys), "get state from"),
            (lambda: d.dust_system_reorder(sys, np.arange(1, 11)), "reorder"),
            (lambda: d.dust_system_set_time(sys, 0), "set time for"),
            (lambda: d.dust_system_compare_data(sys, {}), "compare data for"),
            (lambda: d.dust_system_simulate(sys, np.arange(0, 11)),
             "simulate")]:
        with pytest.raises(d.DustError,
                           match=f"Can't currently {msg} this system: errors "
                           "are pending"):
            fn()
    d.dust_system_update_pars(sys, {"gamma": 0.2})
    d.dust_system_set_state_initial(sys)
    assert d.dust_system_time(sys) == 0


def test_walk_deterministic_and_update_pars(built):
    """test-walk.R:59-66 and 371-386."""
    sys = d.dust_system_create(d.walk(), {"sd": 1}, n_particles=10,
                               deterministic=True)
    d.dust_system_run_to_time(sys, 3)
    np.testing.assert_array_equal(d.dust_system_state(sys), np.zeros((1, 10)))
    sys = d.dust_system_create(d.walk(), {"sd": 1, "random_initial": True},
                               n_particles=10, seed=42)
    d.dust_system_run_to_time(sys, 1)
    s1 = d.dust_system_state(sys)
    d.dust_system_update_pars(sys, {"sd": 10})
    d.dust_system_run_to_time(sys, 2)
    s2 = d.dust_system_state(sys)
    # first increment is N(0, 1), second N(0, 10) from the same streams
    streams = np.frombuffer(d.rng_streams(10, 42), dtype="<u8")
    from oracle import pyoracle
    for k in range(10):
        draws, _ = pyoracle.port_draws("normal", 0, 1, 2,
                                       streams[4 * k:4 * k + 4])
        assert s1[0, k] == draws[0]
        assert s2[0, k] == draws[0] + 10 * draws[1]


def test_reorder_and_set_state(built):
    """test-walk.R:402-425, 290-335."""
    pars = [{"sd": i, "random_initial": True, "len": 3} for i in range(1, 5)]
    sys = d.dust_system_create(d.walk(), pars, n_particles=10, n_groups=4,
                               seed=42)
    d.dust_system_set_state_initial(sys)
    s1 = d.dust_system_state(sys)
    rs = np.random.default_rng(1)
    idx = rs.integers(1, 11, size=(10, 4))
    d.dust_system_reorder(sys, idx)
    s2 = d.dust_system_state(sys)
    for j in range(4):
        np.testing.assert_array_equal(s2[:, :, j], s1[:, idx[:, j] - 1, j])
    # recycling over particles and groups
    s = np.arange(1.0, 13).reshape(3, 1, 4, order="F")
    d.dust_system_set_state(sys, s)
    np.testing.assert_array_equal(d.dust_system_state(sys),
                                  np.broadcast_to(s, (3, 10, 4)))
    d.dust_system_set_state(sys, np.array([7.0]), index_state=[2])
    assert np.all(d.dust_system_state(sys)[1] == 7)
    with pytest.raises(d.DustError, match="Expected dimension 2 of 'state'"):
        d.dust_system_set_state(sys, np.zeros((3, 15, 4)))


def test_rng_state_round_trip(built):
    sys1 = d.dust_system_create(d.walk(), {"sd": 1, "random_initial": True},
                                n_particles=10, seed=42)
    sys2 = d.dust_system_create(d.walk(), {"sd": 1, "random_initial": True},
                                n_particles=10, seed=43)
    assert d.dust_system_rng_state(sys1) != d.dust_system_rng_state(sys2)
    d.dust_system_set_rng_state(sys2, d.dust_system_rng_state(sys1))
    d.dust_system_run_to_time(sys1, 10)
    d.dust_system_run_to_time(sys2, 10)
    np.testing.assert_array_equal(d.dust_system_state(sys1),
                                  d.dust_system_state(sys2))
    with pytest.raises(d.DustError, match="expected 320 but given 319"):
        d.dust_system_set_rng_state(sys1, d.dust_system_rng_state(sys1)[1:])
