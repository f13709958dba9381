"""Filter trajectories on the GPU against dust2's own filter and
trajectories export (golden fixture from tests/golden/make_golden.py;
tests/testthat/test-filter.R "can save trajectories from filter" is the
model).  Trajectories are states of particles drawn from identical
streams, so they are compared exactly, as is the random particle."""

import numpy as np
import pytest

import dust2_gb300 as d
from conftest import golden

pytestmark = pytest.mark.gpu


def make(g):
    times = g["times"]
    rows = g["data"].reshape(times.size, 2)
    cols = {"time": np.repeat(times, 2), "incidence": rows.ravel(),
            "group": np.tile([1, 2], times.size)}
    return d.dust_filter_create(d.sir(), 0, cols,
                                n_particles=int(g["n_particles"]), dt=1.0,
                                seed=g["rng"].astype("<u8").tobytes())


def plist(g):
    gen = d.sir()
    out = []
    for row in g["pars"].reshape(2, gen.n_pars):
        p, off = {}, 0
        for par in gen.parameters:
            v = row[off:off + par["length"]]
            if not np.isnan(v[0]):
                p[par["name"]] = float(v[0])
            off += par["length"]
        out.append(p)
    return out


def as_fixture(traj):
    """R dims (state, particle, group, time) -> [time][group][particle]
    [state] as the fixture stores it."""
    return np.transpose(traj, (3, 2, 1, 0)).ravel()


def test_trajectories_match_reference(built):
    g = golden("trajectories_sir")
    obj = make(g)
    ll = d.dust_likelihood_run(obj, plist(g), save_trajectories=True)
    np.testing.assert_allclose(ll, g["ll"], rtol=1e-12, atol=0)
    traj = d.dust_likelihood_last_trajectories(obj)
    assert traj.shape == (5, int(g["n_particles"]), 2, g["times"].size)
    np.testing.assert_array_equal(as_fixture(traj), g["full"])
    one = d.dust_likelihood_last_trajectories(obj,
                                              select_random_particle=True)
    assert one.shape == (5, 2, g["times"].size)
    want = g["one"].reshape(g["times"].size, 2, 5)
    np.testing.assert_array_equal(np.transpose(one, (2, 1, 0)), want)


def test_trajectories_index_state(built):
    g = golden("trajectories_sir")
    obj = make(g)
    d.dust_likelihood_run(obj, plist(g), save_trajectories=True,
                          index_state=[2, 4])
    traj = d.dust_likelihood_last_trajectories(obj)
    assert traj.shape[0] == 2
    np.testing.assert_array_equal(as_fixture(traj), g["sub"])


def test_trajectories_not_current(built):
    g = golden("trajectories_sir")
    obj = make(g)
    d.dust_likelihood_run(obj, plist(g))
    with pytest.raises(d.DustError, match="Trajectories are not current"):
        d.dust_likelihood_last_trajectories(obj)
    d.dust_likelihood_run(obj, None, save_trajectories=True)
    assert d.dust_likelihood_last_trajectories(obj).shape[0] == 5
    d.dust_likelihood_run(obj, None)
    with pytest.raises(d.DustError, match="Trajectories are not current"):
        d.dust_likelihood_last_trajectories(obj)


def test_trajectories_end_at_last_state(built):
    # the last saved time is the filter's final state (filter.hpp:89-100)
    g = golden("trajectories_sir")
    obj = make(g)
    d.dust_likelihood_run(obj, plist(g), save_trajectories=True)
    traj = d.dust_likelihood_last_trajectories(obj)
    last = d.dust_likelihood_last_state(obj)
    np.testing.assert_array_equal(traj[..., -1], last)


def test_snapshots_match_reference(built):
    g = golden("trajectories_sir")
    obj = make(g)
    d.dust_likelihood_run(obj, plist(g), save_snapshots=g["snapshots"])
    with pytest.raises(d.DustError, match="Trajectories are not current"):
        d.dust_likelihood_last_trajectories(obj)
    snap = d.dust_likelihood_last_snapshots(obj)
    assert snap.shape == (5, int(g["n_particles"]), 2, 2)
    np.testing.assert_array_equal(as_fixture(snap), g["snap"])
    one = d.dust_likelihood_last_snapshots(obj, select_random_particle=True)
    want = g["snap_one"].reshape(2, 2, 5)
    np.testing.assert_array_equal(np.transpose(one, (2, 1, 0)), want)


def test_snapshots_with_trajectories_and_validation(built):
    g = golden("trajectories_sir")
    obj = make(g)
    d.dust_likelihood_run(obj, plist(g), save_trajectories=True,
                          save_snapshots=g["snapshots"])
    np.testing.assert_array_equal(
        as_fixture(d.dust_likelihood_last_trajectories(obj)), g["full"])
    np.testing.assert_array_equal(
        as_fixture(d.dust_likelihood_last_snapshots(obj)), g["snap"])
    with pytest.raises(d.DustError, match="must be found in 'time'"):
        d.dust_likelihood_run(obj, None, save_snapshots=[5.0])
    d.dust_likelihood_run(obj, None)
    with pytest.raises(d.DustError, match="Snapshots are not current"):
        d.dust_likelihood_last_snapshots(obj)
