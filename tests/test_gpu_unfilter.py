"""Deterministic likelihood (dust_unfilter_create + dust_likelihood_run)
on the GPU against dust2's own unfilter (golden fixtures from
tests/golden/make_golden.py, reference unfilter.hpp:42-73) and the CPU
oracle (tests/testthat/test-unfilter.R is the model).

Tolerances: the discrete system (deterministic samplers) is compared
exactly, log-likelihoods and state; the dopri5 system to 1e-10 relative
in the log-likelihood and 1e-9 in the state (the step-size controller
raises the error norm to a fractional power with each platform's pow, so
step sizes may differ in the last bit; both are far inside the solver's
rtol = atol = 1e-6)."""

import numpy as np
import pytest

import dust2_gb300 as d
from conftest import golden

pytestmark = pytest.mark.gpu


def columns(g):
    times = g["times"]
    rows = g["data"].reshape(times.size, 2)
    return {"time": np.repeat(times, 2), "incidence": rows.ravel(),
            "group": np.tile([1, 2], times.size)}


def plist(gen, flat):
    out = []
    for row in flat.reshape(2, gen.n_pars):
        p = {}
        off = 0
        for par in gen.parameters:
            v = row[off:off + par["length"]]
            if not np.isnan(v[0]):
                p[par["name"]] = float(v[0])
            off += par["length"]
        out.append(p)
    return out


def test_unfilter_discrete_matches_reference(built):
    g = golden("unfilter_sir")
    gen = d.sir()
    obj = d.dust_unfilter_create(gen, 0, columns(g), n_particles=3, dt=0.25)
    pars = plist(gen, g["pars"])
    for r in range(2):
        ll = d.dust_likelihood_run(obj, pars)
        assert ll.shape == (3, 2)
        np.testing.assert_array_equal(ll.T, g["ll"][r])
    state = np.empty(2 * 3 * 5)
    d._lib.check(d._lib.lib().dust2_gb300_unfilter_state(
        obj.ptr, d._lib.dptr(state)))
    np.testing.assert_array_equal(state, g["state"])


def test_unfilter_ode_matches_reference(built):
    g = golden("unfilter_sirode")
    gen = d.sirode()
    obj = d.dust_unfilter_create(gen, 0, columns(g), n_particles=2)
    pars = plist(gen, g["pars"])
    for r in range(2):
        ll = d.dust_likelihood_run(obj, pars)
        np.testing.assert_allclose(ll.T, g["ll"][r], rtol=1e-10, atol=0)
    state = np.empty(2 * 2 * 5)
    d._lib.check(d._lib.lib().dust2_gb300_unfilter_state(
        obj.ptr, d._lib.dptr(state)))
    np.testing.assert_allclose(state, g["state"], rtol=1e-9, atol=1e-9)


def test_unfilter_index_group_and_shapes(built):
    g = golden("unfilter_sir")
    gen = d.sir()
    pars = plist(gen, g["pars"])
    obj = d.dust_unfilter_create(gen, 0, columns(g), n_particles=3, dt=0.25)
    d.dust_likelihood_run(obj, pars)
    ll2 = d.dust_likelihood_run(obj, None, index_group=[2])
    np.testing.assert_array_equal(ll2[:, 0], g["ll"][0][1])
    # one particle, one group: a scalar, as the reference drops dimensions
    cols = {"time": g["times"],
            "incidence": g["data"].reshape(-1, 2)[:, 0]}
    one = d.dust_unfilter_create(gen, 0, cols, dt=0.25)
    val = d.dust_likelihood_run(one, pars[0])
    assert isinstance(val, float)
    np.testing.assert_array_equal(val, g["ll"][0][0][0])


def test_unfilter_matches_port_on_many_groups(built, port):
    from dust2_gb300 import workloads
    gen = d.sirode()
    w = workloads.sirode_batched(n_instances=300, seed=5)
    times = np.arange(1, 31, dtype=float)
    rs = np.random.default_rng(3)
    data = rs.poisson(20, (times.size, 300)).astype(float)
    cols = {"time": np.repeat(times, 300), "incidence": data.ravel(),
            "group": np.tile(np.arange(1, 301), times.size)}
    obj = d.dust_unfilter_create(gen, 0, cols, n_particles=1)
    flat = w["pars"].reshape(300, gen.n_pars)
    pl = [{"I0": r[0], "N": r[1], "beta": r[2], "gamma": r[3]} for r in flat]
    ll = d.dust_likelihood_run(obj, pl)
    want, _ = port.unfilter_run("sirode", w["pars"], 300, 1, 0.0, times,
                                data.ravel(), 300, 5)
    np.testing.assert_allclose(ll, want[0][:, 0], rtol=1e-10, atol=0)


def _from_reference(a):
    """[time][group][particle][entry] -> (entry, particle, group, time)."""
    return np.transpose(a, (3, 2, 1, 0))


@pytest.mark.parametrize("adjoint", [False, True])
def test_unfilter_trajectories_match_reference(built, adjoint):
    t = golden("unfilter_trajectories")
    g = golden("unfilter_sir")
    gen = d.sir()
    obj = d.dust_unfilter_create(gen, 0, columns(g), n_particles=3, dt=0.25)
    pars = plist(gen, g["pars"])
    with pytest.raises(d.DustError, match="Trajectories are not current"):
        d.dust_likelihood_last_trajectories(obj)
    ll = d.dust_likelihood_run(obj, pars, save_trajectories=True,
                               save_snapshots=t["snapshots"],
                               adjoint=adjoint)
    np.testing.assert_array_equal(ll.T, t["ll"])
    tr = d.dust_likelihood_last_trajectories(obj)
    assert tr.shape == (5, 3, 2, g["times"].size)
    np.testing.assert_array_equal(tr, _from_reference(t["full"]))
    sn = d.dust_likelihood_last_snapshots(obj)
    assert sn.shape == (5, 3, 2, 2)
    np.testing.assert_array_equal(sn, _from_reference(t["snap"]))
    # index_state is 1-based, as in R: entries 1 and 3 counted from 0
    d.dust_likelihood_run(obj, pars, save_trajectories=True,
                          index_state=[2, 4], adjoint=adjoint)
    np.testing.assert_array_equal(d.dust_likelihood_last_trajectories(obj),
                                  _from_reference(t["sub"]))
    with pytest.raises(d.DustError, match="Snapshots are not current"):
        d.dust_likelihood_last_snapshots(obj)
    d.dust_likelihood_run(obj, pars, adjoint=adjoint)
    with pytest.raises(d.DustError, match="Trajectories are not current"):
        d.dust_likelihood_last_trajectories(obj)


def test_unfilter_ode_trajectories_match_reference(built):
    t = golden("unfilter_trajectories")
    g = golden("unfilter_sirode")
    gen = d.sirode()
    obj = d.dust_unfilter_create(gen, 0, columns(g), n_particles=2)
    pars = plist(gen, g["pars"])
    ll = d.dust_likelihood_run(obj, pars, save_trajectories=True,
                               save_snapshots=t["ode_snapshots"])
    np.testing.assert_allclose(ll.T, t["ll_ode"], rtol=1e-10, atol=0)
    np.testing.assert_allclose(d.dust_likelihood_last_trajectories(obj),
                               _from_reference(t["full_ode"]), rtol=1e-9,
                               atol=1e-9)
    np.testing.assert_allclose(d.dust_likelihood_last_snapshots(obj),
                               _from_reference(t["snap_ode"]), rtol=1e-9,
                               atol=1e-9)


def test_unfilter_trajectories_shapes_and_groups(built):
    """r/unfilter.hpp:84-90 dimension dropping, and trajectories of the
    groups the run covered."""
    t = golden("unfilter_trajectories")
    g = golden("unfilter_sir")
    gen = d.sir()
    pars = plist(gen, g["pars"])
    obj = d.dust_unfilter_create(gen, 0, columns(g), dt=0.25)
    d.dust_likelihood_run(obj, pars, save_trajectories=True)
    tr = d.dust_likelihood_last_trajectories(obj)
    # one particle per group: groups kept, particles folded in
    assert tr.shape == (5, 2, g["times"].size)
    full = _from_reference(t["full"])
    np.testing.assert_array_equal(tr, full[:, 0, :, :])
    d.dust_likelihood_run(obj, None, save_trajectories=True,
                          index_group=[2])
    tr = d.dust_likelihood_last_trajectories(obj)
    assert tr.shape == (5, 1, g["times"].size)
    np.testing.assert_array_equal(tr[:, 0, :], full[:, 0, 1, :])
