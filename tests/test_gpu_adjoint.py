"""Gradients of deterministic likelihoods (dust_likelihood_run(adjoint=
TRUE) + dust_likelihood_last_gradient) on the GPU against dust2's own
unfilter::run_adjoint / last_gradient (golden fixtures from
tests/golden/make_golden.py, reference unfilter.hpp:77-142, 188-229) and
the CPU oracle; tests/testthat/test-unfilter-adjoint.R is the model.

Tolerance: exact.  The sir system's adjoint is plain arithmetic and exp
on a deterministic trajectory, compiled without contraction on both
sides, as the discrete unfilter's log-likelihood is."""

import numpy as np
import pytest

import dust2_gb300 as d
from conftest import golden

pytestmark = pytest.mark.gpu

BASE = {"beta": 0.1, "gamma": 0.2, "N": 1000, "I0": 10, "exp_noise": 1e6}


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


def case(g, label):
    n_groups, t0, dt, ngd = g[f"{label}__meta"]
    n_groups, ngd = int(n_groups), int(ngd)
    times = g[f"{label}__times"]
    rows = g[f"{label}__data"].reshape(times.size, ngd)
    if ngd == 1:
        data = {"time": times, "incidence": rows[:, 0]}
    else:
        data = {"time": np.repeat(times, ngd), "incidence": rows.ravel(),
                "group": np.tile(np.arange(1, ngd + 1), times.size)}
    return n_groups, t0, dt, data


@pytest.mark.parametrize("label", ["four_days", "odd_steps", "four_groups",
                                   "quarter_days", "late_start"])
def test_adjoint_matches_reference(built, label):
    g = golden("adjoint_sir")
    gen = d.sir()
    n_groups, t0, dt, data = case(g, label)
    shared = n_groups > 1 and "group" not in data
    obj = d.dust_unfilter_create(gen, t0, data, dt=dt, n_groups=n_groups,
                                 shared_data=shared)
    pars = plist(gen, g[f"{label}__pars"], n_groups)
    if n_groups == 1:
        pars = pars[0]
    ll = d.dust_likelihood_run(obj, pars, adjoint=True)
    gr = d.dust_likelihood_last_gradient(obj)
    want_ll = g[f"{label}__ll"].ravel()
    want_gr = g[f"{label}__gradient"].reshape(n_groups, 3).T
    np.testing.assert_array_equal(np.ravel(ll), want_ll)
    np.testing.assert_array_equal(np.reshape(gr, (3, n_groups)), want_gr)
    state = np.empty(n_groups * 5)
    d._lib.check(d._lib.lib().dust2_gb300_unfilter_state(
        obj.ptr, d._lib.dptr(state)))
    np.testing.assert_array_equal(state, g[f"{label}__state"])
    # the plain run gives the identical log-likelihood
    ll_plain = d.dust_likelihood_run(obj, None, adjoint=False)
    np.testing.assert_array_equal(np.ravel(ll_plain), want_ll)


def test_adjoint_is_default_and_must_be_current(built):
    gen = d.sir()
    data = {"time": [4.0, 8, 12, 16], "incidence": [1.0, 2, 3, 4]}
    obj = d.dust_unfilter_create(gen, 0, data)
    with pytest.raises(d.DustError, match="Gradient is not current"):
        d.dust_likelihood_last_gradient(obj)
    d.dust_likelihood_run(obj, BASE, adjoint=False)
    with pytest.raises(d.DustError,
                       match="System was not run with 'adjoint = TRUE'"):
        d.dust_likelihood_last_gradient(obj)
    d.dust_likelihood_run(obj, BASE)
    assert d.dust_likelihood_last_gradient(obj).shape == (3,)
    # a later plain run makes the gradient stale again
    d.dust_likelihood_run(obj, BASE, adjoint=False)
    with pytest.raises(d.DustError, match="adjoint = TRUE"):
        d.dust_likelihood_last_gradient(obj)


def test_adjoint_shapes_and_index_group(built):
    g = golden("adjoint_sir")
    gen = d.sir()
    n_groups, t0, dt, data = case(g, "four_groups")
    pars = plist(gen, g["four_groups__pars"], n_groups)
    want = g["four_groups__gradient"].reshape(n_groups, 3).T
    obj = d.dust_unfilter_create(gen, t0, data, n_groups=4,
                                 preserve_particle_dimension=True)
    ll = d.dust_likelihood_run(obj, pars, adjoint=True)
    assert ll.shape == (1, 4)
    gr = d.dust_likelihood_last_gradient(obj)
    assert gr.shape == (3, 1, 4)
    np.testing.assert_array_equal(gr[:, 0, :], want)
    # a run over some groups (1-based, as in R) gives the gradient of
    # those groups, in that order
    d.dust_likelihood_run(obj, None, index_group=[3, 1], adjoint=True)
    gr = d.dust_likelihood_last_gradient(obj)
    assert gr.shape == (3, 1, 2)
    np.testing.assert_array_equal(gr[:, 0, :], want[:, [2, 0]])


def test_adjoint_many_particles(built, port):
    """More than one particle per group (beyond the reference, which
    copies one particle's gradient): every particle of a deterministic
    system carries the same gradient, equal to the oracle's."""
    gen = d.sir()
    times = np.array([3.0, 6, 9, 12, 15])
    inc = np.array([1.0, 3, 2, 5, 4])
    data = {"time": times, "incidence": inc}
    pars = [dict(BASE, beta=0.15), dict(BASE, gamma=0.3, I0=20)]
    obj = d.dust_unfilter_create(gen, 0, data, n_particles=7, n_groups=2,
                                 dt=0.5, shared_data=True)
    ll = d.dust_likelihood_run(obj, pars, adjoint=True)
    gr = d.dust_likelihood_last_gradient(obj)
    assert gr.shape == (3, 7, 2)
    flat = np.concatenate([gen.pack_pars(p) for p in pars])
    want_ll, want_gr, _ = port.unfilter_adjoint("sir", flat, 2, 7, 0.0,
                                                times, inc, 1, 5, dt=0.5)
    np.testing.assert_array_equal(ll, want_ll.T)
    np.testing.assert_array_equal(gr, want_gr.transpose(2, 1, 0))


def test_adjoint_unsupported_systems(built):
    times = np.array([1.0, 2, 3])
    data = {"time": times, "incidence": [1.0, 2, 3]}
    obj = d.dust_unfilter_create(d.sirode(), 0, data)
    pars = {"beta": 0.2, "gamma": 0.1, "N": 1000, "I0": 10}
    ll_default = d.dust_likelihood_run(obj, pars)
    ll_adjoint = d.dust_likelihood_run(obj, pars, adjoint=True)
    assert ll_default == ll_adjoint
    with pytest.raises(d.DustError, match="does not support adjoint"):
        d.dust_likelihood_last_gradient(obj)


def test_adjoint_many_groups_against_oracle(built, port):
    """4096 groups of random parameters, one particle each, 60 daily
    observations at dt = 0.25: every group's log-likelihood and gradient
    equal the oracle's."""
    gen = d.sir()
    rs = np.random.default_rng(21)
    G = 4096
    pars = [dict(BASE, beta=float(b), gamma=float(c), I0=float(i))
            for b, c, i in zip(rs.uniform(0.1, 0.6, G),
                               rs.uniform(0.05, 0.3, G),
                               rs.integers(1, 40, G))]
    times = np.arange(1, 61, dtype=float)
    inc = rs.poisson(6, times.size).astype(float)
    obj = d.dust_unfilter_create(gen, 0, {"time": times, "incidence": inc},
                                 n_groups=G, dt=0.25, shared_data=True)
    ll = d.dust_likelihood_run(obj, pars, adjoint=True)
    gr = d.dust_likelihood_last_gradient(obj)
    flat = np.concatenate([gen.pack_pars(p) for p in pars])
    want_ll, want_gr, _ = port.unfilter_adjoint("sir", flat, G, 1, 0.0,
                                                times, inc, 1, 5, dt=0.25)
    np.testing.assert_array_equal(np.ravel(ll), want_ll.ravel())
    np.testing.assert_array_equal(gr, want_gr[:, 0, :].T)
