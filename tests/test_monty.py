"""The MCMC caller (mirror of dust2's dust_likelihood_monty,
R/monty.R:90-317; tests/testthat/test-monty.R is the model).  CPU tests
cover the packer and the generator hand-off; GPU tests compare densities
with dust_likelihood_run and served chains with plain ones (exactly: the
same seeds give the same chains)."""

import numpy as np
import pytest

import dust2_gb300 as d
from dust2_gb300 import monty


def sir_data(n_obs=10, seed=1):
    rs = np.random.default_rng(seed)
    t = np.arange(1, n_obs + 1, dtype=float)
    return {"time": t, "incidence": rs.poisson(5, n_obs).astype(float)}


def test_packer(built):
    p = monty.Packer(["beta", "gamma"], fixed={"N": 1000})
    assert p.names() == ["beta", "gamma"]
    assert p.unpack([0.1, 0.2]) == {"N": 1000, "beta": 0.1, "gamma": 0.2}
    np.testing.assert_array_equal(p.pack({"beta": 1, "gamma": 2}), [1, 2])
    with pytest.raises(d.DustError, match="length 2"):
        p.unpack([1.0])
    with pytest.raises(d.DustError, match="both sampled and fixed"):
        monty.Packer(["N"], fixed={"N": 1})


def test_rng_hand_off_expands_one_stream(built):
    # R/monty.R:216-223: one 32-byte state becomes every stream by jumps
    obj = d.dust_filter_create(d.sir(), 0, sir_data(), n_particles=7,
                               seed=1)
    model = monty.dust_likelihood_monty(obj, monty.Packer(["beta"]))
    assert model.properties["is_stochastic"]
    seed = d.rng_streams(1, 99)
    model.set_rng_state(seed)
    assert model.get_rng_state() == d.rng_streams(9, seed)


def test_unfilter_model_is_deterministic(built):
    obj = d.dust_unfilter_create(d.sir(), 0, sir_data(), dt=0.25)
    model = monty.dust_likelihood_monty(obj, monty.Packer(["beta"]))
    assert not model.properties["is_stochastic"]
    assert model.get_rng_state is None


@pytest.mark.gpu
def test_density_is_the_likelihood(built):
    data = sir_data()
    packer = monty.Packer(["beta", "gamma"])
    a = d.dust_filter_create(d.sir(), 0, data, n_particles=50, seed=3)
    b = d.dust_filter_create(d.sir(), 0, data, n_particles=50, seed=3)
    model = monty.dust_likelihood_monty(a, packer, save_state=True)
    for x in ([0.2, 0.1], [0.3, 0.1], [0.25, 0.15]):
        want = d.dust_likelihood_run(b, packer.unpack(x))
        assert model.density(x) == want
    obs = model.observe()
    assert obs["state"].shape == (5,)


@pytest.mark.gpu
def test_deterministic_density_is_cached(built):
    obj = d.dust_unfilter_create(d.sir(), 0, sir_data(), dt=0.25)
    model = monty.dust_likelihood_monty(obj, monty.Packer(["beta"]))
    x = [0.2]
    v = model.density(x)
    assert model.density(x) == v
    assert model.density([0.3]) != v


def test_unfilter_model_has_gradient(built):
    # R/monty.R:129: deterministic likelihoods of systems with adjoints
    obj = d.dust_unfilter_create(d.sir(), 0, sir_data())
    model = monty.dust_likelihood_monty(obj, monty.Packer(["beta"]))
    assert model.properties["has_gradient"]
    obj = d.dust_unfilter_create(d.sirode(), 0, sir_data())
    model = monty.dust_likelihood_monty(obj, monty.Packer(["beta"]))
    assert not model.properties["has_gradient"] and model.gradient is None


@pytest.mark.gpu
def test_model_gradient_is_the_last_gradient(built):
    data = sir_data()
    fixed = {"N": 1000, "I0": 10, "exp_noise": 1e6}
    packer = monty.Packer(["beta", "gamma"], fixed=fixed)
    a = d.dust_unfilter_create(d.sir(), 0, data)
    b = d.dust_unfilter_create(d.sir(), 0, data)
    model = monty.dust_likelihood_monty(a, packer)
    for x in ([0.2, 0.1], [0.3, 0.1]):
        want_ll = d.dust_likelihood_run(b, packer.unpack(x), adjoint=True)
        want = d.dust_likelihood_last_gradient(b)
        np.testing.assert_array_equal(model.gradient(x), want)
        assert model.density(x) == want_ll


@pytest.mark.gpu
def test_served_chains_equal_plain_chains(built):
    gen = d.sir()
    packer = monty.Packer(["beta", "gamma"])
    datas = [sir_data(12, seed=s) for s in range(4)]
    x0 = [np.array([0.2, 0.1])] * 4
    vcv = np.diag([1e-4, 1e-4])
    plain = [monty.dust_likelihood_monty(
        d.dust_filter_create(gen, 0, dat, n_particles=64, seed=10 + i),
        packer) for i, dat in enumerate(datas)]
    want = [monty.random_walk(m, vcv, 15, x0[i], seed=i)
            for i, m in enumerate(plain)]
    server = d.dust_likelihood_server(gen, hbm_budget=1e8, max_sessions=8)
    models = [monty.served_model(server, server.open(packer.unpack(x0[i]),
                                                     dat, 64, seed=10 + i),
                                 packer) for i, dat in enumerate(datas)]
    got = monty.run_chains(models, vcv, 15, x0, seed=0)
    for (s1, d1, a1), (s2, d2, a2) in zip(got, want):
        np.testing.assert_array_equal(s1, s2)
        np.testing.assert_array_equal(d1, d2)
        assert a1 == a2
    server.free()
