"""The operation-counting restatement behind the roofline's algorithmic
FP64 basis (oracle/opcount): its filter runs must draw exactly what the
oracle port draws (log-likelihoods equal bit for bit), and its counts
must include the work the model's source fixes in advance."""

import numpy as np
import pytest

from oracle.opcount import count as oc


@pytest.fixture(scope="module")
def sir():
    return oc.workload("sir_batched")


@pytest.fixture(scope="module")
def seir():
    return oc.workload("seir_batched")


def test_counted_sir_filter_equals_port(sir):
    out = oc.count(sir, [0, 5], n_particles=200, n_obs=40)
    assert out["ll_equal_port"]
    per = out["per_particle_step"]
    # two binomial draws per step, each with at least one comparison
    # deciding its algorithm; one Poisson density per 4 steps
    assert per["cmp"] >= 2
    assert per["lgamma"] == pytest.approx(0.25)
    assert 20 < out["flops_per_particle_step"] < 500


def test_counted_seir_filter_equals_port(seir):
    out = oc.count(seir, [3], n_particles=48, n_obs=60)
    assert out["ll_equal_port"]
    per = out["per_particle_step"]
    # the 16 x 16 contact product alone is 256 fused multiply-adds, and
    # each age's infection probability one exp
    assert per["fma"] >= 256
    assert per["exp"] >= 16
    # one negative-binomial density (three lgamma) per 4 steps
    assert per["lgamma"] == pytest.approx(0.75)


def test_counted_dopri5_equals_port():
    # dust2's unfused solver over the counting type integrates exactly
    # as the port does (outputs and step counts), so its counts are those
    # of the reference arithmetic
    out = oc.count_dopri5(64)
    assert out["equal_port"]
    per = out["per_step"]
    # six right-hand sides of sirode per attempted step, each with one
    # division; one square root for the error norm
    assert per["div"] >= 6
    assert per["sqrt"] >= 1
    assert per["fma"] == 0
    assert 300 < out["flops_per_step"] < 700


def test_counts_are_reproducible(sir):
    a = oc.count(sir, [1], n_particles=64, n_obs=10)
    b = oc.count(sir, [1], n_particles=64, n_obs=10)
    assert a == b


def test_counted_run_detects_a_different_draw(sir):
    # the check is real: the counted run on other generator words gives
    # other log-likelihoods than the port on the workload's own
    from oracle import pyoracle
    G = len(sir["n_particles"])
    npar = np.asarray(sir["pars"]).size // G
    pars = np.asarray(sir["pars"]).reshape(G, npar)[[0]].ravel()
    times = sir["times"][:10]
    data = np.asarray(sir["data"]).reshape(sir["times"].size, G)[:10, [0]]
    words = pyoracle.rng_streams(66, sir["seed"])
    other = pyoracle.rng_streams(66, sir["seed"] + 1)
    ll, _, _ = oc.counted_filter("sir_cases", pars, [64], sir["dt"], times,
                                 data, other)
    ll_port, _, _ = pyoracle.port().filter_run(
        "sir_cases", pars, [64], 0.0, times, data.ravel(), 1, sir["dt"],
        words, n_state=4)
    assert ll[0] != ll_port[0, 0]
