"""The generator, samplers and elementary functions shared by the CUDA
kernels and the CPU oracle (dust2_gb300/csrc/dust2gpu/).

* Streams: checked against an independent numpy implementation of
  xoshiro256+ / SplitMix64 / jump (tests/xoshiro.py), including the GF(2)
  skip-ahead the engine uses to seed large stream blocks in parallel.
* Elementary functions: checked against numpy/scipy within a few ulp,
  and exp/log against 50-digit decimal arithmetic within 0.51 ulp.
* Samplers: checked for their distribution (mean, variance, chi-square
  against the exact pmf) on the host build; the GPU tests check that the
  device draws are bit-identical to these.
"""

import math

import numpy as np
import pytest
from scipy import special, stats

import dust2_gb300 as d
import xoshiro
from oracle import pyoracle


def words(b):
    return np.frombuffer(b, dtype="<u8")


def test_streams_match_independent_implementation(built):
    np.testing.assert_array_equal(words(d.rng_streams(20, 42)),
                                  xoshiro.streams(42, 20))
    np.testing.assert_array_equal(words(d.rng_streams(3, 0)),
                                  xoshiro.streams(0, 3))


def test_skip_ahead_blocks_match_sequential_jumps(built):
    # the engine fills blocks of 4096 streams in parallel from a GF(2)
    # skip-ahead; compare streams either side of block boundaries
    n = 8200
    eng = words(d.rng_streams(n, 7)).reshape(n, 4)
    s = xoshiro.seed_state(7)
    for k in range(n):
        if k > 0:
            xoshiro.jump(s)
        if k in (0, 1, 4095, 4096, 4097, 8191, 8192, n - 1):
            assert list(eng[k]) == s, k


def test_raw_seed_continues_by_jumping(built):
    first = d.rng_streams(1, 99)
    np.testing.assert_array_equal(words(d.rng_streams(5, first)),
                                  words(d.rng_streams(5, 99)))


def test_random_real(built):
    st = [int(x) for x in xoshiro.streams(5, 1)]
    expect = [xoshiro.random_real(st) for _ in range(100)]
    got, err = pyoracle.port_draws("real", 0, 0, 100, xoshiro.streams(5, 1))
    assert err == 0
    np.testing.assert_array_equal(got, expect)
    assert np.all((got >= 0) & (got < 1))


def ulp_err(got, expect):
    expect = np.asarray(expect, dtype=np.float64)
    return np.abs(got - expect) / np.spacing(np.abs(expect))


def test_exp_log_accuracy(built):
    rs = np.random.default_rng(1)
    x = np.concatenate([rs.uniform(-745, 709, 20000),
                        rs.uniform(-1, 1, 20000), [0.0, -0.0, 1e-300]])
    e = pyoracle.port_math("exp", x)
    assert np.max(ulp_err(e, np.exp(x))) <= 2
    assert pyoracle.port_math("exp", np.array([1000.0]))[0] == np.inf
    assert pyoracle.port_math("exp", np.array([-1000.0]))[0] == 0
    assert np.isnan(pyoracle.port_math("exp", np.array([np.nan]))[0])
    y = np.concatenate([10 ** rs.uniform(-300, 300, 20000),
                        rs.uniform(0.5, 2, 20000), [1.0, 5e-324, 2.0]])
    ly = pyoracle.port_math("log", y)
    ref = np.log(y)
    nz = ref != 0
    assert np.max(ulp_err(ly[nz], ref[nz])) <= 2
    assert pyoracle.port_math("log", np.array([1.0]))[0] == 0
    assert pyoracle.port_math("log", np.array([0.0]))[0] == -np.inf
    assert np.isnan(pyoracle.port_math("log", np.array([-1.0]))[0])


def _ulps_exact(got, exact):
    """Distance of each double in got from the exact Decimal value, in
    ulps of the correctly rounded result."""
    from decimal import Decimal
    out = []
    for g, e in zip(got, exact):
        sp = Decimal(float(np.spacing(abs(float(e)))))
        out.append(float(abs(Decimal(float(g)) - e) / sp))
    return np.array(out)


def test_exp_log_fixed_point_accuracy(built):
    """The integer fixed-point exp and log against 50-digit decimal
    arithmetic: within 0.51 ulp (nearly always correctly rounded),
    including arguments near 1 for log and near the ends of exp's
    fixed-point range."""
    from decimal import Decimal, getcontext
    getcontext().prec = 50
    rs = np.random.default_rng(7)
    x = np.concatenate([rs.uniform(-703, 703, 1500), rs.uniform(-1, 1, 500),
                        np.exp(rs.uniform(-36, -7, 300)) *
                        rs.choice([-1, 1], 300),
                        [2.0 ** -54, -(2.0 ** -53), 703.99, -703.99]])
    e = pyoracle.port_math("exp", x)
    u = _ulps_exact(e, [Decimal(float(v)).exp() for v in x])
    assert u.max() <= 0.51
    y = np.concatenate([np.exp(rs.uniform(-700, 700, 1000)),
                        1 + rs.uniform(-1e-3, 1e-3, 500),
                        1 + np.exp(rs.uniform(-36, -10, 300)) *
                        rs.choice([-1, 1], 300),
                        [5e-324, 2.2250738585072014e-308,
                         1.7976931348623157e308, 0.5, 2.0]])
    ly = pyoracle.port_math("log", y)
    u = _ulps_exact(ly, [Decimal(float(v)).ln() for v in y])
    assert u.max() <= 0.51


def test_rcp(built):
    """rcp (FP32 seed and two FP64 Newton steps) is within 1 ulp of the
    IEEE quotient."""
    rs = np.random.default_rng(4)
    n = 50000
    y = np.concatenate([rs.uniform(0.5, 2, n),
                        np.exp(rs.uniform(-60, 60, n)) *
                        rs.choice([-1, 1], n),
                        [1.0, 2.0, 0.5, 3.0, 0.1, np.nextafter(1.0, 2.0),
                         np.nextafter(2.0, 1.0)]])
    assert np.max(ulp_err(pyoracle.port_math("rcp", y), 1.0 / y)) <= 1


def test_lgamma_accuracy(built):
    x = np.concatenate([np.arange(1, 200, dtype=float),
                        np.random.default_rng(2).uniform(0.01, 1e6, 20000)])
    lg = pyoracle.port_math("lgamma", x)
    ref = special.gammaln(x)
    big = np.abs(ref) > 1
    assert np.max(np.abs(lg[big] - ref[big]) / np.abs(ref[big])) < 1e-14
    assert np.max(np.abs(lg[~big] - ref[~big])) < 1e-14
    # log(k!) is exact for small integers: lgamma(1) == lgamma(2) == 0
    np.testing.assert_array_equal(pyoracle.port_math("lgamma",
                                                     np.array([1.0, 2.0])),
                                  [0.0, 0.0])


def test_cos_sin_2pi(built):
    t = np.random.default_rng(3).uniform(0, 1, 20000)
    np.testing.assert_allclose(pyoracle.port_math("cos2pi", t),
                               np.cos(2 * np.pi * t), atol=4e-16)
    np.testing.assert_allclose(pyoracle.port_math("sin2pi", t),
                               np.sin(2 * np.pi * t), atol=4e-16)


def chisq_pvalue(draws, pmf, support):
    obs = np.array([np.sum(draws == k) for k in support], dtype=float)
    exp = pmf(support) * draws.size
    keep = exp > 5
    obs, exp = obs[keep], exp[keep]
    exp = exp * obs.sum() / exp.sum()
    return stats.chisquare(obs, exp).pvalue


@pytest.mark.parametrize("n,p", [(10, 0.3), (50, 0.1), (1000, 0.02),
                                 (1000, 0.4), (1e6, 0.3), (40, 0.9),
                                 (123456, 0.001)])
def test_binomial_distribution(built, n, p):
    m = 100000
    x, err = pyoracle.port_draws("binomial", n, p, m, xoshiro.streams(11, 1))
    assert err == 0
    assert np.all(x == np.round(x)) and np.all((x >= 0) & (x <= n))
    mean, var = n * p, n * p * (1 - p)
    assert abs(x.mean() - mean) < 5 * math.sqrt(var / m)
    assert abs(x.var() / var - 1) < 0.05
    lo, hi = stats.binom.ppf([1e-4, 1 - 1e-4], n, p)
    support = np.arange(lo, hi + 1)
    assert chisq_pvalue(x, lambda k: stats.binom.pmf(k, n, p), support) > 1e-4


@pytest.mark.parametrize("lam", [0.5, 3.0, 9.9, 10.0, 55.5, 1e4])
def test_poisson_distribution(built, lam):
    m = 100000
    x, err = pyoracle.port_draws("poisson", lam, 0, m, xoshiro.streams(12, 1))
    assert err == 0
    assert abs(x.mean() - lam) < 5 * math.sqrt(lam / m)
    lo, hi = stats.poisson.ppf([1e-4, 1 - 1e-4], lam)
    support = np.arange(lo, hi + 1)
    assert chisq_pvalue(x, lambda k: stats.poisson.pmf(k, lam),
                        support) > 1e-4


def test_normal_and_exponential(built):
    m = 200000
    x, _ = pyoracle.port_draws("normal", 2.0, 3.0, m, xoshiro.streams(13, 1))
    assert stats.kstest((x - 2) / 3, "norm").pvalue > 1e-4
    y, _ = pyoracle.port_draws("exponential", 0.5, 0, m,
                               xoshiro.streams(14, 1))
    assert stats.kstest(y, "expon", args=(0, 2)).pvalue > 1e-4


def test_sampler_errors_and_edge_cases(built):
    r = xoshiro.streams(1, 1)
    x, err = pyoracle.port_draws("binomial", 10, -0.1, 1, r)
    assert err == 1 and np.isnan(x[0])
    x, err = pyoracle.port_draws("binomial", -1, 0.5, 1, r)
    assert err == 1
    x, err = pyoracle.port_draws("binomial", 10, 0.0, 5, r)
    assert err == 0 and np.all(x == 0)
    x, err = pyoracle.port_draws("binomial", 10, 1.0, 5, r)
    assert np.all(x == 10)
    x, err = pyoracle.port_draws("poisson", -1, 0, 1, r)
    assert err == 2


def test_densities(built):
    x = np.arange(0, 60, dtype=float)
    np.testing.assert_allclose(pyoracle.port_density("poisson", x, 12.5),
                               stats.poisson.logpmf(x, 12.5), rtol=1e-13)
    assert pyoracle.port_density("poisson", np.array([0.0]), 0.0)[0] == 0
    size, mu = 20.0, 17.3
    p = size / (size + mu)
    np.testing.assert_allclose(pyoracle.port_density("negbin", x, size, mu),
                               stats.nbinom.logpmf(x, size, p), rtol=1e-12)
    np.testing.assert_allclose(pyoracle.port_density("normal", x, 3.0, 2.0),
                               stats.norm.logpdf(x, 3.0, 2.0), rtol=1e-13)
