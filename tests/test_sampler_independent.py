"""The engine's binomial and Poisson samplers against a separate restatement
of the published algorithms, written here in Python with the host's libm
exp, log, sqrt and lgamma (instead of the engine's fixed-point exp/log,
table reciprocals and log-factorial table), driven by the independent
numpy generator (tests/xoshiro.py).

The engine's samplers are shared by the CUDA kernels and the CPU oracle,
so GPU = oracle cannot catch an error made in them; the statistical
checks in test_rng_math.py bound such an error only loosely.  Here the
draws themselves must agree, value for value along whole streams, for
arguments in every branch: inversion (BINV, Kachitvichyanukul & Schmeiser
1988) and transformed rejection with squeeze (BTRS, Hormann 1993) for the
binomial, with p > 1/2 by symmetry; multiplication of uniforms (Knuth)
and PTRS (Hormann 1993) for the Poisson.  Multiply-adds that the engine
fuses are fused here too (rounded once, through exact rationals).  The
two sides round their elementary functions and reciprocals differently
(within an ulp or two), so a draw could differ when a comparison falls
within that distance of a boundary; on these streams none does."""

import math
from fractions import Fraction

import numpy as np
import pytest

import xoshiro
from oracle import pyoracle

BINV_MAX_X = 110


def fma(a, b, c):
    """a * b + c rounded once (exact rational arithmetic, then the
    correctly rounded conversion to a double)."""
    return float(Fraction(a) * Fraction(b) + Fraction(c))


def uniform(s):
    return xoshiro.random_real(s)


def binomial_inversion(s, n, p):
    q = 1.0 - p
    sr = p / q
    a = (n + 1.0) * sr
    r0 = math.exp(n * math.log(q))
    while True:
        r = r0
        u = uniform(s)
        x = 0
        while u > r:
            u -= r
            x += 1
            r *= fma(a, 1.0 / x, -sr)
            if x > BINV_MAX_X:
                break
        if x <= BINV_MAX_X:
            return float(x)


def log_factorial(k):
    return math.lgamma(k + 1.0)


def binomial_btrs(s, n, p):
    q = 1.0 - p
    spq = math.sqrt(n * p * q)
    b = fma(2.53, spq, 1.15)
    a = fma(0.01, p, fma(0.0248, b, -0.0873))
    c = fma(n, p, 0.5)
    v_r = fma(-4.2, 1.0 / b, 0.92)
    while True:
        u = uniform(s) - 0.5
        v = uniform(s)
        us = 0.5 - abs(u)
        if us == 0:
            continue
        k = math.floor(fma(fma(2.0 * a, 1.0 / us, b), u, c))
        if us >= 0.07 and v <= v_r:
            return float(k)
        if k < 0 or k > n:
            continue
        alpha = fma(5.1, 1.0 / b, 2.83) * spq
        lpq = math.log(p / q)
        m = math.floor((n + 1.0) * p)
        h = log_factorial(m) + log_factorial(n - m)
        v = math.log(v * alpha / fma(a / us, 1.0 / us, b))
        if v <= fma(k - m, lpq, h - log_factorial(k) - log_factorial(n - k)):
            return float(k)


def binomial(s, n, p):
    if n == 0 or p == 0:
        return 0.0
    if p == 1:
        return float(n)
    flip = p > 0.5
    pp = 1.0 - p if flip else p
    if n * pp < 10:
        x = binomial_inversion(s, n, pp)
    else:
        x = binomial_btrs(s, n, pp)
    return n - x if flip else x


def poisson(s, lam):
    if lam == 0:
        return 0.0
    if lam < 10:
        enlam = math.exp(-lam)
        prod = 1.0
        x = 0
        while True:
            prod *= uniform(s)
            if prod <= enlam:
                return float(x)
            x += 1
    slam = math.sqrt(lam)
    b = fma(2.53, slam, 0.931)
    a = fma(0.02483, b, -0.059)
    vr = fma(-3.6224, 1.0 / (b - 2.0), 0.9277)
    while True:
        u = uniform(s) - 0.5
        v = uniform(s)
        us = 0.5 - abs(u)
        if us == 0:
            continue
        k = math.floor(fma(fma(2.0 * a, 1.0 / us, b), u, lam + 0.43))
        if us >= 0.07 and v <= vr:
            return float(k)
        if k < 0 or (us < 0.013 and v > us):
            continue
        log_invalpha = math.log(fma(1.1328, 1.0 / (b - 3.4), 1.1239))
        if (math.log(v) + log_invalpha - math.log(fma(a / us, 1.0 / us, b))
                <= fma(k, math.log(lam), -lam) - math.lgamma(k + 1.0)):
            return float(k)


BINOMIAL_CASES = [
    # inversion (n * min(p, 1 - p) < 10)
    (5, 0.3), (40, 0.1), (1000, 0.004), (62500, 1e-5), (99, 0.0999),
    (20, 0.9), (300, 0.98),
    # transformed rejection
    (100, 0.1), (1000, 0.3), (62500, 0.05), (1e6, 0.002), (5000, 0.5),
    (200, 0.75), (1e6, 0.99),
]
POISSON_CASES = [0.5, 3.0, 9.99, 10.0, 17.5, 250.0, 1e5]


@pytest.mark.parametrize("n,p", BINOMIAL_CASES)
def test_binomial_draws_match_independent_restatement(n, p):
    seed = int(n * 1000 + p * 1e6) % 100003
    words = xoshiro.streams(seed, 1)
    got, err = pyoracle.port_draws("binomial", n, p, 2000, words)
    assert err == 0
    s = [int(x) for x in words]
    want = [binomial(s, float(n), p) for _ in range(2000)]
    np.testing.assert_array_equal(got, want)


@pytest.mark.parametrize("lam", POISSON_CASES)
def test_poisson_draws_match_independent_restatement(lam):
    words = xoshiro.streams(int(lam * 97) + 1, 1)
    got, err = pyoracle.port_draws("poisson", lam, 0, 2000, words)
    assert err == 0
    s = [int(x) for x in words]
    want = [poisson(s, lam) for _ in range(2000)]
    np.testing.assert_array_equal(got, want)
