"""binomial_sequence (the merged-loop form of K binomial draws that the
age-structured SEIR uses) returns exactly what K calls of binomial()
return: the same draws, the same generator state afterwards and the same
recorded error, over arguments in every branch (inversion, transformed
rejection, symmetry for p > 1/2, n = 0, p = 0 or 1, deterministic
generators, invalid arguments)."""

import ctypes

import numpy as np
import pytest

import xoshiro
from oracle import pyoracle


def batches(merged, k, n, p, words, deterministic=False):
    o = pyoracle.port()
    f = o.lib.oracle_binomial_batches
    f.restype = ctypes.c_int
    n = np.ascontiguousarray(n, dtype=np.float64)
    p = np.ascontiguousarray(p, dtype=np.float64)
    words = np.ascontiguousarray(words, dtype=np.uint64)
    out = np.empty(n.size)
    rng_out = np.empty(4, dtype=np.uint64)
    err = np.empty(3)
    dp = ctypes.POINTER(ctypes.c_double)
    up = ctypes.POINTER(ctypes.c_uint64)
    rc = f(merged, k, n.size // k, n.ctypes.data_as(dp), p.ctypes.data_as(dp),
           words.ctypes.data_as(up), int(deterministic), out.ctypes.data_as(dp),
           rng_out.ctypes.data_as(up), err.ctypes.data_as(dp))
    assert rc == 0
    return out, rng_out, err


def cases(rs, size):
    n = np.floor(np.exp(rs.uniform(0, 14, size)))
    n[rs.uniform(size=size) < 0.05] = 0
    p = np.exp(-rs.uniform(0, 12, size))
    flip = rs.uniform(size=size) < 0.2
    p[flip] = 1 - p[flip]
    p[rs.uniform(size=size) < 0.03] = 0
    p[rs.uniform(size=size) < 0.03] = 1
    return n, p


@pytest.mark.parametrize("k", [3, 12, 48])
def test_merged_draws_equal_one_by_one(k):
    rs = np.random.default_rng(k)
    n, p = cases(rs, 48 * 400)
    words = xoshiro.streams(k + 5, 1)
    a = batches(1, k, n, p, words)
    b = batches(0, k, n, p, words)
    np.testing.assert_array_equal(a[0], b[0])
    np.testing.assert_array_equal(a[1], b[1])
    np.testing.assert_array_equal(a[2], b[2])
    assert a[2][0] == 0


@pytest.mark.parametrize("k", [3, 48])
def test_merged_errors_and_deterministic_equal_one_by_one(k):
    rs = np.random.default_rng(100 + k)
    n, p = cases(rs, 48 * 50)
    n[7] = -1      # invalid n: the first error
    p[40] = 1.5    # invalid p: a later one, not recorded
    n[90] = np.inf
    words = xoshiro.streams(3, 1)
    a = batches(1, k, n, p, words)
    b = batches(0, k, n, p, words)
    np.testing.assert_array_equal(a[0], b[0])
    np.testing.assert_array_equal(a[1], b[1])
    np.testing.assert_array_equal(a[2], b[2])
    assert a[2][0] != 0 and a[2][1] == -1
    d1 = batches(1, k, n, p, words, deterministic=True)
    d0 = batches(0, k, n, p, words, deterministic=True)
    np.testing.assert_array_equal(d1[0], d0[0])
    np.testing.assert_array_equal(d1[1], d0[1])
