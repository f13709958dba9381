"""The resampling entry point that allocates no device memory.

Callers whose GPU memory belongs to another allocator, or who cannot
afford the synchronisation of cudaMalloc/cudaFree at call time, use
dust2_gb300_resample_weight_noalloc, which works in a scratch area
compiled into the library.  Its indices must be identical to those of
dust2_gb300_resample_weight (the allocating entry point running the same
kernels) -- resampling indices are integer results, compared exactly -- on
consecutive calls that reuse the shared scratch area -- and equal to the
CPU oracle's serial algorithm on weights whose decisions sit within
rounding distance of a boundary, where the exact serial fallback runs
inside the scratch area too.

This file is collected last so that a failure here leaves every other
test already run; it also passes on its own in a fresh process."""

import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _call(fn_name, w, u):
    from dust2_gb300 import _lib
    w = np.ascontiguousarray(w, dtype=np.float64)
    idx = np.empty(w.size, dtype=np.uintp)
    fn = getattr(_lib.lib(), fn_name)
    rc = fn(w.ctypes.data_as(_lib.c_double_p), w.size, ctypes.c_double(u),
            idx.ctypes.data_as(_lib.c_size_p))
    if rc != 0:
        raise _lib.DustError(_lib.last_error())
    return idx


@pytest.fixture(scope="module")
def lib_ready():
    import __graft_entry__
    __graft_entry__.build()


def test_no_alloc_matches_allocating_entry_point(lib_ready):
    rs = np.random.default_rng(2024)
    cases = [
        (np.abs(rs.standard_cauchy(65536)), 0.37),  # the maximum size
        (np.abs(rs.standard_cauchy(300)), 0.91),    # smaller, same scratch
        (np.ones(4096), 0.0),                       # exact ties everywhere
        (np.abs(rs.normal(size=1)), 0.5)]
    for w, u in cases:
        expect = _call("dust2_gb300_resample_weight", w, u)
        got1 = _call("dust2_gb300_resample_weight_noalloc", w, u)
        got2 = _call("dust2_gb300_resample_weight_noalloc", w, u)
        np.testing.assert_array_equal(got1, expect)
        np.testing.assert_array_equal(got2, expect)


def test_no_alloc_rejects_sizes_above_its_limit(lib_ready):
    from dust2_gb300 import _lib
    with pytest.raises(_lib.DustError, match="above the limit of 65536"):
        _call("dust2_gb300_resample_weight_noalloc", np.ones(65537), 0.5)


def test_no_alloc_near_ties_match_oracle(lib_ready):
    # weights that make the parallel decision ambiguous (equal weights,
    # powers of two down to subnormals, halfway sums, sparse weights, 700
    # orders of magnitude), so that the exact serial fallback runs in the
    # fixed scratch area; compared with the oracle directly, two calls in
    # a row each
    from oracle import pyoracle
    port = pyoracle.port()
    rs = np.random.default_rng(23)
    n = 40000
    cases = [np.ones(n), np.ldexp(1.0, -rs.integers(0, 1100, n)),
             rs.integers(0, 4, n) * 0.5,
             np.where(rs.uniform(size=n) < 0.95, 0.0, rs.uniform(size=n)),
             np.exp(-700 * rs.uniform(size=n))]
    for w in cases:
        for u in (0.0, 0.5, 1 - 1e-12):
            want = port.resample_weight(w, u)
            for _ in range(2):
                got = _call("dust2_gb300_resample_weight_noalloc", w, u)
                np.testing.assert_array_equal(got, want)


def test_no_alloc_first_call_on_a_second_device(lib_ready):
    # the scratch address is looked up per device on its first call: a
    # first call on device 1 after calls on device 0 must use device 1's
    # own array (boxes with one GPU skip this)
    import dust2_gb300 as d
    if d.device_count() < 2:
        pytest.skip("needs two GPUs")
    rs = np.random.default_rng(4)
    w = np.abs(rs.standard_cauchy(5000))
    expect = _call("dust2_gb300_resample_weight", w, 0.25)
    # the CUDA runtime the library is linked against (already loaded, so
    # this is the same instance and its current device is the library's)
    cudart = ctypes.CDLL("libcudart.so.13")
    np.testing.assert_array_equal(
        _call("dust2_gb300_resample_weight_noalloc", w, 0.25), expect)
    prev = ctypes.c_int()
    assert cudart.cudaGetDevice(ctypes.byref(prev)) == 0
    try:
        assert cudart.cudaSetDevice(1) == 0
        np.testing.assert_array_equal(
            _call("dust2_gb300_resample_weight", w, 0.25), expect)
        np.testing.assert_array_equal(
            _call("dust2_gb300_resample_weight_noalloc", w, 0.25), expect)
    finally:
        cudart.cudaSetDevice(prev.value)
