"""The resampling entry point that allocates no device memory.

Callers whose GPU memory belongs to another allocator, or who cannot
afford the synchronisation of cudaMalloc/cudaFree at call time, use
dust2_gb300_resample_weight_noalloc, which works in a scratch area
compiled into the library.  Its indices must be identical to those of
dust2_gb300_resample_weight (the allocating entry point running the same
kernels) -- resampling indices are integer results, compared exactly -- on
consecutive calls that reuse the shared scratch area.

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
