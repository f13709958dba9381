"""ctypes binding of the C ABI (include/dust2_gb300.h).

The library is built in-tree by dust2_gb300.build; nothing here falls
back to a CPU implementation: if the library is missing, loading fails
with an error that says how to build it, and engine calls on a machine
without a GPU fail with the CUDA error reported by the library.
"""

import ctypes
import re
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
LIB_PATH = ROOT / "_lib" / "libdust2_gb300.so"
HEADER = ROOT.parent / "include" / "dust2_gb300.h"

c_double_p = ctypes.POINTER(ctypes.c_double)
c_size_p = ctypes.POINTER(ctypes.c_size_t)
c_u64_p = ctypes.POINTER(ctypes.c_uint64)
c_i64_p = ctypes.POINTER(ctypes.c_int64)
c_void_pp = ctypes.POINTER(ctypes.c_void_p)


class DustError(RuntimeError):
    """An error reported by the engine (message as the reference's)."""


class OdeControl(ctypes.Structure):
    _fields_ = [
        ("max_steps", ctypes.c_int32),
        ("atol", ctypes.c_double),
        ("rtol", ctypes.c_double),
        ("step_size_min", ctypes.c_double),
        ("step_size_max", ctypes.c_double),
        ("critical_times", c_double_p),
        ("n_critical_times", ctypes.c_size_t),
        ("debug_record_step_times", ctypes.c_int32),
    ]


_SIGNATURES = {
    "dust2_gb300_abi_version": (ctypes.c_int, []),
    "dust2_gb300_last_error": (ctypes.c_size_t,
                               [ctypes.c_char_p, ctypes.c_size_t]),
    "dust2_gb300_device_count": (ctypes.c_int,
                                 [ctypes.POINTER(ctypes.c_int32)]),
    "dust2_gb300_systems": (ctypes.c_int, [ctypes.c_char_p, ctypes.c_size_t]),
    "dust2_gb300_fp64_peak": (ctypes.c_int, [c_double_p]),
    "dust2_gb300_system_info": (ctypes.c_int, [ctypes.c_char_p,
                                               ctypes.c_char_p,
                                               ctypes.c_size_t]),
    "dust2_gb300_rng_streams": (ctypes.c_int, [
        c_u64_p, ctypes.c_size_t, ctypes.c_size_t, c_u64_p]),
    "dust2_gb300_system_alloc": (ctypes.c_int, [
        ctypes.c_char_p, c_double_p, ctypes.c_size_t, ctypes.c_size_t,
        ctypes.c_double, ctypes.c_double, ctypes.POINTER(OdeControl),
        c_u64_p, ctypes.c_size_t, ctypes.c_int32, c_void_pp]),
    "dust2_gb300_system_free": (ctypes.c_int, [ctypes.c_void_p]),
    "dust2_gb300_system_dim": (ctypes.c_int, [ctypes.c_void_p, c_size_p,
                                              c_size_p, c_size_p]),
    "dust2_gb300_system_state": (ctypes.c_int, [ctypes.c_void_p, c_double_p]),
    "dust2_gb300_system_set_state": (ctypes.c_int, [
        ctypes.c_void_p, c_double_p, c_size_p, ctypes.c_size_t, c_size_p,
        ctypes.c_size_t, c_size_p, ctypes.c_size_t, ctypes.c_int32,
        ctypes.c_int32]),
    "dust2_gb300_system_set_state_initial": (ctypes.c_int, [ctypes.c_void_p]),
    "dust2_gb300_system_time": (ctypes.c_int, [ctypes.c_void_p, c_double_p]),
    "dust2_gb300_system_set_time": (ctypes.c_int, [ctypes.c_void_p,
                                                   ctypes.c_double]),
    "dust2_gb300_system_rng_state": (ctypes.c_int, [ctypes.c_void_p,
                                                    c_u64_p]),
    "dust2_gb300_system_set_rng_state": (ctypes.c_int, [
        ctypes.c_void_p, c_u64_p, ctypes.c_size_t]),
    "dust2_gb300_system_update_pars": (ctypes.c_int, [
        ctypes.c_void_p, c_double_p, c_size_p, ctypes.c_size_t]),
    "dust2_gb300_system_run_to_time": (ctypes.c_int, [ctypes.c_void_p,
                                                      ctypes.c_double]),
    "dust2_gb300_system_simulate": (ctypes.c_int, [
        ctypes.c_void_p, c_double_p, ctypes.c_size_t, c_size_p,
        ctypes.c_size_t, c_double_p]),
    "dust2_gb300_system_reorder": (ctypes.c_int, [ctypes.c_void_p, c_size_p,
                                                  ctypes.c_size_t]),
    "dust2_gb300_system_compare_data": (ctypes.c_int, [
        ctypes.c_void_p, c_double_p, ctypes.c_size_t, c_double_p]),
    "dust2_gb300_system_internals": (ctypes.c_int, [
        ctypes.c_void_p, c_double_p, c_double_p, c_i64_p, c_i64_p, c_i64_p]),
    "dust2_gb300_system_step_times": (ctypes.c_int, [
        ctypes.c_void_p, ctypes.c_size_t, c_double_p, ctypes.c_size_t,
        c_size_p]),
    "dust2_gb300_filter_alloc": (ctypes.c_int, [
        ctypes.c_char_p, c_double_p, ctypes.c_size_t, ctypes.c_size_t,
        ctypes.c_double, c_double_p, ctypes.c_size_t, c_double_p,
        ctypes.c_size_t, ctypes.c_double, c_u64_p, ctypes.c_size_t,
        c_void_pp]),
    "dust2_gb300_filter_alloc_continuous": (ctypes.c_int, [
        ctypes.c_char_p, c_double_p, ctypes.c_size_t, ctypes.c_size_t,
        ctypes.c_double, c_double_p, ctypes.c_size_t, c_double_p,
        ctypes.c_size_t, ctypes.c_double, ctypes.POINTER(OdeControl),
        c_u64_p, ctypes.c_size_t, c_void_pp]),
    "dust2_gb300_filter_alloc_uneven": (ctypes.c_int, [
        ctypes.c_char_p, c_double_p, ctypes.c_size_t, c_size_p,
        ctypes.c_double, c_double_p, ctypes.c_size_t, c_double_p,
        ctypes.c_size_t, ctypes.c_double, c_u64_p, ctypes.c_size_t,
        c_void_pp]),
    "dust2_gb300_filter_free": (ctypes.c_int, [ctypes.c_void_p]),
    "dust2_gb300_filter_dim": (ctypes.c_int, [ctypes.c_void_p, c_size_p,
                                              c_size_p, c_size_p, c_size_p]),
    "dust2_gb300_filter_run": (ctypes.c_int, [
        ctypes.c_void_p, c_double_p, c_size_p, ctypes.c_size_t, c_double_p]),
    "dust2_gb300_filter_update_pars": (ctypes.c_int, [
        ctypes.c_void_p, c_double_p, c_size_p, ctypes.c_size_t]),
    "dust2_gb300_filter_rng_state": (ctypes.c_int, [
        ctypes.c_void_p, c_u64_p, ctypes.c_size_t]),
    "dust2_gb300_filter_set_rng_state": (ctypes.c_int, [
        ctypes.c_void_p, c_u64_p, ctypes.c_size_t]),
    "dust2_gb300_filter_last_state": (ctypes.c_int, [
        ctypes.c_void_p, ctypes.c_int32, c_double_p]),
    "dust2_gb300_filter_serial_fallbacks": (ctypes.c_int, [
        ctypes.c_void_p, c_i64_p]),
    "dust2_gb300_resample_weight": (ctypes.c_int, [
        c_double_p, ctypes.c_size_t, ctypes.c_double, c_size_p]),
    "dust2_gb300_resample_weight_noalloc": (ctypes.c_int, [
        c_double_p, ctypes.c_size_t, ctypes.c_double, c_size_p]),
    "dust2_gb300_scale_log_weights": (ctypes.c_int, [
        c_double_p, ctypes.c_size_t, c_double_p]),
    "dust2_gb300_filter_set_serial_resample": (ctypes.c_int, [
        ctypes.c_void_p, ctypes.c_int32]),
    "dust2_gb300_filter_set_fused_tail": (ctypes.c_int, [
        ctypes.c_void_p, ctypes.c_int32]),
    "dust2_gb300_filter_run_async": (ctypes.c_int, [
        ctypes.c_void_p, c_size_p, ctypes.c_size_t]),
    "dust2_gb300_filter_last_log_likelihood": (ctypes.c_int, [
        ctypes.c_void_p, c_double_p]),
    "dust2_gb300_filter_stream": (ctypes.c_int, [
        ctypes.c_void_p, ctypes.POINTER(ctypes.c_void_p)]),
    "dust2_gb300_filter_set_timing": (ctypes.c_int, [
        ctypes.c_void_p, ctypes.c_int32]),
    "dust2_gb300_filter_kernel_times": (ctypes.c_int, [
        ctypes.c_void_p, c_double_p, c_i64_p, c_double_p, c_i64_p]),
    "dust2_gb300_filter_reorder_times": (ctypes.c_int, [
        ctypes.c_void_p, c_double_p, c_i64_p]),
    "dust2_gb300_filter_set_autotune": (ctypes.c_int, [
        ctypes.c_void_p, ctypes.c_int32]),
    "dust2_gb300_filter_set_step_shape": (ctypes.c_int, [
        ctypes.c_void_p, ctypes.c_int32, ctypes.c_int32, ctypes.c_int32]),
    "dust2_gb300_filter_step_shape": (ctypes.c_int, [
        ctypes.c_void_p, ctypes.POINTER(ctypes.c_int32),
        ctypes.POINTER(ctypes.c_int32), ctypes.POINTER(ctypes.c_int32),
        ctypes.POINTER(ctypes.c_int32), c_double_p]),
    "dust2_gb300_system_simulate_device": (ctypes.c_int, [
        ctypes.c_void_p, c_double_p, ctypes.c_size_t, ctypes.c_void_p]),
    "dust2_gb300_system_stream": (ctypes.c_int, [ctypes.c_void_p,
                                                 c_void_pp]),
    "dust2_gb300_filter_set_save_trajectories": (ctypes.c_int, [
        ctypes.c_void_p, ctypes.c_int32, c_size_p, ctypes.c_size_t]),
    "dust2_gb300_filter_trajectory_dim": (ctypes.c_int, [
        ctypes.c_void_p, ctypes.c_int32, c_size_p, c_size_p, c_size_p,
        c_size_p]),
    "dust2_gb300_filter_last_trajectories": (ctypes.c_int, [
        ctypes.c_void_p, ctypes.c_int32, c_double_p]),
    "dust2_gb300_filter_set_save_snapshots": (ctypes.c_int, [
        ctypes.c_void_p, c_size_p, ctypes.c_size_t]),
    "dust2_gb300_filter_snapshot_dim": (ctypes.c_int, [
        ctypes.c_void_p, ctypes.c_int32, c_size_p, c_size_p, c_size_p,
        c_size_p]),
    "dust2_gb300_filter_last_snapshots": (ctypes.c_int, [
        ctypes.c_void_p, ctypes.c_int32, c_double_p]),
    "dust2_gb300_unfilter_alloc": (ctypes.c_int, [
        ctypes.c_char_p, c_double_p, ctypes.c_size_t, ctypes.c_size_t,
        ctypes.c_double, c_double_p, ctypes.c_size_t, c_double_p,
        ctypes.c_size_t, ctypes.c_double, ctypes.POINTER(OdeControl),
        c_void_pp]),
    "dust2_gb300_unfilter_free": (ctypes.c_int, [ctypes.c_void_p]),
    "dust2_gb300_unfilter_run": (ctypes.c_int, [
        ctypes.c_void_p, c_double_p, c_size_p, ctypes.c_size_t, c_double_p]),
    "dust2_gb300_unfilter_run_adjoint": (ctypes.c_int, [
        ctypes.c_void_p, c_double_p, c_size_p, ctypes.c_size_t, c_double_p]),
    "dust2_gb300_unfilter_gradient_dim": (ctypes.c_int, [
        ctypes.c_void_p, c_size_p, c_size_p]),
    "dust2_gb300_unfilter_last_gradient": (ctypes.c_int, [
        ctypes.c_void_p, c_double_p]),
    "dust2_gb300_unfilter_set_save_trajectories": (ctypes.c_int, [
        ctypes.c_void_p, ctypes.c_int32, c_size_p, ctypes.c_size_t]),
    "dust2_gb300_unfilter_set_save_snapshots": (ctypes.c_int, [
        ctypes.c_void_p, c_size_p, ctypes.c_size_t]),
    "dust2_gb300_unfilter_trajectory_dim": (ctypes.c_int, [
        ctypes.c_void_p, c_size_p, c_size_p, c_size_p, c_size_p]),
    "dust2_gb300_unfilter_last_trajectories": (ctypes.c_int, [
        ctypes.c_void_p, c_double_p]),
    "dust2_gb300_unfilter_snapshot_dim": (ctypes.c_int, [
        ctypes.c_void_p, c_size_p, c_size_p, c_size_p, c_size_p]),
    "dust2_gb300_unfilter_last_snapshots": (ctypes.c_int, [
        ctypes.c_void_p, c_double_p]),
    "dust2_gb300_system_packing_state": (ctypes.c_int, [
        ctypes.c_void_p, ctypes.c_char_p, ctypes.c_size_t, c_size_p]),
    "dust2_gb300_filter_packing_state": (ctypes.c_int, [
        ctypes.c_void_p, ctypes.c_char_p, ctypes.c_size_t, c_size_p]),
    "dust2_gb300_unfilter_packing_state": (ctypes.c_int, [
        ctypes.c_void_p, ctypes.c_char_p, ctypes.c_size_t, c_size_p]),
    "dust2_gb300_unfilter_update_pars": (ctypes.c_int, [
        ctypes.c_void_p, c_double_p, c_size_p, ctypes.c_size_t]),
    "dust2_gb300_unfilter_state": (ctypes.c_int, [ctypes.c_void_p,
                                                  c_double_p]),
    "dust2_gb300_unfilter_dim": (ctypes.c_int, [
        ctypes.c_void_p, c_size_p, c_size_p, c_size_p, c_size_p]),
    "dust2_gb300_server_create": (ctypes.c_int, [
        ctypes.c_char_p, ctypes.c_double, ctypes.c_size_t, c_void_pp]),
    "dust2_gb300_server_free": (ctypes.c_int, [ctypes.c_void_p]),
    "dust2_gb300_server_capacity": (ctypes.c_int, [
        ctypes.c_void_p, c_size_p, c_size_p, c_size_p]),
    "dust2_gb300_server_open": (ctypes.c_int, [
        ctypes.c_void_p, c_double_p, ctypes.c_size_t, ctypes.c_double,
        c_double_p, ctypes.c_size_t, c_double_p, ctypes.c_double, c_u64_p,
        ctypes.c_size_t, c_i64_p]),
    "dust2_gb300_server_submit": (ctypes.c_int, [
        ctypes.c_void_p, ctypes.c_int64, c_double_p, c_i64_p]),
    "dust2_gb300_server_wait": (ctypes.c_int, [
        ctypes.c_void_p, ctypes.c_int64, ctypes.c_double, c_double_p,
        c_double_p]),
    "dust2_gb300_server_close": (ctypes.c_int, [
        ctypes.c_void_p, ctypes.c_int64]),
    "dust2_gb300_server_rng_state": (ctypes.c_int, [
        ctypes.c_void_p, ctypes.c_int64, c_u64_p]),
    "dust2_gb300_server_set_timing": (ctypes.c_int, [
        ctypes.c_void_p, ctypes.c_int32]),
    "dust2_gb300_server_stats": (ctypes.c_int, [
        ctypes.c_void_p, c_double_p, ctypes.c_size_t]),
}

PENDING = 2

_lib = None


def declared_symbols():
    """Function names declared in include/dust2_gb300.h."""
    text = HEADER.read_text()
    return sorted(set(re.findall(r"\b(dust2_gb300_[a-z_0-9]+)\s*\(", text)))


def lib():
    """The loaded engine library (raises if it has not been built)."""
    global _lib
    if _lib is None:
        if not LIB_PATH.exists():
            raise DustError(
                f"The dust2_gb300 CUDA library is not built ({LIB_PATH}); "
                "run `python -m dust2_gb300.build` (or "
                "__graft_entry__.build()) first")
        handle = ctypes.CDLL(str(LIB_PATH))
        for name, (res, args) in _SIGNATURES.items():
            fn = getattr(handle, name)
            fn.restype = res
            fn.argtypes = args
        _lib = handle
    return _lib


def last_error():
    buf = ctypes.create_string_buffer(8192)
    lib().dust2_gb300_last_error(buf, len(buf))
    return buf.value.decode()


def check(rc):
    if rc != 0:
        raise DustError(last_error())


def dptr(a):
    """ctypes double pointer of a contiguous float64 array (or NULL)."""
    if a is None:
        return None
    return a.ctypes.data_as(c_double_p)


def sptr(a):
    if a is None:
        return None
    return a.ctypes.data_as(c_size_p)


def uptr(a):
    if a is None:
        return None
    return a.ctypes.data_as(c_u64_p)


def as_f64(x):
    return np.ascontiguousarray(x, dtype=np.float64)


def as_size(x):
    return np.ascontiguousarray(x, dtype=np.uintp)


def as_u64(x):
    return np.ascontiguousarray(x, dtype=np.uint64)


def device_count():
    n = ctypes.c_int32(0)
    check(lib().dust2_gb300_device_count(ctypes.byref(n)))
    return n.value
