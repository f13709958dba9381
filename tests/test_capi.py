"""The C ABI library and the host-side mirror of dust2's R layer, without
a GPU: the library loads, exports every function include/dust2_gb300.h
declares, describes its systems, and the argument checks that happen
before any device work give dust2's messages."""

import ctypes
import json

import numpy as np
import pytest

import dust2_gb300 as d
from dust2_gb300 import _lib, interface


def test_library_exports_every_declared_symbol(built):
    lib = _lib.lib()
    declared = _lib.declared_symbols()
    assert len(declared) >= 35
    for name in declared:
        assert hasattr(lib, name), name
    assert set(declared) == set(_lib._SIGNATURES)
    assert lib.dust2_gb300_abi_version() == 1


def test_ctypes_prototypes_match_header_arity():
    """Every C ABI declaration and its ctypes prototype take the same number
    of arguments (catches a binding that drifted from the header)."""
    import re
    text = _lib.HEADER.read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    decls = re.findall(r"\b(dust2_gb300_[a-z_0-9]+)\s*\(([^;{]*?)\)\s*;",
                       text, flags=re.S)
    assert len(decls) == len(_lib._SIGNATURES)
    for name, params in decls:
        p = params.strip()
        n = 0 if p in ("", "void") else len(p.split(","))
        assert len(_lib._SIGNATURES[name][1]) == n, name


def test_device_count_without_gpu_is_reported(built):
    assert d.device_count() >= 0


def test_system_info(built):
    buf = ctypes.create_string_buffer(1 << 16)
    assert _lib.lib().dust2_gb300_systems(buf, len(buf)) == 0
    names = set(buf.value.decode().split(","))
    assert {"sir", "sir_cases", "sirode", "walk", "logistic",
            "seir_age"} <= names
    gen = d.sir()
    assert gen.time_type == "discrete" and gen.has_compare
    assert [p["name"] for p in gen.parameters] == ["I0", "N", "beta", "gamma",
                                                   "exp_noise"]
    assert d.sirode().time_type == "continuous"
    assert not d.walk().has_compare
    info = json.loads(_info("seir_age"))
    assert info["n_state_max"] == 96
    assert _lib.lib().dust2_gb300_system_info(b"nope", buf, len(buf)) == 1
    assert "Unknown system 'nope'" in _lib.last_error()


def _info(name):
    buf = ctypes.create_string_buffer(1 << 16)
    _lib.check(_lib.lib().dust2_gb300_system_info(name.encode(), buf,
                                                  len(buf)))
    return buf.value.decode()


def test_pack_pars(built):
    gen = d.sir()
    row = gen.pack_pars({"beta": 0.3, "N": 100})
    assert row[2] == 0.3 and row[1] == 100
    assert np.isnan(row[0]) and np.isnan(row[3])
    with pytest.raises(d.DustError, match="must be a scalar"):
        gen.pack_pars({"beta": [1, 2]})
    gen = d.seir_age()
    row = gen.pack_pars({"contact": np.ones((16, 16))})
    assert row.size == 5 + 16 + 256


def test_check_dt_messages(built):
    gen = d.walk()
    assert interface._check_dt(None, gen) == 1
    assert interface._check_dt(0.25, gen) == 0.25
    with pytest.raises(d.DustError, match="greater than 0"):
        interface._check_dt(0, gen)
    with pytest.raises(d.DustError, match="an integer, if greater than 1"):
        interface._check_dt(1.5, gen)
    with pytest.raises(d.DustError, match="the inverse of an integer"):
        interface._check_dt(np.sqrt(2) / 2, gen)
    with pytest.raises(d.DustError, match="Can't use 'dt' with continuous"):
        interface._check_dt(1, d.sirode())


def test_check_time_messages():
    with pytest.raises(d.DustError, match="integer-like, because 'dt' is 1"):
        interface._check_time(1.5, 1.0)
    with pytest.raises(d.DustError, match=r"a multiple of 'dt' \(0.25\)"):
        interface._check_time(1.1, 0.25)
    assert interface._check_time(1.5, 0.1) == 1.5


def test_check_index_messages():
    assert list(interface._check_index([2, 4], 5, "i")) == [1, 3]
    with pytest.raises(d.DustError,
                       match=r"must be in \[1, 3\], but 'index_state\[2\]' "
                       "was 20"):
        interface._check_index([2, 20], 3, "index_state")
    with pytest.raises(d.DustError, match="must be integer-like"):
        interface._check_index([2, 2.9], 3, "index_state")
    with pytest.raises(d.DustError, match="must have nonzero length"):
        interface._check_index([], 3, "index_state")
    with pytest.raises(d.DustError, match="Expected an integer vector"):
        interface._check_index(["2"], 3, "index_state")


def test_prepare_state_recycling_and_messages():
    ps = interface._prepare_state
    v, rp, rg = ps(np.zeros((3, 1, 4)), None, None, None, 3, 10, 4, True,
                   True)
    assert rp and not rg
    v, rp, rg = ps(np.zeros(3), None, None, None, 3, 10, 4, True, True)
    assert rp and rg
    with pytest.raises(d.DustError, match="Expected 'state' to have 3 rows"):
        ps(np.zeros((2, 10)), None, None, None, 3, 10, 1, True, False)
    with pytest.raises(d.DustError, match="to have 1 or 10 columns"):
        ps(np.zeros((3, 15)), None, None, None, 3, 10, 1, True, False)
    with pytest.raises(d.DustError, match="Expected 'state' to be a matrix"):
        ps(np.zeros((3, 10, 1)), None, None, None, 3, 10, 1, True, False)
    with pytest.raises(d.DustError,
                       match="Expected dimension 3 of 'state' to be length "
                       "1 or 4"):
        ps(np.zeros((3, 10, 2)), None, None, None, 3, 10, 4, True, True)


def test_filter_data_preparation(built):
    gen = d.sir()
    data = {"time": [4, 8, 12, 16] * 2, "group": [1] * 4 + [2] * 4,
            "incidence": list(range(1, 9))}
    p = interface._prepare_data(data, None, False, gen)
    assert p["n_groups"] == 2 and list(p["time"]) == [4, 8, 12, 16]
    np.testing.assert_array_equal(p["rows"][:, :, 0],
                                  [[1, 5], [2, 6], [3, 7], [4, 8]])
    with pytest.raises(d.DustError, match="looks grouped"):
        interface._prepare_data({"time": [1, 1], "incidence": [1, 2]}, None,
                                False, gen)
    with pytest.raises(d.DustError, match="Not all groups in 'data' have"):
        interface._prepare_data({"time": [1, 2, 1, 3], "group": [1, 1, 2, 2],
                                 "incidence": [1, 2, 3, 4]}, None, False, gen)
    with pytest.raises(d.DustError, match="Expected 'data' to have 2 groups"):
        interface._prepare_data({"time": [1, 2], "incidence": [1, 2]}, 2,
                                False, gen)


def test_filter_create_validation_without_device(built):
    data = {"time": [4.0, 8, 12, 16], "incidence": [1.0, 2, 3, 4]}
    with pytest.raises(d.DustError, match="'time_start' \\(6\\) is later"):
        d.dust_filter_create(d.sir(), 6, data, n_particles=10)
    with pytest.raises(d.DustError, match="does not have 'compare_data'"):
        d.dust_filter_create(d.walk(), 0, data, n_particles=10)
    with pytest.raises(d.DustError, match="continuous-time models"):
        d.dust_filter_create(d.sirode(), 0, data, n_particles=10)
    obj = d.dust_filter_create(d.sir(), 0, data, n_particles=10, seed=42)
    # before initialisation the rng state is the initial stream block
    assert d.dust_likelihood_rng_state(obj) == d.rng_streams(12, 42)
    with pytest.raises(d.DustError, match="'pars' cannot be NULL"):
        d.dust_likelihood_run(obj, None)
    with pytest.raises(d.DustError, match="'index_group' must be NULL"):
        d.dust_likelihood_run(obj, {"beta": 0.1}, index_group=[1])
    # run options set before the first run are kept for the engine object
    from dust2_gb300 import interface
    assert obj.fused_tail and not obj.serial_resample
    interface.dust_likelihood_set_fused_tail(obj, False)
    interface.dust_likelihood_set_serial_resample(obj, True)
    assert not obj.fused_tail and obj.serial_resample
    unf = d.dust_unfilter_create(d.sir(), 0, data)
    with pytest.raises(d.DustError, match="Expected 'obj' to be a particle"):
        interface.dust_likelihood_set_fused_tail(unf, True)


def test_invalid_handles_are_errors(built):
    lib = _lib.lib()
    t = ctypes.c_double()
    assert lib.dust2_gb300_system_time(None, ctypes.byref(t)) == 1
    assert "Invalid system handle" in _lib.last_error()
    assert lib.dust2_gb300_filter_run(None, None, None, 0, None) == 1
    assert "Invalid filter handle" in _lib.last_error()
    assert lib.dust2_gb300_filter_set_fused_tail(None, 1) == 1
    assert "Invalid filter handle" in _lib.last_error()


def test_server_validation_without_device(built):
    lib = _lib.lib()
    h = ctypes.c_void_p()
    assert lib.dust2_gb300_server_create(b"nope", 1e8, 4,
                                         ctypes.byref(h)) == 1
    assert "Unknown system 'nope'" in _lib.last_error()
    assert lib.dust2_gb300_server_create(b"sir", 1e8, 0,
                                         ctypes.byref(h)) == 1
    assert "'max_sessions'" in _lib.last_error()
    assert lib.dust2_gb300_server_create(b"sirode", 1e8, 4,
                                         ctypes.byref(h)) == 1
    assert "Can't serve likelihoods of the 'sirode' system" in \
        _lib.last_error()
    t = ctypes.c_int64()
    assert lib.dust2_gb300_server_submit(None, 1, None, ctypes.byref(t)) == 1
    assert "Invalid server handle" in _lib.last_error()
    with pytest.raises(d.DustError, match="Can't serve"):
        d.dust_likelihood_server(d.walk())
