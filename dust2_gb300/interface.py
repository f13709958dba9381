"""Host-side mirror of dust2's R verbs, over the C ABI.

R is not available to this engine's users here, so the R layer of dust2
(R/interface.R, R/interface-filter.R, R/interface-likelihood.R,
R/data.R, R/interface-continuous.R) is mirrored in Python with the same
verb names, argument meanings, 1-based indices, array shapes (state x
particle x group [x time]) and error messages.  Every computation goes to
the CUDA engine through include/dust2_gb300.h; nothing here simulates.
"""

import ctypes
import json
import math
import secrets

import numpy as np

from . import _lib
from ._lib import DustError, as_f64, as_size, as_u64, check, dptr, sptr, uptr


# ---------------------------------------------------------------------------
# Generators (dust_system_generator)

class Generator:
    """A compiled-in system (the `sir()` etc. generators of dust2)."""

    def __init__(self, name):
        buf = ctypes.create_string_buffer(1 << 16)
        check(_lib.lib().dust2_gb300_system_info(name.encode(), buf,
                                                  len(buf)))
        info = json.loads(buf.value.decode())
        self.name = info["name"]
        self.time_type = info["time_type"]
        self.has_compare = info["has_compare"]
        self.has_adjoint = info["has_adjoint"]
        self.parameters = info["parameters"]
        self.data_names = info["data"]
        self.default_dt = info.get("default_dt")
        self.n_pars = sum(p["length"] for p in self.parameters)

    def __call__(self):
        return self

    def __repr__(self):
        return f"<dust_system_generator: {self.name}>"

    def pack_pars(self, pars):
        """Flat parameter row (NaN = not given) from a dict."""
        if pars is None:
            pars = {}
        if not isinstance(pars, dict):
            raise DustError("Expected 'pars' to be a named list (dict)")
        known = {p["name"] for p in self.parameters}
        row = np.full(self.n_pars, np.nan)
        off = 0
        for p in self.parameters:
            if p["name"] in pars and pars[p["name"]] is not None:
                v = np.asarray(pars[p["name"]], dtype=np.float64).ravel()
                if p["length"] == 1:
                    if v.size != 1:
                        raise DustError(f"'{p['name']}' must be a scalar")
                    row[off] = v[0]
                else:
                    if v.size > p["length"]:
                        raise DustError(
                            f"'{p['name']}' has more than {p['length']} "
                            "values")
                    row[off:off + v.size] = v
            off += p["length"]
        extra = set(pars) - known
        if extra:
            # dust2 ignores unknown parameters (read by name in C++)
            pass
        return row


def sir():
    return Generator("sir")


def sir_cases():
    return Generator("sir_cases")


def sirode():
    return Generator("sirode")


def walk():
    return Generator("walk")


def logistic():
    return Generator("logistic")


def malaria():
    return Generator("malaria")


def seir_age():
    return Generator("seir_age")


def sirs():
    """SIRS written as a dust2 class (the compat plugin adapter)."""
    return Generator("sirs")


def _generator(generator):
    if isinstance(generator, Generator):
        return generator
    if callable(generator):
        g = generator()
        if isinstance(g, Generator):
            return g
    raise DustError("Expected 'generator' to be a 'dust_system_generator'")


# ---------------------------------------------------------------------------
# Argument helpers (R/util_assert.R, R/check.R, R/interface.R)

def _seed_words(seed):
    if seed is None:
        seed = secrets.randbits(63)
    if isinstance(seed, (bytes, bytearray)):
        if len(seed) % 32 != 0 or len(seed) == 0:
            raise DustError("Expected a raw seed of a multiple of 32 bytes")
        return np.frombuffer(bytes(seed), dtype="<u8").astype(np.uint64)
    if isinstance(seed, (int, np.integer)):
        return np.array([int(seed) % (1 << 64)], dtype=np.uint64)
    raise DustError("Expected 'seed' to be an integer or raw bytes")


def rng_streams(n_streams, seed):
    """Raw state (bytes) of the first n_streams streams of a seed."""
    words = _seed_words(seed)
    out = np.zeros(4 * n_streams, dtype=np.uint64)
    check(_lib.lib().dust2_gb300_rng_streams(uptr(words), words.size,
                                             n_streams, uptr(out)))
    return out.astype("<u8").tobytes()


def _scalar_size(x, name, allow_zero=False):
    if isinstance(x, bool) or not isinstance(x, (int, float, np.integer,
                                                 np.floating)):
        raise DustError(f"Expected '{name}' to be integer")
    if float(x) != math.floor(float(x)):
        raise DustError(f"Expected '{name}' to be integer")
    if x < (0 if allow_zero else 1):
        raise DustError(
            f"'{name}' must be at least {0 if allow_zero else 1}")
    return int(x)


def _check_dt(dt, generator):
    """R/filter-support.R check_system_dt: none for continuous time; a
    mixed-time system may go without (no updates, returned as 0)."""
    if generator.time_type == "continuous":
        if dt is not None:
            raise DustError("Can't use 'dt' with continuous-time systems")
        return None
    if dt is None:
        dt = generator.default_dt
    if dt is None and generator.time_type == "mixed":
        return 0.0
    dt = float(dt)
    if dt <= 0:
        raise DustError("Expected 'dt' to be greater than 0")
    if dt >= 1:
        if dt != math.floor(dt) or math.isinf(dt):
            raise DustError(
                "Expected 'dt' to be an integer, if greater than 1")
    else:
        inv = 1 / dt
        if abs(inv - round(inv)) > 1e-8:
            raise DustError("Expected 'dt' to be the inverse of an integer")
    return dt


def _fmod(n, m):
    """dust2's own remainder (R/util.R:114-116), not C fmod."""
    return np.floor(np.asarray(n) / m) * m - np.asarray(n)


def _check_time(time, dt, name="time"):
    if np.ndim(time) != 0:
        raise DustError(f"'{name}' must be a scalar")
    if isinstance(time, str):
        raise DustError(f"Expected '{name}' to be numeric")
    time = float(time)
    if dt is not None and dt > 0:
        if abs(_fmod(time, dt)) > math.sqrt(np.finfo(float).eps):
            if dt == 1:
                raise DustError(
                    f"'{name}' must be integer-like, because 'dt' is 1")
            raise DustError(f"'{name}' must be a multiple of 'dt' ({dt:g})")
    return time


def _check_index(index, n, name, unique=False):
    """1-based R index -> 0-based uintp array (None stays None)."""
    if index is None:
        return None
    idx = np.atleast_1d(np.asarray(index))
    if idx.size == 0:
        raise DustError(f"'{name}' must have nonzero length")
    if idx.dtype.kind not in "iuf":
        raise DustError(f"Expected an integer vector for '{name}'")
    if idx.dtype.kind == "f":
        bad = np.nonzero(idx != np.round(idx))[0]
        if bad.size:
            raise DustError(
                f"All values of '{name}' must be integer-like, but "
                f"'{name}[{bad[0] + 1}]' was not")
    idx = idx.astype(np.int64)
    bad = np.nonzero((idx < 1) | (idx > n))[0]
    if bad.size:
        i = bad[0]
        raise DustError(
            f"All values of '{name}' must be in [1, {n}], but "
            f"'{name}[{i + 1}]' was {idx[i]}")
    if unique and len(set(idx.tolist())) != idx.size:
        raise DustError(f"All values of '{name}' must be unique")
    return as_size(idx - 1)


def _check_pars(pars, n_groups, index_group, preserve_group_dimension):
    if preserve_group_dimension:
        expected = n_groups if index_group is None else len(index_group)
        if not isinstance(pars, (list, tuple)) or len(pars) != expected:
            what = "n_groups" if index_group is None else "index_group"
            got = len(pars) if isinstance(pars, (list, tuple)) else 1
            raise DustError(
                f"Expected 'pars' to have length {expected} to match "
                f"'{what}', but it had length {got}")
        return list(pars)
    return [pars]


def dust_ode_control(max_steps=10000, atol=1e-6, rtol=1e-6, step_size_min=0,
                     step_size_max=math.inf, critical_times=None,
                     debug_record_step_times=False, save_history=False):
    """R/interface-continuous.R:51-79."""
    if critical_times is None:
        critical_times = []
    critical_times = [float(x) for x in critical_times]
    if any(b <= a for a, b in zip(critical_times, critical_times[1:])):
        raise DustError("Values in 'critical_times' must be increasing")
    if max_steps < 1:
        raise DustError("'max_steps' must be at least 1")
    for nm, v in (("atol", atol), ("rtol", rtol)):
        if not v > 0:
            raise DustError(f"'{nm}' must be greater than 0")
    return {"max_steps": int(max_steps), "atol": float(atol),
            "rtol": float(rtol), "step_size_min": float(step_size_min),
            "step_size_max": float(step_size_max),
            "critical_times": critical_times,
            "debug_record_step_times": bool(debug_record_step_times),
            "save_history": bool(save_history)}


def _ode_control_struct(ctl):
    crit = as_f64(ctl["critical_times"]) if ctl["critical_times"] else None
    s = _lib.OdeControl(ctl["max_steps"], ctl["atol"], ctl["rtol"],
                        ctl["step_size_min"], ctl["step_size_max"],
                        dptr(crit), 0 if crit is None else crit.size,
                        1 if ctl["debug_record_step_times"] else 0)
    return s, crit


# ---------------------------------------------------------------------------
# Systems

class DustSystem:
    """A device-resident system (the `dust_system` object of dust2)."""

    def __init__(self, generator, handle, n_particles, n_groups, dt,
                 ode_control, deterministic, preserve_particle_dimension,
                 preserve_group_dimension):
        self.generator = generator
        self.name = generator.name
        self._handle = handle
        self.n_particles = n_particles
        self.n_groups = n_groups
        self.deterministic = deterministic
        self.preserve_particle_dimension = preserve_particle_dimension
        self.preserve_group_dimension = preserve_group_dimension
        self.time_control = {"dt": dt, "ode_control": ode_control}
        n_state = ctypes.c_size_t()
        n_p = ctypes.c_size_t()
        n_g = ctypes.c_size_t()
        check(_lib.lib().dust2_gb300_system_dim(
            handle, ctypes.byref(n_state), ctypes.byref(n_p),
            ctypes.byref(n_g)))
        self.n_state = n_state.value

    @property
    def ptr(self):
        return self._handle

    def __del__(self):
        h = getattr(self, "_handle", None)
        if h is not None and _lib._lib is not None:
            _lib._lib.dust2_gb300_system_free(h)
            self._handle = None

    def dim(self):
        return tuple([self.n_state] +
                     ([self.n_particles] if self.preserve_particle_dimension
                      else []) +
                     ([self.n_groups] if self.preserve_group_dimension
                      else []))


def dust_system_create(generator, pars=None, n_particles=1, n_groups=1,
                       time=0, dt=None, ode_control=None, seed=None,
                       deterministic=False, n_threads=1,
                       preserve_particle_dimension=False,
                       preserve_group_dimension=False):
    """R/interface.R:68-127."""
    gen = _generator(generator)
    n_particles = _scalar_size(n_particles, "n_particles")
    n_groups = _scalar_size(n_groups, "n_groups")
    _scalar_size(n_threads, "n_threads")
    if not isinstance(deterministic, bool):
        raise DustError("'deterministic' must be scalar logical")
    if gen.time_type == "discrete" and ode_control is not None:
        raise DustError("Can't use 'ode_control' with discrete-time systems")
    dt = _check_dt(dt, gen)
    time = _check_time(time, dt)
    preserve_particle_dimension = preserve_particle_dimension or \
        n_particles > 1
    preserve_group_dimension = preserve_group_dimension or n_groups > 1
    pars = _check_pars(pars, n_groups, None, preserve_group_dimension)
    flat = as_f64(np.concatenate([gen.pack_pars(p) for p in pars]))
    ctl = None
    ctl_struct = None
    if gen.time_type != "discrete":
        ctl = ode_control if ode_control is not None else dust_ode_control()
        ctl_struct, _keep = _ode_control_struct(ctl)
    words = _seed_words(seed)
    handle = ctypes.c_void_p()
    check(_lib.lib().dust2_gb300_system_alloc(
        gen.name.encode(), dptr(flat), n_groups, n_particles, time,
        0.0 if dt is None else dt,
        None if ctl_struct is None else ctypes.byref(ctl_struct),
        uptr(words), words.size, 1 if deterministic else 0,
        ctypes.byref(handle)))
    return DustSystem(gen, handle, n_particles, n_groups, dt, ctl,
                      deterministic, preserve_particle_dimension,
                      preserve_group_dimension)


def _check_sys(sys):
    if not isinstance(sys, DustSystem):
        raise DustError("Expected 'sys' to be a 'dust_system' object")


def _full_state(sys):
    out = np.empty(sys.n_state * sys.n_particles * sys.n_groups)
    check(_lib.lib().dust2_gb300_system_state(sys.ptr, dptr(out)))
    # C order [group][particle][state] -> [state, particle, group]
    return out.reshape(sys.n_groups, sys.n_particles,
                       sys.n_state).transpose(2, 1, 0)


def _shape_state(arr, preserve_particle, preserve_group):
    n_state, n_particles, n_groups = arr.shape
    if preserve_particle and preserve_group:
        return arr
    if preserve_particle or preserve_group:
        return arr.reshape(n_state, n_particles * n_groups, order="F")
    return arr.reshape(-1, order="F")


def dust_system_state(sys, index_state=None, index_particle=None,
                      index_group=None):
    """R/interface.R:154-160, r/system.hpp:89-161."""
    _check_sys(sys)
    s = _full_state(sys)
    if index_state is None and index_particle is None and index_group is None:
        return _shape_state(s, sys.preserve_particle_dimension,
                            sys.preserve_group_dimension)
    if not sys.preserve_group_dimension and index_group is not None:
        raise DustError("Can't provide 'index_group' for a non-grouped system")
    i_s = _check_index(index_state, sys.n_state, "index_state")
    i_p = _check_index(index_particle, sys.n_particles, "index_particle")
    i_g = _check_index(index_group, sys.n_groups, "index_group")
    if i_s is not None:
        s = s[i_s.astype(int), :, :]
    if i_p is not None:
        s = s[:, i_p.astype(int), :]
    if i_g is not None:
        s = s[:, :, i_g.astype(int)]
    return _shape_state(s, sys.preserve_particle_dimension,
                        sys.preserve_group_dimension)


def _prepare_state(state, index_state, index_particle, index_group, n_state,
                   n_particles, n_groups, preserve_particle_dimension,
                   preserve_group_dimension, name="state"):
    """R/interface.R prepare_state: validate shape and work out recycling."""
    def len_from_index(n, idx, nm):
        if idx is None:
            return n
        _check_index(idx, n, nm, unique=True)
        return np.atleast_1d(idx).size
    len_state = len_from_index(n_state, index_state, "index_state")
    len_particles = len_from_index(n_particles, index_particle,
                                   "index_particle")
    len_groups = len_from_index(n_groups, index_group, "index_group")
    state = np.asarray(state, dtype=np.float64)
    d = list(state.shape) if state.ndim > 0 else [1]
    rank = len(d)
    expected = [len_state]
    if preserve_particle_dimension:
        expected.append(len_particles)
    if preserve_group_dimension:
        expected.append(len_groups)
    rank_expected = len(expected)
    desc = {1: "vector", 2: "matrix"}
    if rank > rank_expected:
        re_ = desc.get(rank_expected, f"{rank_expected}-dimensional array")
        r_ = desc.get(rank, f"{rank}-dimensional array")
        raise DustError(f"Expected '{name}' to be a {re_} but was given a "
                        f"{r_}")
    if rank < rank_expected:
        d = d + [1] * (rank_expected - rank)
    ok = [a == b or (i > 0 and a == 1)
          for i, (a, b) in enumerate(zip(d, expected))]
    if all(ok):
        recycle_particle = n_particles > 1 and \
            (d[1] == 1 if preserve_particle_dimension else True)
        recycle_group = n_groups > 1 and d[-1] == 1
        value = np.asfortranarray(state.reshape(d, order="F")).ravel(
            order="F")
        return value, recycle_particle, recycle_group
    if not ok[0]:
        if rank == 1:
            msg = f"Expected '{name}' to have length {len_state}"
        elif rank == 2:
            msg = f"Expected '{name}' to have {len_state} rows"
        else:
            msg = f"Expected dimension 1 of '{name}' to be length {len_state}"
    elif not ok[1]:
        e = expected[1]
        es = "1" if e == 1 else f"1 or {e}"
        if rank == 2:
            msg = f"Expected '{name}' to have {es} columns"
        else:
            msg = f"Expected dimension 2 of '{name}' to be length {es}"
    else:
        e = expected[2]
        es = "1" if e == 1 else f"1 or {e}"
        msg = f"Expected dimension 3 of '{name}' to be length {es}"
    raise DustError(msg)


def dust_system_set_state(sys, state, index_state=None, index_particle=None,
                          index_group=None):
    """R/interface.R:236-250, internals.hpp:10-62."""
    _check_sys(sys)
    value, rp, rg = _prepare_state(
        state, index_state, index_particle, index_group, sys.n_state,
        sys.n_particles, sys.n_groups, sys.preserve_particle_dimension,
        sys.preserve_group_dimension)
    i_s = _check_index(index_state, sys.n_state, "index_state")
    i_p = _check_index(index_particle, sys.n_particles, "index_particle")
    i_g = _check_index(index_group, sys.n_groups, "index_group")
    value = as_f64(value)
    check(_lib.lib().dust2_gb300_system_set_state(
        sys.ptr, dptr(value), sptr(i_s), 0 if i_s is None else i_s.size,
        sptr(i_p), 0 if i_p is None else i_p.size,
        sptr(i_g), 0 if i_g is None else i_g.size, int(rp), int(rg)))


def dust_system_set_state_initial(sys):
    _check_sys(sys)
    check(_lib.lib().dust2_gb300_system_set_state_initial(sys.ptr))


def dust_system_time(sys):
    _check_sys(sys)
    t = ctypes.c_double()
    check(_lib.lib().dust2_gb300_system_time(sys.ptr, ctypes.byref(t)))
    return t.value


def dust_system_set_time(sys, time):
    _check_sys(sys)
    time = _check_time(time, sys.time_control["dt"])
    check(_lib.lib().dust2_gb300_system_set_time(sys.ptr, time))


def dust_system_rng_state(sys):
    """Raw generator state, 32 bytes per particle (little-endian words)."""
    _check_sys(sys)
    out = np.empty(4 * sys.n_particles * sys.n_groups, dtype=np.uint64)
    check(_lib.lib().dust2_gb300_system_rng_state(sys.ptr, uptr(out)))
    return out.astype("<u8").tobytes()


def dust_system_set_rng_state(sys, rng_state):
    _check_sys(sys)
    if not isinstance(rng_state, (bytes, bytearray)):
        raise DustError("Expected a raw vector for 'rng_state'")
    n = len(rng_state)
    expected = 32 * sys.n_particles * sys.n_groups
    if n != expected:
        raise DustError(f"Incorrect length for 'rng_state'; expected "
                        f"{expected} but given {n}")
    words = np.frombuffer(bytes(rng_state), dtype="<u8").astype(np.uint64)
    check(_lib.lib().dust2_gb300_system_set_rng_state(sys.ptr, uptr(words),
                                                      words.size))


def dust_system_update_pars(sys, pars):
    _check_sys(sys)
    pars = _check_pars(pars, sys.n_groups, None, sys.preserve_group_dimension)
    if len(pars) != sys.n_groups:
        raise DustError(f"Expected 'pars' to have length {sys.n_groups} to "
                        "match 'n_groups'")
    flat = as_f64(np.concatenate([sys.generator.pack_pars(p) for p in pars]))
    check(_lib.lib().dust2_gb300_system_update_pars(sys.ptr, dptr(flat),
                                                    None, 0))


def dust_system_run_to_time(sys, time):
    _check_sys(sys)
    if isinstance(time, str):
        raise DustError("Expected 'time' to be numeric")
    check(_lib.lib().dust2_gb300_system_run_to_time(sys.ptr, float(time)))


def _check_times(times, dt, name="times"):
    if times is None or isinstance(times, str):
        raise DustError(f"Expected '{name}' to be numeric")
    times = np.atleast_1d(np.asarray(times, dtype=np.float64))
    if times.size == 0:
        raise DustError(f"Expected at least one value in '{name}'")
    bad = np.nonzero(np.diff(times) <= 0)[0]
    if bad.size:
        msg = f"Values in '{name}' must be increasing"
        if bad.size > 5:
            msg += f"\n...and {bad.size - 4} other errors"
        raise DustError(msg)
    if dt is not None and 0 < dt <= 1:
        rem = _fmod(times, dt)
        bad = np.nonzero(np.abs(rem) > math.sqrt(np.finfo(float).eps))[0]
        if bad.size:
            if dt == 1:
                raise DustError(f"Values in '{name}' must be integer-like, "
                                "because 'dt' is 1")
            raise DustError(f"Values in '{name}' must be multiples of 'dt' "
                            f"({dt:g})")
    return times


def dust_system_simulate(sys, times, index_state=None):
    """R/interface.R:400-412, r/system.hpp:286-327."""
    _check_sys(sys)
    times = as_f64(_check_times(times, sys.time_control["dt"]))
    i_s = _check_index(index_state, sys.n_state, "index_state")
    n_save = sys.n_state if i_s is None else i_s.size
    out = np.empty(n_save * sys.n_particles * sys.n_groups * times.size)
    check(_lib.lib().dust2_gb300_system_simulate(
        sys.ptr, dptr(times), times.size, sptr(i_s),
        0 if i_s is None else i_s.size, dptr(out)))
    arr = out.reshape(times.size, sys.n_groups, sys.n_particles,
                      n_save).transpose(3, 2, 1, 0)
    pp, pg = sys.preserve_particle_dimension, sys.preserve_group_dimension
    if pp and pg:
        return arr
    if pp or pg:
        return arr.reshape(n_save, sys.n_particles * sys.n_groups,
                           times.size, order="F")
    return arr.reshape(n_save * sys.n_particles * sys.n_groups, times.size,
                       order="F")


def dust_system_reorder(sys, index):
    """R/interface.R:437-443, r/system.hpp:199-221 (1-based index)."""
    _check_sys(sys)
    idx = np.asarray(index)
    n_total = sys.n_particles * sys.n_groups
    flat = idx.reshape(-1, order="F")
    if flat.size != n_total:
        raise DustError(f"Expected an index of length {n_total}")
    if np.any(flat < 1) or np.any(flat > sys.n_particles):
        raise DustError(
            f"Expected 'index' values to lie in [1, {sys.n_particles}]")
    z = as_size(flat.astype(np.int64) - 1)
    check(_lib.lib().dust2_gb300_system_reorder(sys.ptr, sptr(z), z.size))


def _data_row(generator, d):
    row = np.full(len(generator.data_names), np.nan)
    if d is None:
        return row
    for i, nm in enumerate(generator.data_names):
        if nm in d and d[nm] is not None:
            v = d[nm]
            row[i] = np.nan if v is None else float(v)
    return row


def dust_system_compare_data(sys, data):
    """R/interface.R:523-537, r/system.hpp:258-284."""
    _check_sys(sys)
    if not sys.generator.has_compare:
        raise DustError(
            f"Can't compare against data; the '{sys.name}' system does not "
            "have 'compare_data' support")
    if not sys.preserve_group_dimension:
        data = [data]
    if len(data) != sys.n_groups:
        raise DustError(f"Expected 'data' to have length {sys.n_groups}, but "
                        f"it had length {len(data)}")
    flat = as_f64(np.concatenate([_data_row(sys.generator, d) for d in data]))
    out = np.empty(sys.n_particles * sys.n_groups)
    check(_lib.lib().dust2_gb300_system_compare_data(sys.ptr, dptr(flat),
                                                     len(data), dptr(out)))
    res = out.reshape(sys.n_groups, sys.n_particles).T
    if sys.preserve_group_dimension and sys.preserve_particle_dimension:
        return res
    return res.reshape(-1, order="F")


def dust_system_internals(sys, include_coefficients=False):
    """R/interface.R:474-504 (statistics only)."""
    _check_sys(sys)
    if sys.generator.time_type == "discrete":
        return None
    n = sys.n_particles * sys.n_groups
    ss = np.empty(n)
    er = np.empty(n)
    ns = np.empty(n, dtype=np.int64)
    na = np.empty(n, dtype=np.int64)
    nr = np.empty(n, dtype=np.int64)
    check(_lib.lib().dust2_gb300_system_internals(
        sys.ptr, dptr(ss), dptr(er), ns.ctypes.data_as(_lib.c_i64_p),
        na.ctypes.data_as(_lib.c_i64_p), nr.ctypes.data_as(_lib.c_i64_p)))
    step_times = []
    for k in range(n):
        cap = 4096
        buf = np.empty(cap)
        cnt = ctypes.c_size_t()
        check(_lib.lib().dust2_gb300_system_step_times(
            sys.ptr, k, dptr(buf), cap, ctypes.byref(cnt)))
        step_times.append(buf[:min(cap, cnt.value)].copy())
    return {"particle": np.arange(1, n + 1), "step_size": ss, "error": er,
            "n_steps": ns, "n_steps_accepted": na, "n_steps_rejected": nr,
            "step_times": step_times}


# ---------------------------------------------------------------------------
# Filters and likelihoods

def dust_filter_data(data, time=None, group=None):
    """R/data.R:24-112 for a dict of columns."""
    if not isinstance(data, dict):
        raise DustError("Expected 'data' to be a data.frame (dict of columns)")
    cols = {k: np.asarray(v) for k, v in data.items()}
    lens = {v.size for v in cols.values()}
    if len(lens) != 1:
        raise DustError("All columns of 'data' must have the same length")
    if lens.pop() == 0:
        raise DustError("Expected 'data' to have at least one row")
    time = time or "time"
    if time not in cols:
        raise DustError(f"Did not find column '{time}' in 'data'")
    t = cols[time].astype(np.float64)
    if np.any(t != np.round(t)):
        raise DustError(f"Expected 'data[[\"{time}\"]]' to be integer-like")
    plausibly_grouped = len(np.unique(t)) < t.size
    if plausibly_grouped and group is None:
        if "group" not in cols:
            raise DustError("'data' looks grouped, but 'group' not specified "
                            "and column 'group' not found")
        group = "group"
    elif group is not None and group not in cols:
        raise DustError(f"Did not find column '{group}' in 'data'")
    if group is None:
        order = np.argsort(t, kind="stable")
        groups = None
        n_groups = 1
    else:
        g = cols[group]
        groups = list(dict.fromkeys(g.tolist()))
        n_groups = len(groups)
        if g.dtype.kind in "iuf":
            if set(groups) != set(range(1, n_groups + 1)):
                raise DustError(
                    f"Expected 'data[[\"{group}\"]]' to contain integer "
                    f"values in [1, {n_groups}], and contain all those values")
        times_by_group = {x: tuple(sorted(t[g == x])) for x in groups}
        if len(set(times_by_group.values())) > 1:
            raise DustError("Not all groups in 'data' have the same times")
        order = np.lexsort((g, t))
    other = [k for k in cols if k not in (time, group)]
    if not other:
        raise DustError("Expected 'data' to have at least one column in "
                        f"addition to '{time}'")
    out = {k: v[order] for k, v in cols.items()}
    return {"data": out, "time": time, "group": group, "groups": groups,
            "n_groups": n_groups}


def _prepare_data(data, n_groups, shared_data, generator):
    """R/data.R:114-175: time-major rows of the system's data columns."""
    fd = data if (isinstance(data, dict) and "n_groups" in data and
                  "data" in data) else dust_filter_data(data)
    n_groups_data = fd["n_groups"]
    if n_groups is None:
        if shared_data:
            raise DustError(
                "Can't use 'shared_data = TRUE' with 'n_groups = NULL'")
        n_groups = n_groups_data
    else:
        expected = 1 if shared_data else n_groups
        if n_groups_data != expected:
            raise DustError(f"Expected 'data' to have {expected} groups, but "
                            f"it had {n_groups_data}")
    cols = fd["data"]
    t = cols[fd["time"]].astype(np.float64)
    if fd["group"] is not None:
        t = t[cols[fd["group"]] == fd["groups"][0]]
    n_time = t.size
    rows = np.full((n_time, n_groups_data, len(generator.data_names)), np.nan)
    for i, nm in enumerate(generator.data_names):
        if nm in cols:
            v = cols[nm].astype(np.float64)
            rows[:, :, i] = v.reshape(n_time, n_groups_data)
    return {"time": t, "n_groups": n_groups,
            "n_groups_data": n_groups_data, "rows": rows,
            "groups": fd["groups"]}


class DustLikelihood:
    """A particle filter (the `dust_filter`/`dust_likelihood` object)."""

    def __init__(self, generator, time_start, data, n_particles, n_groups,
                 dt, initial_rng_state, preserve_group_dimension,
                 n_particles_per_group=None, ode_control=None):
        self.generator = generator
        self.ode_control = ode_control
        self.time_start = time_start
        self.data = data
        self.n_particles = n_particles
        self.n_particles_per_group = n_particles_per_group
        self.n_groups = n_groups
        self.dt = dt
        self.initial_rng_state = initial_rng_state
        self.preserve_group_dimension = preserve_group_dimension
        self.preserve_particle_dimension = True
        self.deterministic = False
        self._handle = None
        self.n_state = None
        # run options, applied to the engine object when it is created
        self.serial_resample = False
        self.fused_tail = True
        self.step_shape = None  # (block, per_tile) forced, else tuned

    @property
    def ptr(self):
        return self._handle

    def apply_options(self):
        lib = _lib.lib()
        check(lib.dust2_gb300_filter_set_serial_resample(
            self._handle, 1 if self.serial_resample else 0))
        check(lib.dust2_gb300_filter_set_fused_tail(
            self._handle, 1 if self.fused_tail else 0))
        if self.step_shape is not None and \
                self.generator.time_type == "discrete":
            check(lib.dust2_gb300_filter_set_step_shape(
                self._handle, int(self.step_shape[0]),
                int(self.step_shape[1]), int(bool(self.step_shape[2]))))

    def initialise(self, pars):
        flat = as_f64(np.concatenate([self.generator.pack_pars(p)
                                      for p in pars]))
        rows = as_f64(self.data["rows"])
        times = as_f64(self.data["time"])
        words = np.frombuffer(self.initial_rng_state,
                              dtype="<u8").astype(np.uint64)
        handle = ctypes.c_void_p()
        if self.generator.time_type == "mixed":
            if self.n_particles_per_group is not None:
                raise DustError("Mixed-time filters need equal particle "
                                "counts per group")
            c = self.ode_control if self.ode_control is not None else \
                dust_ode_control()
            ctl, keep = _ode_control_struct(c)
            check(_lib.lib().dust2_gb300_filter_alloc_continuous(
                self.generator.name.encode(), dptr(flat), self.n_groups,
                self.n_particles, self.time_start, dptr(times), times.size,
                dptr(rows), self.data["n_groups_data"], self.dt,
                ctypes.byref(ctl), uptr(words), words.size,
                ctypes.byref(handle)))
            del keep
        elif self.n_particles_per_group is None:
            check(_lib.lib().dust2_gb300_filter_alloc(
                self.generator.name.encode(), dptr(flat), self.n_groups,
                self.n_particles, self.time_start, dptr(times), times.size,
                dptr(rows), self.data["n_groups_data"], self.dt,
                uptr(words), words.size, ctypes.byref(handle)))
        else:
            npg = as_size(self.n_particles_per_group)
            check(_lib.lib().dust2_gb300_filter_alloc_uneven(
                self.generator.name.encode(), dptr(flat), self.n_groups,
                sptr(npg), self.time_start, dptr(times), times.size,
                dptr(rows), self.data["n_groups_data"], self.dt,
                uptr(words), words.size, ctypes.byref(handle)))
        self._handle = handle
        self.initial_rng_state = None
        self.apply_options()
        n_state = ctypes.c_size_t()
        n_tot = ctypes.c_size_t()
        n_g = ctypes.c_size_t()
        n_t = ctypes.c_size_t()
        check(_lib.lib().dust2_gb300_filter_dim(
            handle, ctypes.byref(n_state), ctypes.byref(n_tot),
            ctypes.byref(n_g), ctypes.byref(n_t)))
        self.n_state = n_state.value
        self.n_particles_total = n_tot.value

    def __del__(self):
        h = getattr(self, "_handle", None)
        if h is not None and _lib._lib is not None:
            _lib._lib.dust2_gb300_filter_free(h)
            self._handle = None


def dust_filter_create(generator, time_start, data, n_particles,
                       n_groups=None, dt=None, ode_control=None,
                       shared_data=False, n_threads=1,
                       preserve_group_dimension=False, seed=None):
    """R/interface-filter.R:37-97."""
    gen = _generator(generator)
    if not gen.has_compare:
        raise DustError(f"Can't create filter; the '{gen.name}' system does "
                        "not have 'compare_data' support")
    uneven = np.ndim(n_particles) > 0
    if uneven:
        npg = [int(x) for x in n_particles]
        if any(x < 1 for x in npg):
            raise DustError("'n_particles' must be at least 1")
    else:
        n_particles = _scalar_size(n_particles, "n_particles")
    d = _prepare_data(data, n_groups, shared_data, gen)
    time_start = float(time_start)
    if time_start > d["time"][0]:
        raise DustError(f"'time_start' ({time_start:g}) is later than the "
                        f"first time in 'data' ({d['time'][0]:g})")
    if gen.time_type == "continuous":
        raise DustError(
            "Can't use 'dust_filter_create()' with continuous-time models")
    if gen.time_type == "discrete" and ode_control is not None:
        raise DustError("Can't use 'ode_control' with discrete-time systems")
    dt = _check_dt(dt, gen)
    n_groups = d["n_groups"]
    if uneven and len(npg) != n_groups:
        raise DustError("Expected one particle count per group")
    preserve_group_dimension = preserve_group_dimension or n_groups > 1
    n_streams = (sum(x + 2 for x in npg) if uneven
                 else n_groups * (n_particles + 2))
    initial = rng_streams(n_streams, seed)
    return DustLikelihood(gen, time_start, d,
                          max(npg) if uneven else n_particles, n_groups, dt,
                          initial, preserve_group_dimension,
                          npg if uneven else None, ode_control)


class DustUnfilter:
    """A deterministic likelihood (the `dust_unfilter` object)."""

    def __init__(self, generator, time_start, data, n_particles, n_groups,
                 dt, ode_control, preserve_particle_dimension,
                 preserve_group_dimension):
        self.generator = generator
        self.time_start = time_start
        self.data = data
        self.n_particles = n_particles
        self.n_particles_per_group = None
        self.n_groups = n_groups
        self.dt = dt
        self.ode_control = ode_control
        self.preserve_particle_dimension = preserve_particle_dimension
        self.preserve_group_dimension = preserve_group_dimension
        self.deterministic = True
        self._handle = None
        self.n_state = None

    @property
    def ptr(self):
        return self._handle

    def initialise(self, pars):
        flat = as_f64(np.concatenate([self.generator.pack_pars(p)
                                      for p in pars]))
        rows = as_f64(self.data["rows"])
        times = as_f64(self.data["time"])
        ctl = None
        keep = None
        if self.generator.time_type != "discrete":
            c = self.ode_control if self.ode_control is not None else \
                dust_ode_control()
            ctl, keep = _ode_control_struct(c)
        handle = ctypes.c_void_p()
        check(_lib.lib().dust2_gb300_unfilter_alloc(
            self.generator.name.encode(), dptr(flat), self.n_groups,
            self.n_particles, self.time_start, dptr(times), times.size,
            dptr(rows), self.data["n_groups_data"],
            self.dt if self.dt is not None else 0.0,
            None if ctl is None else ctypes.byref(ctl),
            ctypes.byref(handle)))
        del keep
        self._handle = handle
        n_state = ctypes.c_size_t()
        n_tot = ctypes.c_size_t()
        n_g = ctypes.c_size_t()
        n_t = ctypes.c_size_t()
        check(_lib.lib().dust2_gb300_unfilter_dim(
            handle, ctypes.byref(n_state), ctypes.byref(n_tot),
            ctypes.byref(n_g), ctypes.byref(n_t)))
        self.n_state = n_state.value

    def __del__(self):
        h = getattr(self, "_handle", None)
        if h is not None and _lib._lib is not None:
            _lib._lib.dust2_gb300_unfilter_free(h)
            self._handle = None


def dust_unfilter_create(generator, time_start, data, n_particles=1,
                         n_groups=None, dt=None, ode_control=None,
                         shared_data=False, n_threads=1,
                         preserve_particle_dimension=False,
                         preserve_group_dimension=False):
    """R/interface-unfilter.R:20-70."""
    gen = _generator(generator)
    if not gen.has_compare:
        raise DustError(f"Can't create unfilter; the '{gen.name}' system "
                        "does not have 'compare_data' support")
    n_particles = _scalar_size(n_particles, "n_particles")
    d = _prepare_data(data, n_groups, shared_data, gen)
    time_start = float(time_start)
    if time_start > d["time"][0]:
        raise DustError(f"'time_start' ({time_start:g}) is later than the "
                        f"first time in 'data' ({d['time'][0]:g})")
    if gen.time_type == "discrete":
        if ode_control is not None:
            raise DustError(
                "Can't use 'ode_control' with discrete-time systems")
        dt = _check_dt(dt, gen)
    elif gen.time_type == "mixed":
        dt = _check_dt(dt, gen)
    elif dt is not None:
        raise DustError("Can't use 'dt' with continuous-time systems")
    n_groups = d["n_groups"]
    return DustUnfilter(gen, time_start, d, n_particles, n_groups, dt,
                        ode_control,
                        preserve_particle_dimension or n_particles > 1,
                        preserve_group_dimension or n_groups > 1)


def _check_lik(obj):
    if not isinstance(obj, (DustLikelihood, DustUnfilter)):
        raise DustError("Expected 'obj' to be a 'dust_likelihood' object")


def dust_likelihood_run(obj, pars, initial=None, save_trajectories=False,
                        index_state=None, index_group=None,
                        save_snapshots=None, adjoint=None):
    """R/interface-likelihood.R:48-114, r/filter.hpp:112-143,
    r/unfilter.hpp:20-62.  `adjoint` (unfilters; default: whether the
    system has adjoint support) runs through the state history and makes
    the gradient available to dust_likelihood_last_gradient."""
    _check_lik(obj)
    if adjoint is None:
        adjoint = obj.generator.has_adjoint
    elif not isinstance(adjoint, (bool, np.bool_)):
        raise DustError("'adjoint' must be a scalar logical")
    snap_index = None
    if save_snapshots is not None:
        # R/interface-likelihood.R:83-92
        snaps = np.atleast_1d(np.asarray(save_snapshots, dtype=float))
        if snaps.size > 1 and np.any(np.diff(snaps) <= 0):
            raise DustError("'save_snapshots' must be increasing")
        times = np.asarray(obj.data["time"], dtype=float)
        ok = np.isin(snaps, times)
        if not np.all(ok):
            bad = ", ".join(f"{v:g}" for v in snaps[~ok])
            raise DustError("All elements of 'save_snapshots' must be found "
                            f"in 'time' (invalid: {bad})")
        snap_index = as_size(np.searchsorted(times, snaps))
    ig = _check_index(index_group, obj.n_groups, "index_group", unique=True)
    if pars is not None:
        pars = _check_pars(pars, obj.n_groups,
                           None if ig is None else list(ig),
                           obj.preserve_group_dimension)
    if obj.ptr is None:
        if pars is None:
            raise DustError(
                "'pars' cannot be NULL, as 'obj' is not initialised")
        if ig is not None:
            raise DustError(
                "'index_group' must be NULL, as 'obj' is not initialised")
        obj.initialise(pars)
    elif pars is not None:
        flat = as_f64(np.concatenate([obj.generator.pack_pars(p)
                                      for p in pars]))
        update = (_lib.lib().dust2_gb300_unfilter_update_pars
                  if isinstance(obj, DustUnfilter) else
                  _lib.lib().dust2_gb300_filter_update_pars)
        check(update(obj.ptr, dptr(flat), sptr(ig),
                     0 if ig is None else ig.size))
    init = None
    if initial is not None:
        if obj.n_particles_per_group is not None:
            raise DustError("'initial' needs equal particle counts per group")
        value, rp, rg = _prepare_state(
            initial, None, None, None, obj.n_state, obj.n_particles,
            obj.n_groups, True, obj.preserve_group_dimension,
            name="initial")
        full = np.asarray(value).reshape(
            (obj.n_state, 1 if rp else obj.n_particles,
             1 if rg else obj.n_groups), order="F")
        full = np.broadcast_to(full, (obj.n_state, obj.n_particles,
                                      obj.n_groups))
        init = as_f64(full.transpose(2, 1, 0))
    n_out = obj.n_groups if ig is None else ig.size
    ist = None
    if save_trajectories:
        ist = _check_index(index_state, obj.n_state, "index_state")
    if isinstance(obj, DustUnfilter):
        check(_lib.lib().dust2_gb300_unfilter_set_save_trajectories(
            obj.ptr, 1 if save_trajectories else 0, sptr(ist),
            0 if ist is None else ist.size))
        check(_lib.lib().dust2_gb300_unfilter_set_save_snapshots(
            obj.ptr, sptr(snap_index), 0 if snap_index is None else
            snap_index.size))
        # r/unfilter.hpp:48-61: n_particles values per group
        ll = np.empty(n_out * obj.n_particles)
        run = (_lib.lib().dust2_gb300_unfilter_run_adjoint if adjoint else
               _lib.lib().dust2_gb300_unfilter_run)
        check(run(obj.ptr, dptr(init), sptr(ig),
                  0 if ig is None else ig.size, dptr(ll)))
        ll = ll.reshape(n_out, obj.n_particles).T
        if obj.preserve_particle_dimension and obj.preserve_group_dimension:
            return ll
        if obj.preserve_particle_dimension:
            return ll[:, 0]
        if obj.preserve_group_dimension:
            return ll[0, :]
        return float(ll[0, 0])
    check(_lib.lib().dust2_gb300_filter_set_save_trajectories(
        obj.ptr, 1 if save_trajectories else 0, sptr(ist),
        0 if ist is None else ist.size))
    check(_lib.lib().dust2_gb300_filter_set_save_snapshots(
        obj.ptr, sptr(snap_index), 0 if snap_index is None else
        snap_index.size))
    ll = np.empty(n_out)
    check(_lib.lib().dust2_gb300_filter_run(
        obj.ptr, dptr(init), sptr(ig), 0 if ig is None else ig.size,
        dptr(ll)))
    if not obj.preserve_group_dimension:
        return float(ll[0])
    return ll


def _packing(obj):
    """[(name, dims)] of the object's state packing (the system class's
    packing_state)."""
    if isinstance(obj, DustSystem):
        fn, ptr = _lib.lib().dust2_gb300_system_packing_state, obj.ptr
    elif isinstance(obj, (DustLikelihood, DustUnfilter)):
        if obj.ptr is None:
            raise DustError("Packer is not yet ready: likelihood has not "
                            "yet been run")
        fn = (_lib.lib().dust2_gb300_unfilter_packing_state
              if isinstance(obj, DustUnfilter) else
              _lib.lib().dust2_gb300_filter_packing_state)
        ptr = obj.ptr
    else:
        raise DustError("Expected 'obj' to be a 'dust_system' or a "
                        "'dust_likelihood'")
    need = ctypes.c_size_t()
    check(fn(ptr, None, 0, ctypes.byref(need)))
    buf = ctypes.create_string_buffer(need.value + 1)
    check(fn(ptr, buf, len(buf), None))
    return [(e["name"], list(e["dims"])) for e in json.loads(buf.value)]


def dust_unpack_index(obj):
    """R/tools.R dust_unpack_index (monty_packer's index()): each named
    block of state and its 1-based positions in the state dimension."""
    out = {}
    pos = 0
    for name, dims in _packing(obj):
        n = int(np.prod(dims)) if dims else 1
        out[name] = np.arange(pos + 1, pos + n + 1)
        pos += n
    return out


def dust_unpack_state(obj, state):
    """R/tools.R dust_unpack_state (monty_packer's unpack()): split the
    first (state) dimension of `state` into the named blocks; a scalar
    block drops that dimension, an array block keeps its own
    dimensions (column-major, as R arrays)."""
    state = np.asarray(state)
    out = {}
    pos = 0
    rest = state.shape[1:]
    for name, dims in _packing(obj):
        n = int(np.prod(dims)) if dims else 1
        block = state[pos:pos + n]
        if not dims:
            out[name] = block[0]
        elif len(dims) > 1:
            out[name] = block.reshape(tuple(dims) + rest, order="F")
        else:
            out[name] = block
        pos += n
    if pos != state.shape[0]:
        raise DustError(f"Expected 'state' to have {pos} rows, but it had "
                        f"{state.shape[0]}")
    return out


def dust_likelihood_last_gradient(obj):
    """R/interface-likelihood.R:309-331, r/unfilter.hpp:153-180: the
    gradient of the last adjoint run's log-likelihood with respect to the
    system's packing_gradient parameters (for sir: beta, gamma, I0),
    shaped as the reference shapes it: a vector for one particle in one
    group, (n_gradient, n_particles * n_groups) when one of the
    dimensions is preserved, (n_gradient, n_particles, n_groups) when
    both are."""
    _check_lik(obj)
    if obj.ptr is None:
        raise DustError("Gradient is not current: likelihood has not yet "
                        "been run")
    if isinstance(obj, DustLikelihood):
        raise DustError("Gradients need a deterministic likelihood "
                        "(an unfilter)")
    n_gr = ctypes.c_size_t()
    n_grp = ctypes.c_size_t()
    check(_lib.lib().dust2_gb300_unfilter_gradient_dim(
        obj.ptr, ctypes.byref(n_gr), ctypes.byref(n_grp)))
    if n_gr.value == 0:
        raise DustError(f"The '{obj.generator.name}' system does not "
                        "support adjoint methods")
    if n_grp.value == 0:
        raise DustError("System was not run with 'adjoint = TRUE'")
    out = np.empty(n_gr.value * obj.n_particles * n_grp.value)
    check(_lib.lib().dust2_gb300_unfilter_last_gradient(obj.ptr, dptr(out)))
    pp, pg = obj.preserve_particle_dimension, obj.preserve_group_dimension
    if pp and pg:
        return out.reshape((n_gr.value, obj.n_particles, n_grp.value),
                           order="F")
    if pp or pg:
        return out.reshape((n_gr.value, obj.n_particles * n_grp.value),
                           order="F")
    return out


def _unfilter_saved(obj, what):
    """r/unfilter.hpp:64-125: trajectories or snapshots of an unfilter
    (no reordering, no particle selection), shaped (state, particle,
    group, time) when both dimensions are preserved, (state, particle x
    group, time) when one is, (state x particle x group, time) when
    neither is."""
    dims = [ctypes.c_size_t() for _ in range(4)]
    dim_fn = getattr(_lib.lib(), f"dust2_gb300_unfilter_{what}_dim")
    check(dim_fn(obj.ptr, *[ctypes.byref(x) for x in dims]))
    n_state, n_particles, n_groups, n_time = [x.value for x in dims]
    out = np.empty(n_state * n_particles * n_groups * n_time)
    name = "trajectories" if what == "trajectory" else "snapshots"
    check(getattr(_lib.lib(), f"dust2_gb300_unfilter_last_{name}")(
        obj.ptr, dptr(out)))
    pp, pg = obj.preserve_particle_dimension, obj.preserve_group_dimension
    if pp and pg:
        shape = (n_state, n_particles, n_groups, n_time)
    elif pp or pg:
        shape = (n_state, n_particles * n_groups, n_time)
    else:
        shape = (n_state * n_particles * n_groups, n_time)
    return out.reshape(shape, order="F")


def dust_likelihood_last_snapshots(obj, select_random_particle=False):
    """R/interface-likelihood.R:255-266, r/filter.hpp:98-137: array
    (state, particle, group, snapshot) with dust2's dimension dropping."""
    _check_lik(obj)
    if obj.ptr is None:
        raise DustError("Snapshots are not current")
    if isinstance(obj, DustUnfilter):
        return _unfilter_saved(obj, "snapshot")
    dims = [ctypes.c_size_t() for _ in range(4)]
    sel = 1 if select_random_particle else 0
    check(_lib.lib().dust2_gb300_filter_snapshot_dim(
        obj.ptr, sel, *[ctypes.byref(x) for x in dims]))
    n_state, n_particles, n_groups, n_snap = [x.value for x in dims]
    out = np.empty(n_state * n_particles * n_groups * n_snap)
    check(_lib.lib().dust2_gb300_filter_last_snapshots(obj.ptr, sel,
                                                       dptr(out)))
    if select_random_particle:
        shape = ((n_state, n_groups, n_snap) if obj.preserve_group_dimension
                 else (n_state, n_groups * n_snap))
    elif obj.preserve_group_dimension:
        shape = (n_state, n_particles, n_groups, n_snap)
    else:
        shape = (n_state, n_particles * n_groups, n_snap)
    return out.reshape(shape, order="F")


def dust_likelihood_last_trajectories(obj, select_random_particle=False):
    """R/interface-likelihood.R dust_likelihood_last_trajectories,
    r/filter.hpp:55-96: array (state, particle, group, time) with dust2's
    dimension dropping."""
    _check_lik(obj)
    if obj.ptr is None:
        raise DustError("Trajectories are not current")
    if isinstance(obj, DustUnfilter):
        return _unfilter_saved(obj, "trajectory")
    dims = [ctypes.c_size_t() for _ in range(4)]
    sel = 1 if select_random_particle else 0
    check(_lib.lib().dust2_gb300_filter_trajectory_dim(
        obj.ptr, sel, *[ctypes.byref(x) for x in dims]))
    n_state, n_particles, n_groups, n_time = [x.value for x in dims]
    out = np.empty(n_state * n_particles * n_groups * n_time)
    check(_lib.lib().dust2_gb300_filter_last_trajectories(obj.ptr, sel,
                                                          dptr(out)))
    if select_random_particle:
        shape = ((n_state, n_groups, n_time) if obj.preserve_group_dimension
                 else (n_state, n_groups * n_time))
    elif obj.preserve_group_dimension:
        shape = (n_state, n_particles, n_groups, n_time)
    else:
        shape = (n_state, n_particles * n_groups, n_time)
    return out.reshape(shape, order="F")


def dust_likelihood_rng_state(obj):
    """Raw state: per group 2 filter streams then the particle streams."""
    _check_lik(obj)
    if obj.ptr is None:
        return obj.initial_rng_state
    n = 4 * (obj.n_particles_total + 2 * obj.n_groups)
    out = np.empty(n, dtype=np.uint64)
    check(_lib.lib().dust2_gb300_filter_rng_state(obj.ptr, uptr(out), n))
    return out.astype("<u8").tobytes()


def dust_likelihood_set_rng_state(obj, rng_state):
    _check_lik(obj)
    if obj.ptr is None:
        if len(rng_state) != len(obj.initial_rng_state):
            raise DustError("Incorrect length for 'rng_state'")
        obj.initial_rng_state = bytes(rng_state)
        return
    words = np.frombuffer(bytes(rng_state), dtype="<u8").astype(np.uint64)
    check(_lib.lib().dust2_gb300_filter_set_rng_state(obj.ptr, uptr(words),
                                                      words.size))


def dust_likelihood_last_state(obj, select_random_particle=False):
    """R/interface-likelihood.R, r/filter.hpp:233-271."""
    _check_lik(obj)
    if obj.ptr is None:
        raise DustError("State is not current")
    if select_random_particle:
        out = np.empty(obj.n_state * obj.n_groups)
    else:
        out = np.empty(obj.n_state * obj.n_particles_total)
    check(_lib.lib().dust2_gb300_filter_last_state(
        obj.ptr, 1 if select_random_particle else 0, dptr(out)))
    if select_random_particle:
        arr = out.reshape(obj.n_groups, obj.n_state).T
        return arr if obj.preserve_group_dimension else arr[:, 0]
    if obj.n_particles_per_group is not None:
        return out
    arr = out.reshape(obj.n_groups, obj.n_particles, obj.n_state).transpose(
        2, 1, 0)
    if obj.preserve_group_dimension:
        return arr
    return arr[:, :, 0]


def dust_likelihood_set_step_shape(obj, block, per_tile=0, persistent=False):
    """Force the step kernel's launch shape of a discrete-time filter:
    group tiles of `block` threads (per_tile 0) or one-warp tiles of
    per_tile particles (block 32), one block per tile or (persistent) a
    device-filling grid taking tiles from a work queue; turns the
    autotuner off.  Results do not depend on it."""
    _check_lik(obj)
    obj.step_shape = (int(block), int(per_tile), bool(persistent))
    if obj.ptr is not None:
        obj.apply_options()


def dust_likelihood_step_shape(obj):
    """The step kernel's launch shape in use: block, per_tile, persistent,
    the number of candidates the autotuner timed and the chosen one's
    time (ms)."""
    _check_lik(obj)
    if obj.ptr is None:
        raise DustError("The filter has not run yet")
    b, p, q, n = (ctypes.c_int32() for _ in range(4))
    ms = ctypes.c_double()
    check(_lib.lib().dust2_gb300_filter_step_shape(
        obj.ptr, ctypes.byref(b), ctypes.byref(p), ctypes.byref(q),
        ctypes.byref(n), ctypes.byref(ms)))
    return {"block": b.value, "per_tile": p.value,
            "persistent": bool(q.value), "n_candidates": n.value,
            "best_ms": ms.value}


def resample_weight(w, u):
    """Systematic resampling indices (0-based) of weights w with uniform u,
    on the GPU (dust2's test_resample_weight, src/test.cpp)."""
    w = as_f64(w)
    idx = np.empty(w.size, dtype=np.uintp)
    check(_lib.lib().dust2_gb300_resample_weight(dptr(w), w.size, float(u),
                                                 sptr(idx)))
    return idx.astype(np.int64)


def scale_log_weights(w):
    """(log mean weight, scaled weights) on the GPU (dust2's
    test_scale_log_weights)."""
    w = np.array(w, dtype=np.float64)
    r = ctypes.c_double()
    check(_lib.lib().dust2_gb300_scale_log_weights(dptr(w), w.size,
                                                   ctypes.byref(r)))
    return r.value, w


def _check_filter(obj):
    if not isinstance(obj, DustLikelihood):
        raise DustError("Expected 'obj' to be a particle filter")


def dust_likelihood_set_serial_resample(obj, serial):
    """Verification mode: resample every group with the serial algorithm.
    Kept by the object, so it may be set before the first run."""
    _check_filter(obj)
    obj.serial_resample = bool(serial)
    if obj.ptr is not None:
        obj.apply_options()


def dust_likelihood_set_fused_tail(obj, fused):
    """Tuning switch: run each observation's weights, resampling and
    reorder as one launch when every group has at most 1024 particles
    (the default), or as separate kernels.  The results are identical.
    Kept by the object, so it may be set before the first run."""
    _check_filter(obj)
    obj.fused_tail = bool(fused)
    if obj.ptr is not None:
        obj.apply_options()


def dust_likelihood_serial_fallbacks(obj):
    """Number of group resamplings recomputed serially (diagnostic)."""
    _check_lik(obj)
    n = ctypes.c_int64()
    check(_lib.lib().dust2_gb300_filter_serial_fallbacks(obj.ptr,
                                                         ctypes.byref(n)))
    return n.value


# ---------------------------------------------------------------------------
# Likelihood server (continuous batching of many likelihood objects; no
# counterpart in dust2, whose MCMC caller R/monty.R:90-317 runs one
# dust_likelihood_run per chain and proposal)

SERVER_STATS = ("device_steps", "particle_steps", "requests_done",
                "resident_sessions", "sessions_waiting", "requests_queued",
                "particle_capacity", "particles_in_use", "max_running",
                "step_kernel_ms", "timed_steps", "kernel_launches")


class DustServer:
    """Serves filter likelihoods of many sessions (one per MCMC chain) on
    one device: submit() queues a run at new parameters and returns at
    once; wait() returns its log-likelihood.  A session is a one-group
    likelihood object (dust_filter_create with n_groups = 1); its results
    equal those of that object run on its own."""

    def __init__(self, generator, hbm_budget=8e9, max_sessions=1024):
        gen = _generator(generator)
        if not gen.has_compare or gen.time_type == "continuous":
            raise DustError(f"Can't serve likelihoods of the '{gen.name}' "
                            "system")
        self.generator = gen
        handle = ctypes.c_void_p()
        check(_lib.lib().dust2_gb300_server_create(
            gen.name.encode(), float(hbm_budget), int(max_sessions),
            ctypes.byref(handle)))
        self._handle = handle

    def __del__(self):
        self.free()

    def free(self):
        h = getattr(self, "_handle", None)
        if h is not None and _lib._lib is not None:
            _lib._lib.dust2_gb300_server_free(h)
        self._handle = None

    def capacity(self):
        v = [ctypes.c_size_t() for _ in range(3)]
        check(_lib.lib().dust2_gb300_server_capacity(
            self._handle, *[ctypes.byref(x) for x in v]))
        return {"n_particles": v[0].value, "n_sessions": v[1].value,
                "n_observations": v[2].value}

    def open(self, pars, data, n_particles, time_start=0, dt=None,
             seed=None):
        """A session with the arguments of dust_filter_create (one group)
        and its first parameters; returns its id."""
        gen = self.generator
        n_particles = _scalar_size(n_particles, "n_particles")
        if n_particles > self.capacity()["n_particles"]:
            raise DustError("This session needs more device memory than the "
                            "server's budget")
        d = _prepare_data(data, None, False, gen)
        if d["n_groups"] != 1:
            raise DustError("A session has exactly one group")
        dt = _check_dt(dt, gen)
        flat = as_f64(gen.pack_pars(pars))
        rows = as_f64(d["rows"])
        times = as_f64(d["time"])
        words = np.frombuffer(rng_streams(n_particles + 2, seed),
                              dtype="<u8").astype(np.uint64)
        sid = ctypes.c_int64()
        check(_lib.lib().dust2_gb300_server_open(
            self._handle, dptr(flat), n_particles, float(time_start),
            dptr(times), times.size, dptr(rows), dt, uptr(words),
            words.size, ctypes.byref(sid)))
        return sid.value

    def submit(self, session, pars=None):
        flat = None if pars is None else as_f64(
            self.generator.pack_pars(pars))
        t = ctypes.c_int64()
        check(_lib.lib().dust2_gb300_server_submit(
            self._handle, int(session), dptr(flat), ctypes.byref(t)))
        return t.value

    def wait(self, ticket, timeout=None):
        """(log-likelihood, latency in seconds); None if `timeout` seconds
        pass first."""
        ll = ctypes.c_double()
        lat = ctypes.c_double()
        rc = _lib.lib().dust2_gb300_server_wait(
            self._handle, int(ticket), -1.0 if timeout is None else
            float(timeout), ctypes.byref(ll), ctypes.byref(lat))
        if rc == _lib.PENDING:
            return None
        check(rc)
        return ll.value, lat.value

    def likelihood(self, session, pars=None):
        return self.wait(self.submit(session, pars))[0]

    def close(self, session):
        check(_lib.lib().dust2_gb300_server_close(self._handle,
                                                  int(session)))

    def rng_state(self, session, n_particles):
        out = np.zeros(4 * (n_particles + 2), dtype=np.uint64)
        check(_lib.lib().dust2_gb300_server_rng_state(
            self._handle, int(session), uptr(out)))
        return out.astype("<u8").tobytes()

    def set_timing(self, enable):
        check(_lib.lib().dust2_gb300_server_set_timing(self._handle,
                                                       int(bool(enable))))

    def stats(self):
        out = np.zeros(len(SERVER_STATS))
        check(_lib.lib().dust2_gb300_server_stats(self._handle, dptr(out),
                                                  out.size))
        return dict(zip(SERVER_STATS, out.tolist()))


def dust_likelihood_server(generator, hbm_budget=8e9, max_sessions=1024):
    """A likelihood server for a discrete-time system with compare_data."""
    return DustServer(generator, hbm_budget, max_sessions)
