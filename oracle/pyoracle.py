"""TEST INFRASTRUCTURE (oracle): ctypes access to the CPU oracle.

`port` is the CPU restatement (oracle/port/oracle.cpp, built everywhere);
`ref` is dust2's own engine compiled from the reference sources with the
project's monty stand-in (oracle/ref_driver.cpp, built only where the
reference tree exists).  Both expose the same functions, so tests can
run one against the other and against the CUDA engine.
"""

import ctypes
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
PORT_LIB = HERE / "_build" / "liboracle.so"
REF_LIB = HERE / "_ref" / "libdust2_ref.so"

_d = ctypes.POINTER(ctypes.c_double)
_u = ctypes.POINTER(ctypes.c_uint64)
_i = ctypes.POINTER(ctypes.c_int)
_l = ctypes.POINTER(ctypes.c_int64)
_c = ctypes.c_char_p
_n = ctypes.c_int


class OracleError(RuntimeError):
    pass


def _dp(a):
    return None if a is None else np.ascontiguousarray(
        a, dtype=np.float64).ctypes.data_as(_d)


class Oracle:
    """One oracle library (port or reference build)."""

    def __init__(self, path, kind):
        self.kind = kind
        self.path = Path(path)
        self.lib = ctypes.CDLL(str(path))
        p = "oracle_" if kind == "port" else "ref_"
        self.prefix = p
        lib = self.lib
        self._sim = getattr(lib, p + "discrete_simulate")
        self._cmp = getattr(lib, p + "compare")
        self._flt = getattr(lib, p + "filter_run")
        self._ode = getattr(lib, p + "ode_simulate")
        self._unf = getattr(lib, p + "unfilter_run")
        self._slw = getattr(lib, p + "scale_log_weights")
        self._slw.restype = ctypes.c_double
        self._slw.argtypes = [_n, _d]
        self._rsw = getattr(lib, p + "resample_weight")
        self._rsw.restype = None
        self._rsw.argtypes = [_n, _d, ctypes.c_double, _l]
        if kind == "port":
            lib.oracle_max_threads.restype = ctypes.c_int

    def max_threads(self):
        return self.lib.oracle_max_threads() if self.kind == "port" else 1

    def _call(self, fn, *args):
        err = ctypes.create_string_buffer(4096)
        rc = fn(*args, err, len(err))
        if rc != 0:
            raise OracleError(err.value.decode())

    def discrete_simulate(self, name, pars, n_groups, n_particles, time, dt,
                          rng, times, deterministic=False, initial=None,
                          n_threads=1):
        pars = np.ascontiguousarray(pars, dtype=np.float64)
        times = np.ascontiguousarray(times, dtype=np.float64)
        rng = np.ascontiguousarray(rng, dtype=np.uint64)
        n_total = n_groups * n_particles
        n_state = None
        out = None
        # the state size is not known here; ask with a generous buffer
        buf = np.empty(times.size * n_total * 128)
        rng_out = np.empty(4 * n_total, dtype=np.uint64)
        args = [_c(name.encode()), _dp(pars), _n(n_groups), _n(n_particles),
                ctypes.c_double(time), ctypes.c_double(dt),
                rng.ctypes.data_as(_u), _n(int(deterministic)),
                _dp(initial), _dp(times), _n(times.size), _dp(buf),
                rng_out.ctypes.data_as(_u)]
        if self.kind == "port":
            args.append(_n(n_threads))
        self._call(self._sim, *args)
        n_state = None
        return buf, rng_out

    def filter_run(self, name, pars, n_particles, time_start, times, data,
                   n_groups_data, dt, rng, n_runs=1, initial=None,
                   index_group=None, n_state=None, n_threads=1):
        """n_particles: list per group (port) or equal counts (ref)."""
        pars = np.ascontiguousarray(pars, dtype=np.float64)
        times = np.ascontiguousarray(times, dtype=np.float64)
        data = np.ascontiguousarray(data, dtype=np.float64)
        rng = np.ascontiguousarray(rng, dtype=np.uint64)
        npg = list(n_particles)
        G = len(npg)
        n_total = sum(npg)
        ll = np.full(n_runs * G, np.nan)
        state = np.empty(n_total * (n_state or 128))
        rng_out = np.empty(4 * (n_total + 2 * G), dtype=np.uint64)
        if self.kind == "port":
            npa = np.ascontiguousarray(npg, dtype=np.intc)
            ig = None if index_group is None else np.ascontiguousarray(
                index_group, dtype=np.intc)
            self._call(self._flt, _c(name.encode()), _dp(pars), _n(G),
                       npa.ctypes.data_as(_i), ctypes.c_double(time_start),
                       _dp(times), _n(times.size), _dp(data),
                       _n(n_groups_data), ctypes.c_double(dt),
                       rng.ctypes.data_as(_u), _n(n_runs), _dp(initial),
                       None if ig is None else ig.ctypes.data_as(_i),
                       _n(0 if ig is None else ig.size), _dp(ll), _dp(state),
                       rng_out.ctypes.data_as(_u), _n(n_threads))
        else:
            if len(set(npg)) != 1 or index_group is not None:
                raise OracleError("the reference filter needs equal counts")
            self._call(self._flt, _c(name.encode()), _dp(pars), _n(G),
                       _n(npg[0]), ctypes.c_double(time_start), _dp(times),
                       _n(times.size), _dp(data), _n(n_groups_data),
                       ctypes.c_double(dt), rng.ctypes.data_as(_u),
                       _n(n_runs), _dp(initial), _dp(ll), _dp(state),
                       rng_out.ctypes.data_as(_u))
        return ll.reshape(n_runs, G), state, rng_out

    def compare(self, name, pars, n_groups, n_particles, time, state, data,
                n_groups_data, rng):
        pars = np.ascontiguousarray(pars, dtype=np.float64)
        state = np.ascontiguousarray(state, dtype=np.float64)
        data = np.ascontiguousarray(data, dtype=np.float64)
        rng = np.ascontiguousarray(rng, dtype=np.uint64)
        n_total = n_groups * n_particles
        out = np.empty(n_total)
        rng_out = np.empty(4 * n_total, dtype=np.uint64)
        self._call(self._cmp, _c(name.encode()), _dp(pars), _n(n_groups),
                   _n(n_particles), ctypes.c_double(time), _dp(state),
                   _dp(data), _n(n_groups_data), rng.ctypes.data_as(_u),
                   _dp(out), rng_out.ctypes.data_as(_u))
        return out, rng_out

    def ode_simulate(self, name, pars, n_groups, n_particles, time, times,
                     n_state, max_steps=10000, atol=1e-6, rtol=1e-6,
                     step_size_min=np.finfo(float).eps,
                     step_size_max=np.inf, critical_times=(), n_threads=1):
        pars = np.ascontiguousarray(pars, dtype=np.float64)
        times = np.ascontiguousarray(times, dtype=np.float64)
        crit = np.ascontiguousarray(critical_times, dtype=np.float64)
        n_total = n_groups * n_particles
        out = np.empty(times.size * n_total * n_state)
        stats = np.empty(3 * n_total, dtype=np.int64)
        args = [_c(name.encode()), _dp(pars), _n(n_groups), _n(n_particles),
                ctypes.c_double(time), _n(max_steps), ctypes.c_double(atol),
                ctypes.c_double(rtol), ctypes.c_double(step_size_min),
                ctypes.c_double(step_size_max),
                crit.ctypes.data_as(_d) if crit.size else None,
                _n(crit.size), _dp(times), _n(times.size), _dp(out),
                stats.ctypes.data_as(_l)]
        if self.kind == "port":
            args.append(_n(n_threads))
        self._call(self._ode, *args)
        return out, stats.reshape(n_total, 3)

    def unfilter_run(self, name, pars, n_groups, n_particles, time_start,
                     times, data, n_groups_data, n_state, dt=1.0,
                     max_steps=10000, atol=1e-6, rtol=1e-6,
                     step_size_min=np.finfo(float).eps,
                     step_size_max=np.inf, n_runs=1, n_threads=1):
        """Deterministic likelihood runs (dust2::unfilter); returns
        (ll [n_runs][group][particle], state after the last run)."""
        pars = np.ascontiguousarray(pars, dtype=np.float64)
        times = np.ascontiguousarray(times, dtype=np.float64)
        data = np.ascontiguousarray(data, dtype=np.float64)
        n_total = n_groups * n_particles
        ll = np.empty(n_runs * n_total)
        state = np.empty(n_total * n_state)
        args = [_c(name.encode()), _dp(pars), _n(n_groups), _n(n_particles),
                ctypes.c_double(time_start), _dp(times), _n(times.size),
                _dp(data), _n(n_groups_data), ctypes.c_double(dt),
                _n(max_steps), ctypes.c_double(atol), ctypes.c_double(rtol),
                ctypes.c_double(step_size_min),
                ctypes.c_double(step_size_max), _n(n_runs), _dp(ll),
                _dp(state)]
        if self.kind == "port":
            args.append(_n(n_threads))
        self._call(self._unf, *args)
        return ll.reshape(n_runs, n_groups, n_particles), state

    def mixed_simulate(self, name, pars, n_groups, n_particles, time, dt,
                       rng, times, n_state, max_steps=10000, atol=1e-6,
                       rtol=1e-6, step_size_min=np.finfo(float).eps,
                       step_size_max=np.inf):
        """A mixed-time system (dust_continuous with updates every dt)
        from its initial conditions through `times`; rng: 4 words per
        particle.  Returns (state [time][group][particle][state], solver
        counts [particle][3])."""
        pars = np.ascontiguousarray(pars, dtype=np.float64)
        times = np.ascontiguousarray(times, dtype=np.float64)
        rng = np.ascontiguousarray(rng, dtype=np.uint64)
        n_total = n_groups * n_particles
        out = np.empty(times.size * n_total * n_state)
        stats = np.empty(3 * n_total, dtype=np.int64)
        self._call(getattr(self.lib, self.prefix + "mixed_simulate"),
                   _c(name.encode()), _dp(pars), _n(n_groups),
                   _n(n_particles), ctypes.c_double(time),
                   ctypes.c_double(dt), _n(max_steps), ctypes.c_double(atol),
                   ctypes.c_double(rtol), ctypes.c_double(step_size_min),
                   ctypes.c_double(step_size_max), rng.ctypes.data_as(_u),
                   _dp(times), _n(times.size), _dp(out),
                   stats.ctypes.data_as(_l))
        return (out.reshape(times.size, n_groups, n_particles, n_state),
                stats.reshape(n_total, 3))

    def mixed_filter_run(self, name, pars, n_groups, n_particles,
                         time_start, times, data, n_groups_data, dt, rng,
                         n_state, n_runs=1, max_steps=10000, atol=1e-6,
                         rtol=1e-6, step_size_min=np.finfo(float).eps,
                         step_size_max=np.inf):
        """Particle filter runs over a mixed-time system; returns (ll
        [n_runs][group], final state [group][particle][state], raw
        generator state)."""
        pars = np.ascontiguousarray(pars, dtype=np.float64)
        times = np.ascontiguousarray(times, dtype=np.float64)
        data = np.ascontiguousarray(data, dtype=np.float64)
        rng = np.ascontiguousarray(rng, dtype=np.uint64)
        ll = np.empty(n_runs * n_groups)
        state = np.empty(n_groups * n_particles * n_state)
        rng_out = np.empty(rng.size, dtype=np.uint64)
        self._call(getattr(self.lib, self.prefix + "mixed_filter_run"),
                   _c(name.encode()), _dp(pars), _n(n_groups),
                   _n(n_particles), ctypes.c_double(time_start), _dp(times),
                   _n(times.size), _dp(data), _n(n_groups_data),
                   ctypes.c_double(dt), _n(max_steps), ctypes.c_double(atol),
                   ctypes.c_double(rtol), ctypes.c_double(step_size_min),
                   ctypes.c_double(step_size_max), rng.ctypes.data_as(_u),
                   _n(n_runs), _dp(ll), _dp(state),
                   rng_out.ctypes.data_as(_u))
        return (ll.reshape(n_runs, n_groups),
                state.reshape(n_groups, n_particles, n_state), rng_out)

    def unfilter_states(self, name, pars, n_groups, n_particles, time_start,
                        times, data, n_groups_data, n_state, dt=1.0,
                        max_steps=10000, atol=1e-6, rtol=1e-6,
                        step_size_min=np.finfo(float).eps,
                        step_size_max=np.inf):
        """(port) One deterministic likelihood run returning (ll [group]
        [particle], the full state at every data time [time][group]
        [particle][state])."""
        pars = np.ascontiguousarray(pars, dtype=np.float64)
        times = np.ascontiguousarray(times, dtype=np.float64)
        data = np.ascontiguousarray(data, dtype=np.float64)
        n_total = n_groups * n_particles
        ll = np.empty(n_total)
        states = np.empty(times.size * n_total * n_state)
        self._call(self.lib.oracle_unfilter_states, _c(name.encode()),
                   _dp(pars), _n(n_groups), _n(n_particles),
                   ctypes.c_double(time_start), _dp(times), _n(times.size),
                   _dp(data), _n(n_groups_data), ctypes.c_double(dt),
                   _n(max_steps), ctypes.c_double(atol),
                   ctypes.c_double(rtol), ctypes.c_double(step_size_min),
                   ctypes.c_double(step_size_max), _dp(ll), _dp(states))
        return (ll.reshape(n_groups, n_particles),
                states.reshape(times.size, n_groups, n_particles, n_state))

    def unfilter_trajectories(self, name, pars, n_groups, n_particles,
                              time_start, times, data, n_groups_data, dt,
                              n_state, index_state=None, snapshots=None,
                              adjoint=False):
        """(reference) One unfilter run (run_adjoint when `adjoint`)
        saving trajectories of index_state (None = all) and snapshots at
        the data times `snapshots`; returns (ll [group][particle],
        trajectories [time][group][particle][entry], snapshots
        [snapshot][group][particle][state])."""
        pars = np.ascontiguousarray(pars, dtype=np.float64)
        times = np.ascontiguousarray(times, dtype=np.float64)
        data = np.ascontiguousarray(data, dtype=np.float64)
        ist = (np.zeros(0, dtype=np.int32) if index_state is None else
               np.ascontiguousarray(index_state, dtype=np.int32))
        n_save = n_state if index_state is None else ist.size
        snaps = (np.zeros(0) if snapshots is None else
                 np.ascontiguousarray(snapshots, dtype=np.float64))
        n_total = n_groups * n_particles
        ll = np.empty(n_total)
        traj = np.empty(times.size * n_total * n_save)
        snap = np.empty(max(1, snaps.size * n_total * n_state))
        ip = ctypes.POINTER(ctypes.c_int)
        self._call(self.lib.ref_unfilter_trajectories, _c(name.encode()),
                   _dp(pars), _n(n_groups), _n(n_particles),
                   ctypes.c_double(time_start), _dp(times), _n(times.size),
                   _dp(data), _n(n_groups_data), ctypes.c_double(dt),
                   ist.ctypes.data_as(ip), _n(ist.size), _dp(snaps),
                   _n(snaps.size), _n(1 if adjoint else 0), _dp(ll),
                   _dp(traj), _dp(snap))
        return (ll.reshape(n_groups, n_particles),
                traj.reshape(times.size, n_groups, n_particles, n_save),
                snap[:snaps.size * n_total * n_state].reshape(
                    snaps.size, n_groups, n_particles, n_state))

    def unfilter_adjoint(self, name, pars, n_groups, n_particles,
                         time_start, times, data, n_groups_data, n_state,
                         dt=1.0, n_gradient=3):
        """One adjoint run of a deterministic likelihood and its gradient
        (unfilter::run_adjoint + last_gradient); returns (ll [group]
        [particle], gradient [group][particle][n_gradient], state).  The
        reference build takes one particle per group."""
        if self.kind == "ref" and n_particles != 1:
            raise OracleError("the reference computes gradients for one "
                              "particle per group")
        pars = np.ascontiguousarray(pars, dtype=np.float64)
        times = np.ascontiguousarray(times, dtype=np.float64)
        data = np.ascontiguousarray(data, dtype=np.float64)
        n_total = n_groups * n_particles
        ll = np.empty(n_total)
        gr = np.empty(n_total * n_gradient)
        state = np.empty(n_total * n_state)
        fn = getattr(self.lib, self.prefix + "unfilter_adjoint")
        args = [_c(name.encode()), _dp(pars), _n(n_groups)]
        if self.kind == "port":
            args.append(_n(n_particles))
        args += [ctypes.c_double(time_start), _dp(times), _n(times.size),
                 _dp(data), _n(n_groups_data), ctypes.c_double(dt), _dp(ll),
                 _dp(gr), _dp(state)]
        self._call(fn, *args)
        return (ll.reshape(n_groups, n_particles),
                gr.reshape(n_groups, n_particles, n_gradient), state)

    def filter_trajectories(self, name, pars, n_groups, n_particles,
                            time_start, times, data, n_groups_data, dt, rng,
                            n_state_saved, index_state=None, select=None,
                            select_random=False, snapshots=None, n_state=5,
                            n_threads=1):
        """One filter run saving trajectories (and snapshots at the data
        times `snapshots`), exported with reordering: (ll [group],
        trajectories [time][group][particle][state], select, snapshots
        [snapshot][group][particle][state]).  The port takes `select`
        (particle per group); the reference draws it (select_random) and
        returns it."""
        pars = np.ascontiguousarray(pars, dtype=np.float64)
        times = np.ascontiguousarray(times, dtype=np.float64)
        data = np.ascontiguousarray(data, dtype=np.float64)
        rng = np.ascontiguousarray(rng, dtype=np.uint64)
        ist = (np.zeros(0, dtype=np.int32) if index_state is None else
               np.ascontiguousarray(index_state, dtype=np.int32))
        n_out = 1 if (select is not None or select_random) else n_particles
        ll = np.empty(n_groups)
        out = np.empty(times.size * n_groups * n_out * n_state_saved)
        ip = ctypes.POINTER(ctypes.c_int)
        snaps = (np.zeros(0) if snapshots is None else
                 np.ascontiguousarray(snapshots, dtype=np.float64))
        snap_obs = np.ascontiguousarray(np.searchsorted(times, snaps),
                                        dtype=np.int32)
        snap_out = np.empty(max(1, snaps.size * n_groups * n_out * n_state))
        if self.kind == "port":
            sel = (None if select is None else
                   np.ascontiguousarray(select, dtype=np.int32))
            self._call(self.lib.oracle_filter_trajectories,
                       _c(name.encode()), _dp(pars), _n(n_groups),
                       _n(n_particles), ctypes.c_double(time_start),
                       _dp(times), _n(times.size), _dp(data),
                       _n(n_groups_data), ctypes.c_double(dt),
                       rng.ctypes.data_as(ctypes.POINTER(ctypes.c_uint64)),
                       ist.ctypes.data_as(ip), _n(ist.size),
                       snap_obs.ctypes.data_as(ip), _n(snap_obs.size),
                       None if sel is None else sel.ctypes.data_as(ip),
                       _dp(ll), _dp(out), _dp(snap_out), _n(n_threads))
            return ll, out, sel, snap_out[:snaps.size * n_groups * n_out *
                                          n_state]
        sel = np.zeros(n_groups, dtype=np.int32)
        self._call(self.lib.ref_filter_trajectories,
                   _c(name.encode()), _dp(pars), _n(n_groups),
                   _n(n_particles), ctypes.c_double(time_start), _dp(times),
                   _n(times.size), _dp(data), _n(n_groups_data),
                   ctypes.c_double(dt),
                   rng.ctypes.data_as(ctypes.POINTER(ctypes.c_uint64)),
                   ist.ctypes.data_as(ip), _n(ist.size), _dp(snaps),
                   _n(snaps.size), _n(1 if select_random else 0), _dp(ll),
                   _dp(out), _dp(snap_out), sel.ctypes.data_as(ip))
        return (ll, out, (sel if select_random else None),
                snap_out[:snaps.size * n_groups * n_out * n_state])

    def scale_log_weights(self, w):
        w = np.array(w, dtype=np.float64)
        ret = self._slw(w.size, w.ctypes.data_as(_d))
        return ret, w

    def resample_weight(self, w, u):
        w = np.ascontiguousarray(w, dtype=np.float64)
        idx = np.empty(w.size, dtype=np.int64)
        self._rsw(w.size, w.ctypes.data_as(_d), float(u),
                  idx.ctypes.data_as(_l))
        return idx


_port = None
_ref = None


def port():
    """The CPU restatement (builds it if needed)."""
    global _port
    if _port is None:
        from . import build
        build.build_port()
        _port = Oracle(PORT_LIB, "port")
    return _port


_port_timing = None


def port_timing():
    """The timing build of the restatement (host libm exp and log, as
    dust2 evaluates them): for timing the CPU path only."""
    global _port_timing
    if _port_timing is None:
        from . import build
        _port_timing = Oracle(build.build_port(libm=True), "port")
    return _port_timing


def ref():
    """dust2's own engine, or None where the reference build is absent."""
    global _ref
    if _ref is None:
        if not REF_LIB.exists():
            from . import build
            if build.build_ref() is None:
                return None
        _ref = Oracle(REF_LIB, "ref")
    return _ref


def port_math(fn, x):
    """The project's exp/log/lgamma/cos2pi/sin2pi/rcp evaluated on the
    host."""
    o = port()
    x = np.ascontiguousarray(x, dtype=np.float64)
    out = np.empty_like(x)
    f = o.lib.oracle_math
    f.restype = None
    code = {"exp": 0, "log": 1, "lgamma": 2, "cos2pi": 3, "sin2pi": 4,
            "rcp": 5}[fn]
    f(ctypes.c_int(code), x.ctypes.data_as(_d), ctypes.c_int(x.size),
      out.ctypes.data_as(_d))
    return out


def port_draws(dist, a, b, n, rng):
    """n draws of a sampler from one stream; returns (draws, error code)."""
    o = port()
    rng = np.ascontiguousarray(rng, dtype=np.uint64)
    out = np.empty(n)
    f = o.lib.oracle_draws
    f.restype = ctypes.c_int
    code = {"binomial": 0, "poisson": 1, "normal": 2, "exponential": 3,
            "uniform": 4, "real": 5}[dist]
    err = f(ctypes.c_int(code), ctypes.c_double(a), ctypes.c_double(b),
            ctypes.c_int(n), rng.ctypes.data_as(_u), out.ctypes.data_as(_d))
    return out, err


def port_density(dist, x, a, b=0.0):
    o = port()
    x = np.ascontiguousarray(x, dtype=np.float64)
    out = np.empty_like(x)
    f = o.lib.oracle_density
    f.restype = None
    code = {"poisson": 0, "negbin": 1, "normal": 2}[dist]
    f(ctypes.c_int(code), x.ctypes.data_as(_d), ctypes.c_int(x.size),
      ctypes.c_double(a), ctypes.c_double(b), out.ctypes.data_as(_d))
    return out


def rng_streams(n_streams, seed):
    """Words (uint64) of the first n_streams streams of an integer seed,
    computed by the oracle (no CUDA library involved)."""
    o = port()
    out = np.empty(4 * n_streams, dtype=np.uint64)
    f = o.lib.oracle_rng_streams
    f.restype = None
    f(ctypes.c_uint64(int(seed) % (1 << 64)), ctypes.c_int(n_streams),
      out.ctypes.data_as(_u))
    return out


def pack_pars(name, pars):
    """A flat parameter row (NaN where not given) of a discrete-time
    system from a dict, laid out by the system's parameter table as the
    oracle reads it (no CUDA library involved)."""
    o = port()
    buf = ctypes.create_string_buffer(1 << 14)
    f = o.lib.oracle_parameters
    f.restype = ctypes.c_int
    if f(name.encode(), buf, len(buf)) < 0:
        raise OracleError(f"unknown system {name}")
    table = [(ln.split()[0], int(ln.split()[1]))
             for ln in buf.value.decode().splitlines()]
    row = np.full(sum(n for _, n in table), np.nan)
    off = 0
    for nm, n in table:
        if nm in pars and pars[nm] is not None:
            v = np.asarray(pars[nm], dtype=np.float64).ravel()
            row[off:off + v.size] = v
        off += n
    return row
