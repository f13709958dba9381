"""Generate the golden fixtures in tests/golden/ from dust2's own engine.

The reference engine (inst/include/dust2 compiled unmodified with the
project's monty stand-in, oracle/ref_driver.cpp) is run on seeded
synthetic inputs and its outputs are saved as .npz files.  The GPU tests
compare the CUDA engine against these files on machines where the
reference sources are absent.  Streams are generated by the independent
numpy implementation in tests/xoshiro.py, so the fixtures do not depend
on the engine under test.

Run from the repository root:  python tests/golden/make_golden.py
(`--unfilter` / `--trajectories` / `--adjoint` /
`--unfilter-trajectories` / `--mixed` write only those fixtures).
"""

import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))
sys.path.insert(0, str(ROOT / "tests"))

from oracle import pyoracle  # noqa: E402
import xoshiro  # noqa: E402
import workload_data  # noqa: E402
from dust2_gb300 import workloads  # noqa: E402

OUT = Path(__file__).resolve().parent


def save(name, **kw):
    np.savez_compressed(OUT / f"{name}.npz", **kw)
    print("wrote", name)


def main():
    ref = pyoracle.ref()
    if ref is None:
        raise SystemExit("the reference sources are needed to make fixtures")

    # 1. The filter of tests/testthat/test-filter.R "can run particle
    #    filter": sir, 100 particles, data at 4,8,12,16, dt = 1, 20 runs;
    #    here with 2 groups (test-filter.R "nested particle filter").
    pars = workload_data.sir_pars([
        {"beta": 0.1, "gamma": 0.2, "N": 1000, "I0": 10, "exp_noise": 1e6},
        {"beta": 0.2, "gamma": 0.2, "N": 1000, "I0": 10, "exp_noise": 1e6}])
    n = 100
    rng = xoshiro.streams(42, 2 * (n + 2))
    times = np.array([4.0, 8, 12, 16])
    data = np.array([1.0, 2, 2, 3, 3, 4, 4, 5])
    ll, state, rng_out = ref.filter_run("sir", pars, [n, n], 0.0, times, data,
                                        2, 1.0, rng, n_runs=20, n_state=5)
    save("filter_sir_2groups", pars=pars, n_particles=n, rng=rng,
         times=times, data=data, dt=1.0, ll=ll, state=state[:2 * n * 5],
         rng_out=rng_out)

    # 2. Missing data in one group only (test-filter.R:470-515).
    data_na = np.array([1.0, 2, 2, np.nan, np.nan, 4, np.nan, np.nan, 5, 6])
    times5 = np.array([4.0, 8, 12, 16, 20])
    ll, state, rng_out = ref.filter_run("sir", pars, [n, n], 0.0, times5,
                                        data_na, 2, 1.0, rng, n_runs=5,
                                        n_state=5)
    save("filter_sir_missing", pars=pars, n_particles=n, rng=rng,
         times=times5, data=data_na, dt=1.0, ll=ll, state=state[:2 * n * 5],
         rng_out=rng_out)

    # 3. The single-group SIR filter workload: 1000 particles, 100 daily
    #    observations, dt = 0.25, data from the model at seed 42 plus
    #    Poisson noise.
    w = workload_data.sir_small(ref)
    rng = xoshiro.streams(w["seed"], w["n_particles"] + 2)
    ll, state, rng_out = ref.filter_run(
        "sir_cases", w["pars"], [w["n_particles"]], 0.0, w["times"],
        w["data"], 1, w["dt"], rng, n_runs=3, n_state=4)
    save("filter_sir_cases_1000", pars=w["pars"],
         n_particles=w["n_particles"], rng=rng, times=w["times"],
         data=w["data"], dt=w["dt"], ll=ll,
         state=state[:w["n_particles"] * 4], rng_out=rng_out)

    # 4. Plain stepping (dust_system_run_to_time / simulate) of each
    #    discrete system, 3 groups x 7 particles.
    for name, plist, dt, tmax in [
            ("sir", [{"beta": 0.3, "gamma": 0.1, "N": 1000, "I0": 10,
                      "exp_noise": 1e6}] * 3, 0.25, 30),
            ("walk", [{"sd": 1.0, "len": 3, "random_initial": 1},
                      {"sd": 2.0, "len": 3, "random_initial": 1},
                      {"sd": 3.0, "len": 3, "random_initial": 1}], 0.5, 10),
            ("seir_age", workloads.seir_plist([1.5, 2.0, 2.5]), 0.25, 20)]:
        flat = workload_data.pack(name, plist)
        G, np_ = 3, 7
        rng = xoshiro.streams(7, G * np_)
        tt = np.arange(0, tmax + 1, dtype=float)
        sim, rng_out = ref.discrete_simulate(name, flat, G, np_, 0.0, dt, rng,
                                             tt)
        n_state = {"sir": 5, "walk": 3, "seir_age": 96}[name]
        save(f"simulate_{name}", pars=flat, n_groups=G, n_particles=np_,
             rng=rng, dt=dt, times=tt,
             out=sim[:tt.size * G * np_ * n_state], rng_out=rng_out)

    # 5. compare_data of sir with exponential noise (test-sir.R:31-46).
    flat = workload_data.pack("sir", [{"exp_noise": 0.5}])
    rs = np.random.default_rng(3)
    st = np.zeros((10, 5))
    st[:, 4] = rs.poisson(30, 10)
    rng = xoshiro.streams(42, 10)
    out, rng_out = ref.compare("sir", flat, 1, 10, 0.0, st.ravel(),
                               np.array([30.0]), 1, rng)
    save("compare_sir", pars=flat, state=st.ravel(), rng=rng, out=out,
         rng_out=rng_out)

    # 6. dopri5: sirode and logistic.
    flat = workload_data.pack("sirode", [
        {"beta": 0.2, "gamma": 0.1, "N": 1000, "I0": 10},
        {"beta": 0.4, "gamma": 0.05, "N": 1e6, "I0": 50}])
    tt = np.arange(0, 201, dtype=float)
    out, stats = ref.ode_simulate("sirode", flat, 2, 2, 0.0, tt, 5)
    save("ode_sirode", pars=flat, times=tt, out=out, stats=stats)
    flat = workload_data.pack("logistic", [
        {"n": 3, "r": [0.1, 0.2, 0.3], "K": [100, 100, 100]}])
    tt = np.arange(0, 51, dtype=float)
    out, stats = ref.ode_simulate("logistic", flat, 1, 1, 0.0, tt, 4)
    save("ode_logistic", pars=flat, times=tt, out=out, stats=stats)
    out, stats = ref.ode_simulate("sirode", workload_data.pack(
        "sirode", [{"beta": 0.2, "gamma": 0.1, "N": 1000, "I0": 10}]),
        1, 1, 0.0, np.array([0.0, 50.0]), 5, critical_times=[10, 20, 30])
    save("ode_sirode_critical", out=out, stats=stats)

    # 7. Systematic resampling and log-weight scaling helpers
    #    (test-filter-details.R:1-64).
    rs = np.random.default_rng(1)
    w = np.abs(rs.standard_cauchy(20))
    u = rs.uniform()
    cases = {"w": w, "u": np.array([u, 0.0, 1 - 1e-8])}
    cases["idx"] = np.stack([ref.resample_weight(w, uu) for uu in cases["u"]])
    lw = np.log(rs.uniform(size=50)) * 10
    lw[[3, 17]] = np.nan
    r1, w1 = ref.scale_log_weights(lw)
    r2, w2 = ref.scale_log_weights(np.full(5, -np.inf))
    r3, w3 = ref.scale_log_weights(np.array([-3.5]))
    save("filter_details", **cases, lw=lw, lw_ret=np.array([r1, r2, r3]),
         lw_w1=w1, lw_w2=w2, lw_w3=w3)
    unfilters(ref)
    trajectories(ref)
    adjoints(ref)
    unfilter_trajectories(ref)
    mixed(ref)


def unfilters(ref):
    """8. Deterministic likelihoods (dust2::unfilter, test-unfilter.R):
    a discrete SIR of 2 groups x 3 particles (dt = 0.25) and the sirode
    ODE of 2 groups x 2 particles, data every 4 days with one missing
    value, 2 runs each."""
    times = np.arange(4, 41, 4, dtype=float)
    rs = np.random.default_rng(8)
    data = rs.poisson(8, 2 * times.size).astype(float)
    data[5] = np.nan
    pars = workload_data.sir_pars([
        {"beta": 0.2, "gamma": 0.1, "N": 1000, "I0": 10},
        {"beta": 0.3, "gamma": 0.15, "N": 2000, "I0": 5}])
    ll, state = ref.unfilter_run("sir", pars, 2, 3, 0.0, times, data, 2, 5,
                                 dt=0.25, n_runs=2)
    save("unfilter_sir", pars=pars, times=times, data=data, ll=ll,
         state=state)
    pars = workload_data.pack("sirode", [
        {"beta": 0.2, "gamma": 0.1, "N": 1000, "I0": 10},
        {"beta": 0.3, "gamma": 0.15, "N": 2000, "I0": 5}])
    ll, state = ref.unfilter_run("sirode", pars, 2, 2, 0.0, times, data, 2,
                                 5, n_runs=2)
    save("unfilter_sirode", pars=pars, times=times, data=data, ll=ll,
         state=state)


def trajectories(ref):
    """9. Filter trajectories and snapshots with reordering (test-filter.R
    "can save trajectories from filter", "can save snapshots"): sir, 2
    groups x 50 particles, all state, state entries 2 and 4 (0-based 1 and
    3), one random particle per group, snapshots at times 8 and 16."""
    pars = workload_data.sir_pars([
        {"beta": 0.1, "gamma": 0.2, "N": 1000, "I0": 10, "exp_noise": 1e6},
        {"beta": 0.2, "gamma": 0.2, "N": 1000, "I0": 10, "exp_noise": 1e6}])
    n = 50
    rng = xoshiro.streams(7, 2 * (n + 2))
    times = np.array([4.0, 8, 12, 16, 20])
    data = np.array([1.0, 2, 2, 3, 3, 4, 4, 5, 6, 6])
    snapshots = np.array([8.0, 16.0])
    ll, full, _, snap = ref.filter_trajectories(
        "sir", pars, 2, n, 0.0, times, data, 2, 1.0, rng, 5,
        snapshots=snapshots)
    _, sub, _, _ = ref.filter_trajectories(
        "sir", pars, 2, n, 0.0, times, data, 2, 1.0, rng, 2,
        index_state=[1, 3])
    _, one, sel, snap_one = ref.filter_trajectories(
        "sir", pars, 2, n, 0.0, times, data, 2, 1.0, rng, 5,
        select_random=True, snapshots=snapshots)
    save("trajectories_sir", pars=pars, n_particles=n, rng=rng, times=times,
         data=data, ll=ll, full=full, sub=sub, one=one, select=sel,
         snapshots=snapshots, snap=snap, snap_one=snap_one)


ADJOINT_CASES = [
    # (label, groups' parameters, time_start, times, dt, n_groups_data)
    ("four_days", [{}], 0.0, [4.0, 8, 12, 16], 1.0, 1),
    ("odd_steps", [{}], 0.0, [3.0, 6, 9, 12], 1.0, 1),
    ("four_groups", [{"beta": 0.1 * (i + 1)} for i in range(4)], 0.0,
     [4.0, 8, 12, 16], 1.0, 4),
    ("quarter_days", [{"beta": 0.3, "gamma": 0.1}], 0.0,
     [float(t) for t in range(1, 21)], 0.25, 1),
    ("late_start", [{"beta": 0.25}, {"beta": 0.15, "I0": 30}], 2.0,
     [5.0, 9, 10, 15], 0.5, 1),
]


def adjoints(ref):
    """10. Gradients of deterministic likelihoods (unfilter::run_adjoint +
    last_gradient, test-unfilter-adjoint.R): the sir system, one particle
    per group (the reference copies gradients for one particle only),
    beta/gamma/N/I0/exp_noise = 0.1/0.2/1000/10/1e6 unless a case
    changes them; incidence 1, 2, ... per group and time."""
    out = {}
    for label, groups, t0, times, dt, ngd in ADJOINT_CASES:
        base = {"beta": 0.1, "gamma": 0.2, "N": 1000, "I0": 10,
                "exp_noise": 1e6}
        pars = workload_data.sir_pars([dict(base, **g) for g in groups])
        times = np.array(times)
        data = np.arange(1, times.size * ngd + 1, dtype=float)
        ll, gr, state = ref.unfilter_adjoint("sir", pars, len(groups), 1,
                                             t0, times, data, ngd, 5, dt=dt)
        for k, v in [("pars", pars), ("times", times), ("data", data),
                     ("ll", ll), ("gradient", gr), ("state", state),
                     ("meta", np.array([len(groups), t0, dt, ngd]))]:
            out[f"{label}__{k}"] = v
    save("adjoint_sir", labels=np.array([c[0] for c in ADJOINT_CASES]),
         **out)


def unfilter_trajectories(ref):
    """11. Deterministic likelihood trajectories and snapshots
    (unfilter.hpp:42-110 trajectories_.add, r/unfilter.hpp:64-125,
    test-unfilter.R / test-unfilter-adjoint.R "can save trajectories"):
    the unfilter_sir inputs (2 groups x 3 particles, dt = 0.25) with all
    state and entries 1, 3 (0-based), snapshots at times 8 and 20, through
    run and run_adjoint; the sirode inputs (2 x 2) with a snapshot at
    12."""
    g = np.load(OUT / "unfilter_sir.npz")
    times, data, pars = g["times"], g["data"], g["pars"]
    snaps = np.array([8.0, 20.0])
    ll, full, snap = ref.unfilter_trajectories(
        "sir", pars, 2, 3, 0.0, times, data, 2, 0.25, 5, snapshots=snaps)
    _, sub, _ = ref.unfilter_trajectories(
        "sir", pars, 2, 3, 0.0, times, data, 2, 0.25, 5, index_state=[1, 3])
    ll_a, full_a, snap_a = ref.unfilter_trajectories(
        "sir", pars, 2, 3, 0.0, times, data, 2, 0.25, 5, snapshots=snaps,
        adjoint=True)
    g = np.load(OUT / "unfilter_sirode.npz")
    ode_snaps = np.array([12.0])
    ll_o, full_o, snap_o = ref.unfilter_trajectories(
        "sirode", g["pars"], 2, 2, 0.0, g["times"], g["data"], 2, 0.0, 5,
        snapshots=ode_snaps)
    save("unfilter_trajectories", snapshots=snaps, ll=ll, full=full,
         snap=snap, sub=sub, ll_adjoint=ll_a, full_adjoint=full_a,
         snap_adjoint=snap_a, ode_snapshots=ode_snaps, ll_ode=ll_o,
         full_ode=full_o, snap_ode=snap_o)


MIXED_SIMULATE_CASES = [
    # (label, dt, output times)
    ("ode_only", 0.0, [float(t) for t in range(21)]),
    ("daily", 1.0, [float(t) for t in range(21)]),
    ("coarse", 1.0, [4.0, 8.0, 12.0, 16.0]),
    ("uneven", 2.0, [3.0, 5.0, 9.0, 10.0, 16.0]),
]


def mixed(ref):
    """12. Mixed-time systems (continuous/system.hpp:80-106, 544-585,
    test-malaria.R, test-filter.R "can run filter on mixed time models"):
    the malaria system, 2 groups (a = 1/3 and 0.4) x 4 particles from
    seeded streams, through each case of MIXED_SIMULATE_CASES; filters of
    1 group x 100 particles (the reference test's data, dt = 1, 5 runs)
    and 3 groups x 40 particles (per-group data, dt = 0.5, 3 runs); an
    unfilter of 2 groups at dt = 1."""
    pars = workload_data.pack("malaria", [{}, {"a": 0.4}])
    rng = xoshiro.streams(13, 8)
    out = {"sim_pars": pars, "sim_rng": rng}
    for label, dt, times in MIXED_SIMULATE_CASES:
        y, stats = ref.mixed_simulate("malaria", pars, 2, 4, 0.0, dt, rng,
                                      np.array(times), 20)
        out[f"sim_{label}"] = y
        out[f"sim_{label}_stats"] = stats
    times = np.array([4.0, 8, 12, 16])
    data = np.array([[2.0, 1], [4, 2], [6, 3], [8, 3]])
    p1 = workload_data.pack("malaria", [{}])
    rng1 = xoshiro.streams(42, 102)
    ll, state, rng_out = ref.mixed_filter_run(
        "malaria", p1, 1, 100, 0.0, times, data.ravel(), 1, 1.0, rng1, 20,
        n_runs=5)
    out.update(f1_pars=p1, f1_times=times, f1_data=data, f1_rng=rng1,
               f1_ll=ll, f1_state=state, f1_rng_out=rng_out)
    p3 = workload_data.pack("malaria", [{"a": 0.3}, {"a": 0.35},
                                        {"r": 0.02}])
    rs = np.random.default_rng(12)
    times3 = np.arange(2.0, 31.0, 2.0)
    tested = rs.integers(5, 30, (times3.size, 3)).astype(float)
    positive = np.floor(tested * rs.uniform(0.6, 0.95, tested.shape))
    data3 = np.stack([tested, positive], axis=-1)
    rng3 = xoshiro.streams(5, 3 * 42)
    ll3, state3, rng3_out = ref.mixed_filter_run(
        "malaria", p3, 3, 40, 0.0, times3, data3.ravel(), 3, 0.5, rng3, 20,
        n_runs=3)
    out.update(f3_pars=p3, f3_times=times3, f3_data=data3, f3_rng=rng3,
               f3_ll=ll3, f3_state=state3, f3_rng_out=rng3_out)
    ll_u, state_u = ref.unfilter_run("malaria", pars, 2, 1, 0.0, times,
                                     np.repeat(data[:, None, :], 2,
                                               axis=1).ravel(), 2, 20,
                                     dt=1.0, n_runs=1)
    out.update(u_times=times, u_data=data, u_ll=ll_u, u_state=state_u)
    save("mixed_malaria", **out)


if __name__ == "__main__":
    if sys.argv[1:] == ["--mixed"]:
        mixed(pyoracle.ref())
    elif sys.argv[1:] == ["--adjoint"]:
        adjoints(pyoracle.ref())
    elif sys.argv[1:] == ["--unfilter-trajectories"]:
        unfilter_trajectories(pyoracle.ref())
    elif sys.argv[1:] == ["--unfilter"]:
        unfilters(pyoracle.ref())
    elif sys.argv[1:] == ["--trajectories"]:
        trajectories(pyoracle.ref())
    else:
        main()
