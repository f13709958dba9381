"""Particle filter on the GPU against dust2's own engine (golden fixtures)
and the CPU oracle (tests/testthat/test-filter.R is the model).

Tolerances: resampling indices, particle state and generator state are
compared exactly; log-likelihoods to 1e-12 relative (the parallel sum of
weights rounds differently from the serial one, by < n ulp)."""

import numpy as np
import pytest

import dust2_gb300 as d
import xoshiro
from conftest import golden

pytestmark = pytest.mark.gpu

RTOL_LL = 1e-12


def assert_ll(a, b):
    a = np.asarray(a, dtype=float)
    b = np.asarray(b, dtype=float)
    assert a.shape == b.shape
    np.testing.assert_array_equal(np.isfinite(a), np.isfinite(b))
    fin = np.isfinite(a)
    np.testing.assert_allclose(a[fin], b[fin], rtol=RTOL_LL, atol=0)
    np.testing.assert_array_equal(a[~fin], b[~fin])


def make_filter(gen, g, n_particles, n_groups, rng):
    """A filter over fixture data with the fixture's raw streams."""
    times = g["times"]
    rows = g["data"].reshape(times.size, -1)
    cols = {"time": np.repeat(times, rows.shape[1]),
            "incidence": rows.ravel()}
    if rows.shape[1] > 1:
        cols["group"] = np.tile(np.arange(1, rows.shape[1] + 1), times.size)
    return d.dust_filter_create(gen, 0, cols, n_particles=n_particles,
                                n_groups=n_groups, dt=float(g["dt"]),
                                seed=rng.astype("<u8").tobytes())


def plist_from(gen, flat, n_groups):
    out = []
    for row in flat.reshape(n_groups, gen.n_pars):
        p = {}
        off = 0
        for par in gen.parameters:
            v = row[off:off + par["length"]]
            if not np.isnan(v[0]):
                p[par["name"]] = v[0] if par["length"] == 1 else v
            off += par["length"]
        out.append(p)
    return out


@pytest.mark.parametrize("name", ["filter_sir_2groups", "filter_sir_missing"])
def test_filter_matches_reference_engine(built, name):
    g = golden(name)
    gen = d.sir()
    n = int(g["n_particles"])
    obj = make_filter(gen, g, n, 2, g["rng"])
    assert d.dust_likelihood_rng_state(obj) == g["rng"].astype("<u8").tobytes()
    pars = plist_from(gen, g["pars"], 2)
    ll = np.stack([d.dust_likelihood_run(obj, pars if i == 0 else None)
                   for i in range(g["ll"].shape[0])])
    assert_ll(ll, g["ll"])
    state = d.dust_likelihood_last_state(obj)
    np.testing.assert_array_equal(
        state.transpose(2, 1, 0).ravel(), g["state"])
    rng = np.frombuffer(d.dust_likelihood_rng_state(obj), dtype="<u8")
    np.testing.assert_array_equal(rng, g["rng_out"])


def test_single_group_workload_matches_reference_engine(built):
    g = golden("filter_sir_cases_1000")
    gen = d.sir_cases()
    obj = make_filter(gen, g, int(g["n_particles"]), None, g["rng"])
    pars = plist_from(gen, g["pars"], 1)[0]
    ll = [d.dust_likelihood_run(obj, pars) for _ in range(g["ll"].shape[0])]
    assert_ll(np.array(ll), g["ll"][:, 0])
    state = d.dust_likelihood_last_state(obj)
    np.testing.assert_array_equal(state.T.ravel(), g["state"])
    rng = np.frombuffer(d.dust_likelihood_rng_state(obj), dtype="<u8")
    np.testing.assert_array_equal(rng, g["rng_out"])


def _uneven_case(seed, n_particles, n_times=30, dt=0.25):
    G = len(n_particles)
    rs = np.random.default_rng(seed)
    plist = [{"N": 1e5, "I0": float(rs.integers(5, 50)),
              "beta": float(rs.uniform(0.15, 0.5)),
              "gamma": float(rs.uniform(0.05, 0.2))} for _ in range(G)]
    times = np.arange(1, n_times + 1, dtype=float)
    data = rs.poisson(20, size=(n_times, G)).astype(float)
    data[rs.uniform(size=data.shape) < 0.05] = np.nan
    return plist, times, data


@pytest.mark.parametrize("n_particles", [[512, 700, 1024, 1], [3000, 257],
                                         [33, 33, 33]])
def test_uneven_groups_match_oracle(port, n_particles):
    gen = d.sir_cases()
    plist, times, data = _uneven_case(5, n_particles)
    G = len(n_particles)
    cols = {"time": np.repeat(times, G), "group": np.tile(np.arange(1, G + 1),
                                                          times.size),
            "incidence": data.ravel()}
    obj = d.dust_filter_create(gen, 0, cols, n_particles=n_particles,
                               dt=0.25, seed=99)
    words = np.frombuffer(d.dust_likelihood_rng_state(obj), dtype="<u8")
    ll = np.stack([d.dust_likelihood_run(obj, plist) for _ in range(3)])
    flat = np.concatenate([gen.pack_pars(p) for p in plist])
    ll_cpu, state_cpu, rng_cpu = port.filter_run(
        "sir_cases", flat, n_particles, 0.0, times, data.ravel(), G, 0.25,
        words, n_runs=3, n_state=4)
    assert_ll(ll, ll_cpu)
    n_total = sum(n_particles)
    np.testing.assert_array_equal(d.dust_likelihood_last_state(obj),
                                  state_cpu[:n_total * 4])
    rng = np.frombuffer(d.dust_likelihood_rng_state(obj), dtype="<u8")
    np.testing.assert_array_equal(rng, rng_cpu)


def test_large_groups_match_oracle(port):
    """Groups spanning many tiles, where the exactness check of the
    parallel resampler matters."""
    n_particles = [8192, 20000, 4099]
    gen = d.sir_cases()
    plist, times, data = _uneven_case(11, n_particles, n_times=25)
    G = len(n_particles)
    cols = {"time": np.repeat(times, G), "group": np.tile(np.arange(1, G + 1),
                                                          times.size),
            "incidence": data.ravel()}
    obj = d.dust_filter_create(gen, 0, cols, n_particles=n_particles,
                               dt=0.25, seed=7)
    words = np.frombuffer(d.dust_likelihood_rng_state(obj), dtype="<u8")
    ll = d.dust_likelihood_run(obj, plist)
    flat = np.concatenate([gen.pack_pars(p) for p in plist])
    ll_cpu, state_cpu, _ = port.filter_run(
        "sir_cases", flat, n_particles, 0.0, times, data.ravel(), G, 0.25,
        words, n_state=4, n_threads=port.max_threads())
    assert_ll(ll, ll_cpu[0])
    np.testing.assert_array_equal(d.dust_likelihood_last_state(obj),
                                  state_cpu[:sum(n_particles) * 4])


def test_index_group_subset_matches_oracle(port):
    gen = d.sir()
    n = 50
    pars = [{"beta": 0.1 * (i + 1), "gamma": 0.2, "N": 1000, "I0": 10,
             "exp_noise": 1e6} for i in range(3)]
    times = np.array([4.0, 8, 12, 16])
    data = np.arange(1, 13, dtype=float).reshape(4, 3)
    cols = {"time": np.repeat(times, 3), "group": np.tile([1, 2, 3], 4),
            "incidence": data.ravel()}
    obj = d.dust_filter_create(gen, 0, cols, n_particles=n, seed=42)
    words = np.frombuffer(d.dust_likelihood_rng_state(obj), dtype="<u8")
    d.dust_likelihood_run(obj, pars)
    ll = d.dust_likelihood_run(obj, [pars[2], pars[0]], index_group=[3, 1])
    flat = np.concatenate([gen.pack_pars(p) for p in pars])
    ll_cpu, _, rng_cpu = port.filter_run("sir", flat, [n] * 3, 0.0, times,
                                         data.ravel(), 3, 1.0, words,
                                         n_runs=1, n_state=5)
    ll_cpu2, _, rng_cpu2 = port.filter_run(
        "sir", flat, [n] * 3, 0.0, times, data.ravel(), 3, 1.0, rng_cpu,
        n_runs=1, index_group=[2, 0], n_state=5)
    assert_ll(ll, ll_cpu2[0, [2, 0]])
    rng = np.frombuffer(d.dust_likelihood_rng_state(obj), dtype="<u8")
    np.testing.assert_array_equal(rng, rng_cpu2)


def test_initial_state_matches_oracle(port):
    gen = d.sir()
    pars = {"beta": 0.1, "gamma": 0.2, "N": 1000, "I0": 10, "exp_noise": 1e6}
    state = np.array([1000 - 17, 17, 0, 0, 0], dtype=float)
    times = np.array([4.0, 8, 12, 16])
    data = {"time": times, "incidence": np.array([1.0, 2, 3, 4])}
    obj = d.dust_filter_create(gen, 0, data, n_particles=100, seed=42)
    words = np.frombuffer(d.dust_likelihood_rng_state(obj), dtype="<u8")
    ll = [d.dust_likelihood_run(obj, pars, initial=state.reshape(5, 1))
          for _ in range(5)]
    init = np.tile(state, 100)
    ll_cpu, _, _ = port.filter_run("sir", gen.pack_pars(pars), [100], 0.0,
                                   times, data["incidence"], 1, 1.0, words,
                                   n_runs=5, initial=init, n_state=5)
    assert_ll(np.array(ll), ll_cpu[:, 0])


def test_group_equals_single_group_filter(built):
    """test-filter.R:151-204: group g of a multi-group filter equals a
    one-group filter seeded with that group's stream block."""
    gen = d.sir()
    n = 100
    pars = [{"beta": 0.1, "gamma": 0.2, "N": 1000, "I0": 10, "exp_noise": 1e6},
            {"beta": 0.2, "gamma": 0.2, "N": 1000, "I0": 10, "exp_noise": 1e6}]
    times = np.array([4.0, 8, 12, 16])
    inc = np.array([1.0, 2, 3, 4, 2, 3, 4, 5])
    cols = {"time": np.concatenate([times, times]),
            "group": np.repeat([1, 2], 4), "incidence": inc}
    obj = d.dust_filter_create(gen, 0, cols, n_particles=n, seed=42)
    s = d.dust_likelihood_rng_state(obj)
    assert s == d.rng_streams(2 * (n + 2), 42)
    res = np.stack([d.dust_likelihood_run(obj, pars) for _ in range(5)])
    obj1 = d.dust_filter_create(gen, 0, {"time": times,
                                         "incidence": inc[:4]},
                                n_particles=n, seed=42)
    res1 = [d.dust_likelihood_run(obj1, pars[0]) for _ in range(5)]
    seed2 = s[32 * (n + 2):32 * (n + 3)]
    obj2 = d.dust_filter_create(gen, 0, {"time": times,
                                         "incidence": inc[4:]},
                                n_particles=n, seed=seed2)
    assert d.dust_likelihood_rng_state(obj2) == s[32 * (n + 2):]
    res2 = [d.dust_likelihood_run(obj2, pars[1]) for _ in range(5)]
    np.testing.assert_array_equal(res[:, 0], res1)
    np.testing.assert_array_equal(res[:, 1], res2)


def test_filter_does_not_advance_second_stream(built):
    """test-filter.R:118-148."""
    gen = d.sir()
    pars = {"beta": 0.1, "gamma": 0.2, "N": 1000, "I0": 10, "exp_noise": 1e6}
    data = {"time": np.array([4.0, 8, 12, 16]),
            "incidence": np.array([1.0, 2, 3, 4])}
    n = 100
    obj = d.dust_filter_create(gen, 0, data, n_particles=n, seed=42)
    s0 = d.dust_likelihood_rng_state(obj)
    assert len(s0) == 32 * (n + 2)
    d.dust_likelihood_run(obj, pars)
    s1 = d.dust_likelihood_rng_state(obj)
    assert s1[32:64] == s0[32:64]
    d.dust_likelihood_run(obj, pars)
    s2 = d.dust_likelihood_rng_state(obj)
    assert s2[32:64] == s0[32:64]
    d.dust_likelihood_last_state(obj, select_random_particle=True)
    s3 = d.dust_likelihood_rng_state(obj)
    r = [int(x) for x in np.frombuffer(s1[32:64], dtype="<u8")]
    xoshiro.random_real(r)
    assert s3[32:64] == np.array(r, dtype="<u8").tobytes()
    assert s3[:32] == s2[:32] and s3[64:] == s2[64:]


def test_missing_data_equals_dropped_rows(built):
    """test-filter.R:439-457."""
    gen = d.sir()
    pars = {"beta": 0.1, "gamma": 0.2, "N": 1000, "I0": 10, "exp_noise": 1e6}
    t = np.array([4.0, 8, 12, 16])
    obj1 = d.dust_filter_create(gen, 0, {"time": t, "incidence": np.array(
        [1, 2, np.nan, 4])}, n_particles=100, seed=42)
    obj2 = d.dust_filter_create(gen, 0, {"time": t[[0, 1, 3]],
                                         "incidence": np.array([1.0, 2, 4])},
                                n_particles=100, seed=42)
    ll1 = [d.dust_likelihood_run(obj1, pars) for _ in range(10)]
    ll2 = [d.dust_likelihood_run(obj2, pars) for _ in range(10)]
    assert ll1 == ll2


def test_rng_state_round_trip(built):
    """test-filter.R:249-307."""
    gen = d.sir()
    pars = [{"beta": 0.1, "gamma": 0.2, "N": 1000, "I0": 10,
             "exp_noise": 1e6}] * 2
    t = np.array([4.0, 8, 12, 16])
    cols = {"time": np.repeat(t, 2), "group": np.tile([1, 2], 4),
            "incidence": np.arange(1, 9, dtype=float)}
    obj1 = d.dust_filter_create(gen, 0, cols, n_particles=100, seed=42)
    obj2 = d.dust_filter_create(gen, 0, cols, n_particles=100, seed=43)
    assert not np.array_equal(d.dust_likelihood_run(obj1, pars),
                              d.dust_likelihood_run(obj2, pars))
    s1 = d.dust_likelihood_rng_state(obj1)
    d.dust_likelihood_set_rng_state(obj2, s1)
    assert d.dust_likelihood_rng_state(obj2) == s1
    np.testing.assert_array_equal(d.dust_likelihood_run(obj1, pars),
                                  d.dust_likelihood_run(obj2, pars))


def test_filter_errors(built):
    gen = d.sir()
    t = np.array([4.0, 8, 12, 16])
    data = {"time": t, "incidence": np.array([1.0, 2, 3, 4])}
    obj = d.dust_filter_create(gen, 0, data, n_particles=10)
    with pytest.raises(d.DustError, match="'pars' cannot be NULL"):
        d.dust_likelihood_run(obj, None)
    with pytest.raises(d.DustError, match="State is not current"):
        d.dust_likelihood_last_state(obj)
    with pytest.raises(d.DustError, match="is later than the first time"):
        d.dust_filter_create(gen, 6, data, n_particles=10)
    with pytest.raises(d.DustError, match="Expected 'data' to have 2 groups"):
        d.dust_filter_create(gen, 0, data, n_particles=10, n_groups=2)
    with pytest.raises(d.DustError, match="does not have 'compare_data'"):
        d.dust_filter_create(d.walk(), 0, data, n_particles=10)
    bad = {"beta": 0.1, "gamma": -0.2, "N": 1000, "I0": 10}
    with pytest.raises(d.DustError, match="particles reported errors"):
        d.dust_likelihood_run(obj, bad)
    # a failed run does not poison the next one (reset re-initialises)
    ok = {"beta": 0.1, "gamma": 0.2, "N": 1000, "I0": 10}
    assert np.isfinite(d.dust_likelihood_run(obj, ok))


def test_forced_serial_resampling_is_identical(port):
    """The parallel resampler with its exactness check and the serial
    algorithm give identical filters (and both equal the oracle)."""
    from dust2_gb300 import interface
    n_particles = [30000, 4096, 700]
    gen = d.sir_cases()
    plist, times, data = _uneven_case(21, n_particles, n_times=20)
    G = len(n_particles)
    cols = {"time": np.repeat(times, G), "group": np.tile(np.arange(1, G + 1),
                                                          times.size),
            "incidence": data.ravel()}
    res = []
    for serial in (False, True):
        obj = d.dust_filter_create(gen, 0, cols, n_particles=n_particles,
                                   dt=0.25, seed=3)
        d.dust_likelihood_run(obj, plist)
        interface.dust_likelihood_set_serial_resample(obj, serial)
        ll = d.dust_likelihood_run(obj, plist)
        res.append((ll, d.dust_likelihood_last_state(obj),
                    d.dust_likelihood_rng_state(obj)))
        if serial:
            # every (time, group) with data is resampled serially
            n_resampled = int(np.sum(~np.isnan(data)))
            assert d.dust_likelihood_serial_fallbacks(obj) >= n_resampled
    np.testing.assert_array_equal(res[0][1], res[1][1])
    assert res[0][2] == res[1][2]
    assert_ll(res[0][0], res[1][0])


@pytest.mark.parametrize("n_particles", [[1000, 1, 33, 512, 1024, 96],
                                         [700, 700, 700]])
def test_fused_tail_is_identical(n_particles):
    """The one-launch tail for groups of at most 1024 particles and the
    separate kernels give the same bits: log-likelihoods (including a group
    whose weights are all -Inf, and a one-particle group), final states,
    generator states and (equal groups) trajectories, with and without
    forced serial resampling."""
    from dust2_gb300 import interface
    gen = d.sir_cases()
    plist, times, data = _uneven_case(8, n_particles, n_times=25)
    G = len(n_particles)
    data[:, G - 1] = 1e307  # every particle's log density is -Inf
    traj = len(set(n_particles)) == 1
    cols = {"time": np.repeat(times, G), "group": np.tile(np.arange(1, G + 1),
                                                          times.size),
            "incidence": data.ravel()}
    for serial in (False, True):
        res = []
        for fused in (True, False):
            obj = d.dust_filter_create(gen, 0, cols, n_particles=n_particles,
                                       dt=0.25, seed=11)
            interface.dust_likelihood_set_fused_tail(obj, fused)
            interface.dust_likelihood_set_serial_resample(obj, serial)
            ll = [d.dust_likelihood_run(obj, plist, save_trajectories=traj)
                  for _ in range(2)]
            res.append((np.array(ll),
                        d.dust_likelihood_last_trajectories(obj) if traj
                        else None,
                        d.dust_likelihood_last_state(obj),
                        d.dust_likelihood_rng_state(obj),
                        d.dust_likelihood_serial_fallbacks(obj)))
        assert np.all(np.isneginf(res[0][0][:, G - 1]))
        assert np.all(np.isfinite(res[0][0][:, :G - 1]))
        np.testing.assert_array_equal(res[0][0], res[1][0])
        np.testing.assert_array_equal(res[0][1], res[1][1])
        np.testing.assert_array_equal(res[0][2], res[1][2])
        assert res[0][3] == res[1][3]
        assert res[0][4] == res[1][4]


def test_resample_weight_adversarial(port):
    """Weights that make the parallel decision ambiguous, so that the
    serial running sum is taken (and its binade-segmented exact form is
    exercised): equal weights, powers of two down to subnormals, exact
    halfway cases, sparse weights and a range of 700 orders of magnitude."""
    rs = np.random.default_rng(17)
    cases = []
    for n in (1000, 40000):
        cases.append(np.ones(n))
        cases.append(np.ldexp(1.0, -rs.integers(0, 1100, n)))
        cases.append(rs.integers(0, 4, n) * 0.5)
        cases.append(np.where(rs.uniform(size=n) < 0.95, 0.0,
                              rs.uniform(size=n)))
        cases.append(np.exp(-700 * rs.uniform(size=n)))
        cases.append(np.ldexp(rs.integers(0, 1000, n).astype(float),
                              rs.integers(-30, 30, n)))
    for w in cases:
        for u in (0.0, 0.5, rs.uniform(), 1 - 1e-12):
            np.testing.assert_array_equal(d.resample_weight(w, u),
                                          port.resample_weight(w, u))


def test_resample_weight_hook(port):
    """test-filter-details.R:1-22 through the GPU kernels, including exact
    ties, where the parallel decision must defer to the serial one."""
    g = golden("filter_details")
    for u, idx in zip(g["u"], g["idx"]):
        np.testing.assert_array_equal(d.resample_weight(g["w"], u), idx)
    rs = np.random.default_rng(5)
    for n in (1, 2, 255, 256, 257, 5000, 100000):
        w = np.abs(rs.standard_cauchy(n))
        for u in (0.0, rs.uniform(), 1 - 1e-12):
            np.testing.assert_array_equal(d.resample_weight(w, u),
                                          port.resample_weight(w, u))
    # every boundary an exact tie: prefix sums and targets are integers
    w = np.ones(1000)
    for u in (0.0, 0.5):
        np.testing.assert_array_equal(d.resample_weight(w, u),
                                      port.resample_weight(w, u))
    w = np.zeros(50)
    w[7] = 3.0
    np.testing.assert_array_equal(d.resample_weight(w, 0.3),
                                  port.resample_weight(w, 0.3))


def test_scale_log_weights_hook(port):
    """test-filter-details.R:55-64 through the GPU kernels."""
    g = golden("filter_details")
    r, w = d.scale_log_weights(g["lw"])
    assert abs(r - g["lw_ret"][0]) <= 1e-12 * abs(g["lw_ret"][0])
    np.testing.assert_allclose(w, g["lw_w1"], rtol=4.5e-16, atol=0)
    assert w[3] == 0 and w[17] == 0
    r, w = d.scale_log_weights(np.full(5, -np.inf))
    assert r == -np.inf
    np.testing.assert_array_equal(w, np.full(5, -np.inf))
    r, w = d.scale_log_weights(np.array([-3.5]))
    assert r == -3.5
    rs = np.random.default_rng(8)
    x = rs.normal(-50, 20, 70000)
    r, w = d.scale_log_weights(x)
    rp, wp = port.scale_log_weights(x)
    assert abs(r - rp) <= 1e-12 * abs(rp)
    np.testing.assert_allclose(w, wp, rtol=4.5e-16, atol=1e-300)


def test_step_shapes_give_identical_results(port):
    """Every launch shape of the step kernel (group tiles of 32-256
    threads, one-warp tiles of 1-16 particles, one block per tile or a
    persistent grid taking tiles from a work queue) gives the same
    log-likelihoods, state and generators, equal to the oracle's; the
    autotuner times the candidates and keeps one of them."""
    gen = d.sir_cases()
    npg = [700, 33, 1500]
    rs = np.random.default_rng(8)
    plist = [{"beta": 0.2 + 0.1 * g, "gamma": 0.1, "N": 1e4, "I0": 10}
             for g in range(3)]
    times = np.arange(1, 31, dtype=float)
    data = rs.poisson(20, (times.size, 3)).astype(float)
    cols = {"time": np.repeat(times, 3), "incidence": data.ravel(),
            "group": np.tile(np.arange(1, 4), times.size)}
    results = []
    for shape in [(32, 0, False), (64, 0, False), (128, 0, False),
                  (256, 0, False), (32, 1, False), (32, 3, False),
                  (32, 16, False), (64, 0, True), (256, 0, True),
                  (32, 2, True), None]:
        obj = d.dust_filter_create(gen, 0, cols, n_particles=npg, dt=0.25,
                                   seed=21)
        if shape is not None:
            d.dust_likelihood_set_step_shape(obj, *shape)
        words = np.frombuffer(d.dust_likelihood_rng_state(obj), dtype="<u8")
        ll = d.dust_likelihood_run(obj, plist)
        state = np.asarray(d.dust_likelihood_last_state(obj)).ravel()
        rng = np.frombuffer(d.dust_likelihood_rng_state(obj), dtype="<u8")
        info = d.dust_likelihood_step_shape(obj)
        if shape is not None:
            assert (info["block"], info["per_tile"],
                    info["persistent"]) == shape
            assert info["n_candidates"] == 0
        else:
            assert info["n_candidates"] >= 8  # tuned among the candidates
            assert info["best_ms"] > 0
        results.append((ll, state, rng))
    flat = np.concatenate([gen.pack_pars(p) for p in plist])
    want, want_state, want_rng = port.filter_run(
        "sir_cases", flat, npg, 0.0, times, data.ravel(), 3, 0.25, words,
        n_state=4)
    for ll, state, rng in results:
        np.testing.assert_allclose(ll, want[0], rtol=1e-12, atol=0)
        np.testing.assert_array_equal(ll, results[0][0])
        np.testing.assert_array_equal(state, want_state[:sum(npg) * 4])
        np.testing.assert_array_equal(rng, want_rng)
