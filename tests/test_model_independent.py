"""Filter runs restated end to end in plain Python, against the oracle port.

The engine's samplers and system classes are shared by the CUDA kernels
and the CPU oracle, so the oracle cannot catch an error made identically
in both (test_sampler_independent.py covers the samplers alone).  Here
the benchmark's two filtered models -- the SIR with a Poisson compare and
the 16-age SEIR with a negative-binomial compare -- and dust2's bootstrap
filter (run_to_time with the daily zero_every reset, compare_data,
scale_log_weights, systematic resample_weight, reorder; dust2's
filter.hpp:42-104, filter_details.hpp:11-74) are written again from the
model definitions with the host's libm, the independent numpy generator
(tests/xoshiro.py) and the independent samplers of
test_sampler_independent.py.  The port must agree: particle state and
generator words exactly (the same draws along every stream), the
log-likelihood to 1e-12 relative (libm and the engine round their
elementary functions differently by at most an ulp)."""

import math

import numpy as np

import xoshiro
from oracle import pyoracle
from test_sampler_independent import binomial, fma


def scale_log_weights(w):
    if len(w) == 1:
        return w[0], w
    w = [-math.inf if math.isnan(x) else x for x in w]
    mx = max(w)
    if mx == -math.inf:
        return mx, w
    w = [math.exp(x - mx) for x in w]
    tot = 0.0
    for x in w:
        tot += x
    return math.log(tot / len(w)) + mx, w


def resample_weight(w, u):
    n = len(w)
    tot = 0.0
    for x in w:
        tot += x
    uu0 = tot * u / n
    du = tot / n
    ww = 0.0
    j = 0
    idx = []
    for i in range(n):
        uu = uu0 + i * du
        while ww < uu and j < n:
            ww += w[j]
            j += 1
        idx.append(j - 1 if j > 0 else 0)
    return idx


def filter_run(model, n, times, data, dt, words):
    """One group of n particles; words: the raw generator words of its
    stream block [2 filter streams | n particle streams].  Returns (ll,
    final state per particle, generator words per stream)."""
    streams = [[int(x) for x in words[4 * k:4 * k + 4]] for k in range(n + 2)]
    frng, rngs = streams[0], streams[2:]
    state = [model.initial() for _ in range(n)]
    time, ll = 0.0, 0.0
    for t, d in zip(times, data):
        n_steps = round((t - time) / dt)
        for j in range(n):
            for i in range(n_steps):
                time_i = time + i * dt
                if math.fmod(time_i, 1.0) == 0:
                    model.zero(state[j])
                state[j] = model.update(rngs[j], state[j], dt)
        time += n_steps * dt
        w = [model.compare(state[j], d) for j in range(n)]
        if any(x != 0 for x in w):
            inc, w = scale_log_weights(w)
            ll += inc
            idx = resample_weight(w, xoshiro.random_real(frng))
            state = [list(state[k]) for k in idx]
    return ll, state, streams


class SIR:
    """sir_cases: S, I, R, daily incidence; Poisson(incidence + 1e-6)."""

    def __init__(self, p):
        self.p = p

    def initial(self):
        return [self.p["N"] - self.p["I0"], self.p["I0"], 0.0, 0.0]

    def zero(self, y):
        y[3] = 0.0

    def update(self, s, y, dt):
        beta, gamma, N = self.p["beta"], self.p["gamma"], self.p["N"]
        S, I, R, inc = y
        p_SI = 1 - math.exp(-beta * I / N * dt)
        p_IR = 1 - math.exp(-gamma * dt)
        n_SI = binomial(s, S, p_SI)
        n_IR = binomial(s, I, p_IR)
        return [S - n_SI, I + n_SI - n_IR, R + n_IR, inc + n_SI]

    def compare(self, y, x):
        if math.isnan(x):
            return 0.0
        lam = y[3] + 1e-6
        return x * math.log(lam) - lam - math.lgamma(x + 1.0)


class SEIR:
    """seir_age: per age S, E, I, R, cumulative and daily incidence;
    infection from a contact matrix scaled to R0 by its spectral radius;
    negative-binomial(size, mu = total daily incidence + 1e-6)."""

    A = 16

    def __init__(self, p):
        A = self.A
        self.c = [[float(v) for v in p["contact"][a * A:(a + 1) * A]]
                  for a in range(A)]
        self.N = [62500.0] * A
        self.I0, self.sigma, self.gamma = p["I0"], p["sigma"], p["gamma"]
        self.size = p["size"]
        # spectral radius by power iteration, as the system derives it
        x, rho = [1.0] * A, 0.0
        for _ in range(1000):
            y = []
            for a in range(A):
                acc = 0.0
                for b in range(A):
                    acc += self.c[a][b] * x[b]
                y.append(acc)
            norm = max(abs(v) for v in y)
            x = [v / norm for v in y]
            if abs(norm - rho) < 1e-14 * norm:
                rho = norm
                break
            rho = norm
        self.beta = p["R0"] * self.gamma / rho
        self.inv_N = [1.0 / v for v in self.N]

    def initial(self):
        A = self.A
        return ([n - self.I0 for n in self.N] + [0.0] * A + [self.I0] * A +
                [0.0] * (3 * A))

    def zero(self, y):
        for a in range(self.A):
            y[5 * self.A + a] = 0.0

    def update(self, s, y, dt):
        A = self.A
        S, E, I = y[:A], y[A:2 * A], y[2 * A:3 * A]
        R, cum, inc = y[3 * A:4 * A], y[4 * A:5 * A], y[5 * A:]
        x = [I[b] * self.inv_N[b] for b in range(A)]
        p_SE = []
        for a in range(A):
            acc = 0.0
            for b in range(A):
                acc = fma(self.c[a][b], x[b], acc)
            p_SE.append(1 - math.exp(-(self.beta * acc) * dt))
        p_EI = 1 - math.exp(-self.sigma * dt)
        p_IR = 1 - math.exp(-self.gamma * dt)
        out = list(y)
        for a in range(A):
            n_SE = binomial(s, S[a], p_SE[a])
            n_EI = binomial(s, E[a], p_EI)
            n_IR = binomial(s, I[a], p_IR)
            out[a] = S[a] - n_SE
            out[A + a] = E[a] + n_SE - n_EI
            out[2 * A + a] = I[a] + n_EI - n_IR
            out[3 * A + a] = R[a] + n_IR
            out[4 * A + a] = cum[a] + n_EI
            out[5 * A + a] = inc[a] + n_EI
        return out

    def compare(self, y, x):
        if math.isnan(x):
            return 0.0
        mu = 0.0
        for a in range(self.A):
            mu += y[5 * self.A + a]
        mu += 1e-6
        size = self.size
        lsm = math.log(size + mu)
        return (math.lgamma(x + size) - math.lgamma(size) -
                math.lgamma(x + 1.0) + size * (math.log(size) - lsm) +
                x * (math.log(mu) - lsm))


def _check(name, model, p, n, times, data, seed, n_state):
    words = xoshiro.streams(seed, n + 2)
    ll, state, streams = filter_run(model, n, times, data, 0.25, words)
    flat = pyoracle.pack_pars(name, p)
    ll_port, st_port, rng_port = pyoracle.port().filter_run(
        name, flat, [n], 0.0, times, np.asarray(data, dtype=float), 1, 0.25,
        words, n_state=n_state)
    np.testing.assert_allclose(ll, ll_port[0, 0], rtol=1e-12, atol=0)
    np.testing.assert_array_equal(
        np.asarray(state).ravel(), st_port[:n * n_state])
    np.testing.assert_array_equal(
        np.array([w for s in streams for w in s], dtype=np.uint64),
        rng_port[:4 * (n + 2)])
    return ll


def test_sir_filter_restated_equals_port():
    p = {"N": 1e6, "I0": 37.0, "beta": 0.31, "gamma": 0.11}
    times = np.arange(1, 31, dtype=float)
    rs = np.random.default_rng(8)
    data = rs.poisson(np.linspace(5, 400, times.size)).astype(float)
    data[7] = np.nan  # a missing observation draws nothing, weighs 0
    ll = _check("sir_cases", SIR(p), p, 160, times, data, 71, 4)
    assert np.isfinite(ll)


def test_seir_filter_restated_equals_port():
    from dust2_gb300 import workloads
    p = workloads.seir_plist([2.2])[0]
    p["I0"] = 40.0  # every compartment busy from the first days
    times = np.arange(1, 17, dtype=float)
    rs = np.random.default_rng(9)
    data = rs.negative_binomial(20, 20 / (20 + np.linspace(60, 600, 16)))
    ll = _check("seir_age", SEIR(p), p, 24, times, data.astype(float), 53,
                96)
    assert np.isfinite(ll)
