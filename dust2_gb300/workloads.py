"""Synthetic inputs of the benchmark workloads (no external datasets).

Each builder takes a `simulate` callable, so the same recipe runs on the
CUDA engine (benchmarks) and on the CPU oracle (test fixtures):
    simulate(name, flat_pars, n_groups, n_particles, dt, seed, times)
      -> array [n_times][group][particle][state]
Parameter packing uses the system's parameter table: from the library by
default, or from any `packer(name, pars) -> row` given (the CPU oracle's,
so that CPU-only callers need not load the CUDA library).
"""

import math

import numpy as np

from .interface import Generator


def pack(name, plist, packer=None):
    if packer is None:
        row = Generator(name).pack_pars
    else:
        def row(p):
            return packer(name, p)
    return np.concatenate([row(p) for p in plist])


def sir_small(simulate, packer=None):
    """Single-group SIR filter: N=1000, I0=10, beta=0.2, gamma=0.1,
    dt=0.25, 1000 particles, 100 daily observations simulated by the same
    model from seed 42 plus Poisson observation noise."""
    p = {"N": 1000, "I0": 10, "beta": 0.2, "gamma": 0.1}
    flat = pack("sir_cases", [p], packer)
    times = np.arange(1, 101, dtype=float)
    sim = simulate("sir_cases", flat, 1, 1, 0.25, 42, times)
    cases = np.asarray(sim).reshape(times.size, 4)[:, 3]
    rs = np.random.default_rng(42)
    data = rs.poisson(cases + 1e-6).astype(float)
    return {"pars": flat, "plist": [p], "times": times, "data": data,
            "dt": 0.25, "n_particles": 1000, "seed": 42}


def sir_batched(simulate, n_groups=64, seed=1, n_obs=200, packer=None):
    """Batched SIR filter: 64 groups with beta ~ U(0.1, 0.5), gamma ~
    U(0.05, 0.2), N = 1e6, I0 ~ U{1..100}; particle counts
    round(2^U(9, 15)); 200 daily observations per group simulated from
    seed 1 plus Poisson noise."""
    rs = np.random.default_rng(seed)
    plist = []
    for _ in range(n_groups):
        plist.append({"N": 1e6, "I0": float(rs.integers(1, 101)),
                      "beta": float(rs.uniform(0.1, 0.5)),
                      "gamma": float(rs.uniform(0.05, 0.2))})
    n_particles = [int(round(2 ** rs.uniform(9, 15))) for _ in range(n_groups)]
    flat = pack("sir_cases", plist, packer)
    times = np.arange(1, n_obs + 1, dtype=float)
    sim = simulate("sir_cases", flat, n_groups, 1, 0.25, seed, times)
    cases = np.asarray(sim).reshape(times.size, n_groups, 4)[:, :, 3]
    data = rs.poisson(cases + 1e-6).astype(float)  # [time][group]
    return {"pars": flat, "plist": plist, "times": times, "data": data,
            "dt": 0.25, "n_particles": n_particles, "seed": seed}


def contact_matrix(seed=7, n_age=16):
    """Random symmetric contact matrix, entries Gamma(2, 1) / 16."""
    rs = np.random.default_rng(seed)
    a = rs.gamma(2.0, 1.0, size=(n_age, n_age)) / 16
    return np.triu(a) + np.triu(a, 1).T


def seir_plist(r0_values, seed=7):
    c = contact_matrix(seed)
    return [{"R0": float(r), "sigma": 0.2, "gamma": 0.1, "size": 20,
             "I0": 1, "contact": c.ravel()} for r in r0_values]


def seir_batched(simulate, n_groups=32, n_particles=8192, seed=3,
                 n_obs=365, packer=None):
    """Age-structured SEIR filter: 16 ages, contact matrix from seed 7,
    sigma = 0.2, gamma = 0.1, R0 ~ U(1.2, 3) per group, dt = 0.25,
    32 groups x 8192 particles; 365 daily observations of total incidence
    per group simulated from seed 3 plus negative-binomial (size 20)
    observation noise."""
    rs = np.random.default_rng(seed)
    r0 = rs.uniform(1.2, 3.0, n_groups)
    plist = seir_plist(r0)
    flat = pack("seir_age", plist, packer)
    times = np.arange(1, n_obs + 1, dtype=float)
    sim = simulate("seir_age", flat, n_groups, 1, 0.25, seed, times)
    inc = np.asarray(sim).reshape(times.size, n_groups, 96)[:, :, 80:96]
    mu = inc.sum(axis=2) + 1e-6
    size = 20.0
    data = rs.negative_binomial(size, size / (size + mu)).astype(float)
    return {"pars": flat, "plist": plist, "times": times, "data": data,
            "dt": 0.25, "n_particles": [n_particles] * n_groups,
            "seed": seed}


def serving_clients(simulate, n_clients=64, rounds=2, seed=11, rate=200.0,
                    n_days=365, packer=None):
    """Likelihood requests of concurrent MCMC chains on the age-structured
    SEIR: one session per client with particles round(2^U(9, 15)) (log-
    uniform in 512..32768) and U{50..365} days of data (simulated total
    incidence from seed 11 plus negative-binomial noise, size 20); each
    request a new R0 ~ U(1.2, 3).  Arrivals: the clients' first requests
    form a Poisson stream at `rate` per second; after a result a client
    waits an exponential time with mean n_clients / rate before its next
    request (each chain has one request outstanding at a time)."""
    rs = np.random.default_rng(seed)
    r0 = rs.uniform(1.2, 3.0, n_clients)
    plist = seir_plist(r0)
    flat = pack("seir_age", plist, packer)
    times = np.arange(1, n_days + 1, dtype=float)
    sim = simulate("seir_age", flat, n_clients, 1, 0.25, seed, times)
    inc = np.asarray(sim).reshape(n_days, n_clients, 96)[:, :, 80:96]
    mu = inc.sum(axis=2) + 1e-6
    size = 20.0
    data = rs.negative_binomial(size, size / (size + mu)).astype(float)
    sizes = [(int(round(2 ** rs.uniform(9, 15))), int(rs.integers(50, 366)))
             for _ in range(n_clients)]
    first = np.cumsum(rs.exponential(1.0 / rate, n_clients))
    # each client's proposals and think times come from its own stream,
    # so the first r requests are the same whatever `rounds` is
    think = np.empty((n_clients, rounds))
    clients = []
    for i, (n, n_obs) in enumerate(sizes):
        cs = np.random.default_rng([seed, i])
        r0_seq = cs.uniform(1.2, 3.0, rounds)
        think[i] = cs.exponential(n_clients / rate, rounds)
        clients.append({
            "n_particles": n,
            "data": {"time": times[:n_obs], "incidence": data[:n_obs, i]},
            "pars": [dict(plist[i], R0=float(r)) for r in r0_seq],
            "seed": seed * 1000 + i,
            "particle_steps": n * n_obs * 4})
    return {"clients": clients, "first_arrival": first, "think": think,
            "rate": rate, "dt": 0.25}


def sirode_batched(n_instances=262144, seed=3):
    """dopri5 workload: beta ~ U(0.1, 0.5), gamma ~ U(0.05, 0.2), N = 1e6,
    I0 ~ U(1, 100); one parameter group per instance."""
    rs = np.random.default_rng(seed)
    beta = rs.uniform(0.1, 0.5, n_instances)
    gamma = rs.uniform(0.05, 0.2, n_instances)
    i0 = rs.uniform(1, 100, n_instances)
    # the sirode parameter table: I0, N, beta, gamma
    flat = np.empty((n_instances, 4))
    flat[:, 0] = i0
    flat[:, 1] = 1e6
    flat[:, 2] = beta
    flat[:, 3] = gamma
    return {"pars": flat.ravel(), "n_groups": n_instances,
            "times": np.arange(0, 201, dtype=float)}
