"""Test-side glue: the benchmark input recipes (dust2_gb300.workloads)
driven by a CPU oracle instead of the CUDA engine."""

import numpy as np

import xoshiro
from dust2_gb300 import workloads


def oracle_simulate(oracle):
    def simulate(name, flat, n_groups, n_particles, dt, seed, times):
        rng = xoshiro.streams(seed, n_groups * n_particles)
        out, _ = oracle.discrete_simulate(name, flat, n_groups, n_particles,
                                          0.0, dt, rng, times)
        n_state = {"sir_cases": 4, "sir": 5}[name]
        return out[:times.size * n_groups * n_particles * n_state]
    return simulate


def sir_small(oracle):
    return workloads.sir_small(oracle_simulate(oracle))


def pack(name, plist):
    return workloads.pack(name, plist)


def sir_pars(plist):
    return pack("sir", plist)


def seir_pars(r0_values):
    return pack("seir_age", workloads.seir_plist(r0_values))
