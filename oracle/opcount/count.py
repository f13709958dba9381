"""TEST INFRASTRUCTURE (oracle): algorithmic FP64 operations per
particle-step of the discrete filter's step + compare work.

Runs oracle/opcount/opcount.cpp (the SIR and age-structured SEIR systems
and the binomial sampler restated over an operation-counting real type)
as a particle filter on a sample of the benchmark's batched workloads,
checks that its log-likelihoods equal the oracle port's bit for bit (so
the counted run drew exactly the engine's draws), and prints the counts
per particle-step; and dust2's dopri5 with the sirode system over the
same type on the batched dopri5 workload, checked equal to the port's
integration, per attempted step:

    python -m oracle.opcount.count [--workload sir_batched|seir_batched|
                                               ode_batched]

Flops: +, -, *, / (a reciprocal counts as one division) and sqrt one
each, a fused multiply-add two.  Comparisons, floors and calls of exp,
log, log k! and lgamma are reported beside them, not as flops.  The
inputs are the benchmark's (dust2_gb300/workloads.py), simulated, packed
and seeded by the oracle, so this never loads the CUDA library.
"""

import argparse
import ctypes
import json
import subprocess
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ORACLE = HERE.parent
REPO = ORACLE.parent
CSRC = REPO / "dust2_gb300" / "csrc"
SRC = HERE / "opcount.cpp"
LIB = ORACLE / "_build" / "libopcount.so"

OPS = ["add", "mul", "div", "fma", "sqrt", "cmp", "floor", "exp", "log",
       "log_factorial", "lgamma", "pow"]
N_STATE = {"sir_cases": 4, "seir_age": 96}
STEPS_PER_OBS = 4


def build(force=False):
    inputs = [SRC] + list((CSRC / "dust2gpu").glob("*.hpp")) + \
        list((CSRC / "systems").glob("*.hpp"))
    newest = max(p.stat().st_mtime for p in inputs)
    if not force and LIB.exists() and LIB.stat().st_mtime >= newest:
        return LIB
    LIB.parent.mkdir(exist_ok=True)
    tmp = LIB.with_suffix(".so.tmp")
    cmd = ["g++", "-std=c++17", "-O2", "-fPIC", "-shared",
           "-ffp-contract=off", "-fno-strict-aliasing", "-I", str(CSRC),
           "-I", str(CSRC / "compat"), str(SRC), "-o", str(tmp)]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"opcount build failed:\n{res.stderr}")
    tmp.replace(LIB)
    return LIB


def _lib():
    lib = ctypes.CDLL(str(build()))
    lib.opcount_n_ops.restype = ctypes.c_int
    assert lib.opcount_n_ops() == len(OPS)
    lib.opcount_filter.restype = ctypes.c_int
    return lib


def counted_filter(system, pars, n_particles, dt, times, data, words):
    """Filter runs of every group given; returns (ll per group, step op
    counts, compare op counts) as dicts keyed by OPS."""
    d = ctypes.POINTER(ctypes.c_double)
    u = ctypes.POINTER(ctypes.c_uint64)
    G = len(n_particles)
    pars = np.ascontiguousarray(pars, dtype=np.float64)
    times = np.ascontiguousarray(times, dtype=np.float64)
    data = np.ascontiguousarray(data, dtype=np.float64)
    words = np.ascontiguousarray(words, dtype=np.uint64)
    npa = np.ascontiguousarray(n_particles, dtype=np.intc)
    ll = np.empty(G)
    step = np.zeros(len(OPS), dtype=np.uint64)
    comp = np.zeros(len(OPS), dtype=np.uint64)
    rc = _lib().opcount_filter(
        system.encode(), pars.ctypes.data_as(d),
        ctypes.c_int(pars.size // G), ctypes.c_int(G),
        npa.ctypes.data_as(ctypes.POINTER(ctypes.c_int)),
        ctypes.c_double(dt), times.ctypes.data_as(d),
        ctypes.c_int(times.size), data.ctypes.data_as(d),
        words.ctypes.data_as(u), ll.ctypes.data_as(d),
        step.ctypes.data_as(u), comp.ctypes.data_as(u))
    if rc != 0:
        raise RuntimeError(f"opcount: unknown system {system}")
    return (ll, dict(zip(OPS, (int(x) for x in step))),
            dict(zip(OPS, (int(x) for x in comp))))


def flops(c):
    return c["add"] + c["mul"] + c["div"] + c["sqrt"] + 2 * c["fma"]


def counted_dopri5(pars, times):
    """sirode instances (packed rows: I0, N, beta, gamma) integrated from 0
    through `times` by dust2's dopri5 over the counting type; returns
    (out [time][instance][5], attempted steps per instance, op counts)."""
    d = ctypes.POINTER(ctypes.c_double)
    pars = np.ascontiguousarray(pars, dtype=np.float64)
    times = np.ascontiguousarray(times, dtype=np.float64)
    n = pars.size // 4
    out = np.empty(times.size * n * 5)
    steps = np.empty(n, dtype=np.int64)
    ops = np.zeros(len(OPS), dtype=np.uint64)
    _lib().opcount_dopri5_sirode(
        pars.ctypes.data_as(d), ctypes.c_int(4), ctypes.c_int(n),
        times.ctypes.data_as(d), ctypes.c_int(times.size),
        out.ctypes.data_as(d),
        steps.ctypes.data_as(ctypes.POINTER(ctypes.c_int64)),
        ops.ctypes.data_as(ctypes.POINTER(ctypes.c_uint64)))
    return out, steps, dict(zip(OPS, (int(x) for x in ops)))


def count_dopri5(n_instances):
    """The first n_instances of the batched dopri5 workload, checked
    against the oracle port (outputs and step counts equal bit for bit);
    returns op counts per attempted step."""
    from oracle import pyoracle
    from dust2_gb300 import workloads
    w = workloads.sirode_batched(n_instances=n_instances)
    out, steps, ops = counted_dopri5(w["pars"], w["times"])
    want, stats = pyoracle.port().ode_simulate(
        "sirode", w["pars"], n_instances, 1, 0.0, w["times"], 5)
    if not (np.array_equal(out, want) and
            np.array_equal(steps, stats[:, 0])):
        raise RuntimeError("counted dopri5 differs from the port")
    total = int(steps.sum())
    return {"attempted_steps": total,
            "flops_per_step": flops(ops) / total,
            "per_step": {k: ops[k] / total for k in OPS},
            "equal_port": True}


def oracle_simulate():
    from oracle import pyoracle

    def simulate(name, flat, n_groups, n_particles, dt, seed, times):
        rng = pyoracle.rng_streams(n_groups * n_particles, seed)
        out, _ = pyoracle.port().discrete_simulate(
            name, flat, n_groups, n_particles, 0.0, dt, rng, times)
        return out[:times.size * n_groups * n_particles * N_STATE[name]]
    return simulate


def workload(name):
    from oracle import pyoracle
    from dust2_gb300 import workloads
    sim = oracle_simulate()
    if name == "sir_batched":
        w = workloads.sir_batched(sim, packer=pyoracle.pack_pars)
        w["system"] = "sir_cases"
    elif name == "seir_batched":
        w = workloads.seir_batched(sim, packer=pyoracle.pack_pars)
        w["system"] = "seir_age"
    else:
        raise ValueError(name)
    return w


def count(w, groups, n_particles=None, n_obs=None):
    """Counted filter run on the given groups of workload w (particle
    counts as the workload's unless given; the first n_obs data times),
    checked against the oracle port; returns a summary dict."""
    from oracle import pyoracle
    G_all = len(w["n_particles"])
    npar = np.asarray(w["pars"]).size // G_all
    pars = np.asarray(w["pars"]).reshape(G_all, npar)[groups].ravel()
    times = np.asarray(w["times"])[:n_obs]
    data = np.asarray(w["data"]).reshape(w["times"].size, G_all)
    data = data[:times.size, groups]
    npg = [n_particles or w["n_particles"][g] for g in groups]
    words = pyoracle.rng_streams(sum(n + 2 for n in npg), w["seed"])
    ll, step, comp = counted_filter(w["system"], pars, npg, w["dt"], times,
                                    data, words)
    ll_port, _, _ = pyoracle.port().filter_run(
        w["system"], pars, npg, 0.0, times, data.ravel(), len(groups),
        w["dt"], words, n_state=N_STATE[w["system"]])
    if not np.array_equal(ll, ll_port[0]):
        raise RuntimeError(f"counted run differs from the port: {ll} vs "
                           f"{ll_port[0]}")
    ps = sum(npg) * times.size * STEPS_PER_OBS
    total = {k: step[k] + comp[k] for k in OPS}
    return {"particle_steps": ps,
            "flops_per_particle_step": flops(total) / ps,
            "step_flops_per_particle_step": flops(step) / ps,
            "compare_flops_per_particle_step": flops(comp) / ps,
            "per_particle_step": {k: total[k] / ps for k in OPS},
            "ll_equal_port": True}


def main():
    p = argparse.ArgumentParser()
    p.add_argument("--workload", default=None)
    args = p.parse_args()
    samples = {"sir_batched": dict(groups=list(range(8))),
               "seir_batched": dict(groups=[0, 1, 2, 3], n_particles=1024)}
    names = [args.workload] if args.workload else \
        list(samples) + ["ode_batched"]
    for name in names:
        if name == "ode_batched":
            out = count_dopri5(16384)
            out["workload"] = name
            out["sample"] = "instances 1-16384, integrated 0..200"
            print(json.dumps(out))
            continue
        s = samples[name]
        out = count(workload(name), **s)
        out["workload"] = name
        out["sample"] = (f"groups {s['groups']}, "
                         f"{s.get('n_particles') or 'all'} particles each, "
                         "all observations")
        print(json.dumps(out))
        sys.stdout.flush()


if __name__ == "__main__":
    main()
