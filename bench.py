"""Benchmark of the dust2 hot path on one GB300.

Default workload (`--workload serve_seir`): filter likelihoods of the
age-structured stochastic SEIR (16 ages, 96 FP64 states, dt 0.25,
negative-binomial compare) requested by 64 concurrent MCMC-chain clients:
first requests a Poisson stream at 200/s, then one request outstanding
per client with exponential think times; per client a session with
round(2^U(9, 15)) particles and U{50..365} days of data (seed 11), a new
R0 ~ U(1.2, 3) per request.  A step is 16 requests (20 steps: 5 per
client).  The line reports the served engine (continuous batching on one
likelihood server) against the plain path (the same requests one by one
through dust_likelihood_run), p50/p99 latency of both, the plain path's
per-request share of the device's full rate (and so the most any batching
could gain), the roofline of the SEIR step kernel and the CPU path on a
bounded sample.

Other workloads (`--workload`): sir_batched (64 SIR groups, uneven
particle counts round(2^U(9, 15)), 200 observations), seir_batched (32
SEIR groups x 8192 particles, 365 observations), sir_small (one SIR group
of 1000 particles, 100 observations), ode_batched (262,144 sirode
instances, dopri5 to t = 200).  Data are synthetic everywhere: the model
itself generates them from fixed seeds.

Filter workloads report:
  value   particle-steps/s of whole likelihood runs, device-timed with CUDA
          events on the filter's stream, inputs resident on the device, L2
          flushed (256 MB write) between timed runs;
  e2e     the same metric through the public API (dust_likelihood_run:
          parameters copied host->device, log-likelihoods device->host,
          every step), wall-clock;
  roofline  for the dominant kernel (the step+compare kernel) against the
          FP64 pipe: executed FP64 operations per particle-step (ncu SASS
          counters of this kernel, stated in the constant below) times the
          particle-steps of one launch, over the kernel's device time
          measured live with CUDA events; peak from a DFMA microbenchmark
          run in this process; plus the HBM roofline of the reorder gather;
  cpu_baseline  the CPU restatement of dust2's engine (OpenMP over all
          host cores) on a bounded sample of the same workload.

`--impl reference` times that CPU implementation alone (the reference arm),
with inputs built by the oracle, so it never loads the CUDA library.
Multi-GPU (torchrun) runs independent replicas, one per GPU: the path has
no cross-group exchange.
"""

import argparse
import json
import math
import os
import subprocess
import sys
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

# Executed FP64 operations (DADD + DMUL + 2 DFMA, per thread) per
# particle-step of the step+compare kernel, per workload, from the ncu SASS
# counters of that kernel (summaries under profiles/): whole-run averages
# of an earlier build, scaled by the ratio of the current build's count to
# that build's at the same observation (one-launch captures).  A workload
# without an entry reports no achieved rate.
FP64_OPS_PER_PARTICLE_STEP = {"sir_batched": 180.9, "seir_batched": 3028.9,
                              "ode_batched": 552.0}
# FP64-pipe thread instructions (arithmetic, comparisons, conversions) per
# unit, from the same captures: the pipe's own roofline (every instruction
# takes one lane-slot; the DFMA peak in TFLOP/s is two flops per slot).
FP64_PIPE_INST_PER_UNIT = {"sir_batched": 132.7, "seir_batched": 2155.8,
                           "ode_batched": 351.5}


# A second basis for the FP64 roofline, independent of moving work off
# the FP64 pipe: the FP64 operations (DADD + DMUL + 2 DFMA) the same step
# kernel executed per particle-step when exp and log were still evaluated
# in FP64 (Tang's table methods), measured by ncu on that build (whole
# runs of the batched workloads).  The integer fixed-point exp and log of
# the current build compute the same values with no FP64 instruction, so
# this counts the FP64 work of the algorithm as a plain FP64
# implementation would issue it.
FP64_FORMULATION_OPS = {"sir_batched": 259.6, "seir_batched": 4552.2}


def formulation_roofline(workload, units_per_s, peak_tflops):
    ops = FP64_FORMULATION_OPS.get(workload)
    if ops is None or not units_per_s:
        return None
    achieved = ops * units_per_s / 1e12
    return {"flops_per_unit": ops, "achieved": achieved,
            "frac": achieved / peak_tflops, "unit": "TFLOP/s",
            "basis": "FP64 ops per particle-step of the step kernel with "
                     "exp/log in FP64 (ncu, earlier build)"}


# The algorithmic basis: FP64 operations per particle-step of the step +
# compare work counted by running the systems and the binomial sampler
# over an operation-counting real type (oracle/opcount: +, -, *, / and
# sqrt one flop each, a fused multiply-add two; exp, log, log k! and
# lgamma counted as calls, not flops), on a sample of each batched
# workload whose log-likelihoods equal the oracle port's bit for bit
# (`python -m oracle.opcount.count`: batched SIR groups 1-8, all
# particles; batched SEIR groups 1-4 at 1024 particles; all observations),
# and, per attempted step, dust2's unfused dopri5 with the sirode system
# over the same type on instances 1-16384 of the dopri5 workload (outputs
# and step counts equal to the port's).
FP64_ALGORITHMIC_OPS = {"sir_batched": 59.95, "seir_batched": 1738.7,
                        "ode_batched": 443.7}
ALGORITHMIC_CALLS = {
    "sir_batched": {"exp": 1.66, "log": 1.28, "log_factorial": 1.72,
                    "lgamma": 0.25},
    "seir_batched": {"exp": 44.4, "log": 26.7, "log_factorial": 35.2,
                     "lgamma": 0.75},
    "ode_batched": {"pow": 1.08}}


def algorithmic_roofline(workload, units_per_s, peak_tflops):
    ops = FP64_ALGORITHMIC_OPS.get(workload)
    if ops is None or not units_per_s:
        return None
    achieved = ops * units_per_s / 1e12
    return {"flops_per_unit": ops, "achieved": achieved,
            "frac": achieved / peak_tflops, "unit": "TFLOP/s",
            "calls_per_unit": ALGORITHMIC_CALLS[workload],
            "basis": "FP64 operations of the model and samplers counted "
                     "by an operation-counting real type (oracle/opcount)"}


# DRAM bytes (dram__bytes_read.sum + dram__bytes_write.sum) per unit of the
# same kernel, from ncu captures (SIR: a whole run; SEIR: one launch at
# observation 200, the state in a per-thread local-memory array; dopri5:
# one launch over all outputs); `traffic` is this times the units of one
# launch.
DRAM_BYTES_PER_UNIT = {"sir_batched": 19.4, "seir_batched": 1598.0,
                       "ode_batched": 36.5}


# The CPU path is timed with the oracle's timing build: the host's libm
# exp and log, as dust2 evaluates them through monty, in place of the
# integer fixed-point functions the GPU uses (which are slower on a CPU).
CPU_MATH = "host libm exp/log (as dust2/monty call them)"


def traffic_per_launch(workload, units_per_launch):
    b = DRAM_BYTES_PER_UNIT.get(workload)
    return None if b is None else b * units_per_launch


def hbm_peak():
    """Measured HBM copy bandwidth (GB/s) of the GB300s, or the
    earlier fallback measurement when the driver's file is absent."""
    try:
        with open(ROOT / "MEASURED_PEAKS.json") as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        return 6800.0, "fallback"


def reorder_roofline(n_particles, n_state, ms, n_launches):
    """HBM roofline of the reorder gather (discrete/system.hpp:170-181):
    per particle n_state doubles read and written plus its 4-byte source
    index, over the mean CUDA-event time of one launch.  None when no
    launch was timed (the fused cluster tail)."""
    if n_launches <= 0 or ms <= 0:
        return None
    per_launch = ms / n_launches
    nbytes = n_particles * (16 * n_state + 4)
    achieved = nbytes / (per_launch * 1e-3) / 1e9
    peak, source = hbm_peak()
    return {"bound": "hbm", "kernel": "k_reorder", "bytes_per_launch": nbytes,
            "launch_ms": per_launch, "achieved": achieved, "peak": peak,
            "unit": "GB/s", "frac": achieved / peak,
            "peak_source": f"{source} (MEASURED_PEAKS.json hbm_gbs: "
                           "a STREAM-style copy)"}


def pipe_roofline(workload, units_per_s, peak_tflops):
    """Useful FP64-pipe thread instructions per second against the pipe's
    peak (peak DFMA flops / 2)."""
    n = FP64_PIPE_INST_PER_UNIT.get(workload)
    if n is None or units_per_s is None:
        return None
    peak = peak_tflops * 1e12 / 2
    return {"inst_per_unit": n, "achieved_inst_per_s": n * units_per_s,
            "peak_inst_per_s": peak, "frac": n * units_per_s / peak}
STEPS_PER_OBS = 4  # dt = 0.25, daily observations


def parse_args():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=20)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", choices=["gb300", "reference"], default="gb300")
    p.add_argument("--workload", default="serve_seir",
                   choices=["sir_batched", "sir_small", "seir_batched",
                            "serve_seir", "ode_batched"])
    p.add_argument("--hbm-budget", type=float, default=16e9,
                   help="device memory budget of the likelihood server")
    p.add_argument("--ode-instances", type=int, default=262144,
                   help="instances of the dopri5 workload (smaller cases "
                        "for profiling)")
    p.add_argument("--no-cpu-baseline", action="store_true")
    p.add_argument("--cpu-seconds", type=float, default=12.0,
                   help="target CPU time of the bounded CPU sample")
    p.add_argument("--step-shape", default=None,
                   help="filter workloads: force the step kernel's launch "
                        "shape, block,per_tile,persistent (e.g. 64,0,0), "
                        "instead of the autotuner's choice")
    return p.parse_args()


def dist_info():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", str(rank)))
    return rank, world, local


class ClockSampler:
    """nvidia-smi clocks and throttle reasons during the timed region."""

    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,"
             "clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
             "clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,"
             "clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.gpu_index = gpu_index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--query-gpu={self.QUERY}", "--format=csv,"
                 "noheader,nounits", "-lms", "200", "-i", str(self.gpu_index)],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except OSError:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [],
                    "samples": 0}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown",
                 "sw_power_cap"]
        for line in self.lines:
            parts = [x.strip() for x in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx.append(float(parts[2]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": float(np.median(sm)) if sm else None,
                "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def max_over_ranks(x, world, device):
    """The largest value of x over the ranks (the slowest replica's time);
    x itself on one rank."""
    if world <= 1:
        return float(x)
    import torch
    import torch.distributed as dist
    t = torch.tensor([float(x)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def whole_job_rate(units_per_rank, world, seconds_max):
    """Units processed by all replicas per second of the slowest one."""
    return units_per_rank * world / seconds_max


def fp64_peak_tflops():
    """DFMA throughput microbenchmark (FP64 FMA chains, all SMs)."""
    import ctypes
    from dust2_gb300 import _lib
    t = ctypes.c_double()
    _lib.check(_lib.lib().dust2_gb300_fp64_peak(ctypes.byref(t)))
    return t.value


N_STATE = {"sir_cases": 4, "sir": 5, "seir_age": 96}


def build_workload(name, simulate, packer=None):
    from dust2_gb300 import workloads
    if name == "sir_batched":
        w = workloads.sir_batched(simulate, packer=packer)
        w["system"] = "sir_cases"
    elif name == "seir_batched":
        w = workloads.seir_batched(simulate, packer=packer)
        w["system"] = "seir_age"
    else:
        w = workloads.sir_small(simulate, packer=packer)
        w["data"] = w["data"].reshape(-1, 1)
        w["n_particles"] = [w["n_particles"]]
        w["system"] = "sir_cases"
    w["n_state"] = N_STATE[w["system"]]
    return w


def filter_config(args, w, world=1):
    """The config object of both arms of the filter benchmarks."""
    npg = w["n_particles"]
    n_obs = w["times"].size
    return {"workload": args.workload, "system": w["system"],
            "n_groups": len(npg), "n_particles_total": sum(npg),
            "n_observations": n_obs,
            "steps_per_observation": STEPS_PER_OBS,
            "particle_steps_per_step": sum(npg) * n_obs * STEPS_PER_OBS,
            "l2": "flushed (256 MB write) between timed steps",
            "parallelism": f"replicas x{world}"}


def data_columns(w):
    times = w["times"]
    G = len(w["n_particles"])
    cols = {"time": np.repeat(times, G), "incidence": w["data"].ravel()}
    if G > 1:
        cols["group"] = np.tile(np.arange(1, G + 1), times.size)
    return cols


def run_cpu(w, n_groups, n_threads, n_runs=1):
    """Run the CPU oracle on the first n_groups groups of the workload;
    returns (seconds per run, particle-steps per run).  Inputs are packed
    and seeded by the oracle itself."""
    from oracle import pyoracle
    port = pyoracle.port_timing()
    npg = w["n_particles"][:n_groups]
    G_all = len(w["n_particles"])
    npar = np.asarray(w["pars"]).size // G_all
    pars = np.asarray(w["pars"]).reshape(G_all, npar)[:n_groups].ravel()
    data = np.asarray(w["data"]).reshape(w["times"].size, G_all)[:, :n_groups]
    n_streams = sum(n + 2 for n in npg)
    rng = pyoracle.rng_streams(n_streams, w["seed"])
    t0 = time.perf_counter()
    port.filter_run(w["system"], pars, npg, 0.0, w["times"], data.ravel(),
                    n_groups, w["dt"], rng, n_runs=n_runs,
                    n_state=w["n_state"], n_threads=n_threads)
    dt = (time.perf_counter() - t0) / n_runs
    ps = sum(npg) * w["times"].size * STEPS_PER_OBS
    return dt, ps


def cpu_sample_groups(w, target_seconds, threads):
    """How many leading groups of the workload take about target_seconds
    on the CPU (calibrated on the first group)."""
    t1, ps1 = run_cpu(w, 1, threads)
    rate = ps1 / max(t1, 1e-9)
    G = len(w["n_particles"])
    n_groups = 1
    total = ps1
    per_group = [n * w["times"].size * STEPS_PER_OBS for n in w["n_particles"]]
    while n_groups < G and total / rate < target_seconds:
        total += per_group[n_groups]
        n_groups += 1
    return n_groups


def cpu_sample_text(w, n_groups):
    G = len(w["n_particles"])
    return (f"groups 1-{n_groups} of {G} ({sum(w['n_particles'][:n_groups])}"
            f" particles), all {w['times'].size} observations, one "
            "likelihood evaluation")


def cpu_baseline(w, target_seconds):
    from oracle import pyoracle
    threads = pyoracle.port_timing().max_threads()
    n_groups = cpu_sample_groups(w, target_seconds, threads)
    t, ps = run_cpu(w, n_groups, threads)
    return {"value": ps / t, "unit": "particle-steps/s", "cores": threads,
            "kind": "port", "sample": cpu_sample_text(w, n_groups),
            "seconds": t, "math": CPU_MATH}


def gpu_simulate_factory():
    import dust2_gb300 as d
    from dust2_gb300 import _lib

    def simulate(name, flat, n_groups, n_particles, dt, seed, times):
        import ctypes
        flat = _lib.as_f64(flat)
        times = _lib.as_f64(times)
        words = np.array([seed], dtype=np.uint64)
        h = ctypes.c_void_p()
        _lib.check(_lib.lib().dust2_gb300_system_alloc(
            name.encode(), _lib.dptr(flat), n_groups, n_particles, 0.0, dt,
            None, _lib.uptr(words), 1, 0, ctypes.byref(h)))
        try:
            _lib.check(_lib.lib().dust2_gb300_system_set_state_initial(h))
            n_state = N_STATE[name]
            out = np.empty(times.size * n_groups * n_particles * n_state)
            _lib.check(_lib.lib().dust2_gb300_system_simulate(
                h, _lib.dptr(times), times.size, None, 0, _lib.dptr(out)))
        finally:
            _lib.lib().dust2_gb300_system_free(h)
        return out
    return simulate


def gpu_arm(args, rank, world, local):
    import ctypes

    import torch
    import torch.distributed as dist

    torch.cuda.set_device(local)
    if world > 1:
        dist.init_process_group("nccl" if torch.cuda.is_available() else
                                "gloo")
    import __graft_entry__
    __graft_entry__.build()
    import dust2_gb300 as d
    from dust2_gb300 import _lib

    w = build_workload(args.workload, gpu_simulate_factory())
    gen = d.Generator(w["system"])
    npg = w["n_particles"]
    obj = d.dust_filter_create(gen, 0, data_columns(w),
                               n_particles=npg if len(npg) > 1 else npg[0],
                               dt=w["dt"], seed=w["seed"])
    plist = w["plist"] if len(npg) > 1 else w["plist"][0]
    if args.step_shape:
        b, pt, pe = (int(x) for x in args.step_shape.split(","))
        d.dust_likelihood_set_step_shape(obj, b, pt, bool(pe))
    d.dust_likelihood_run(obj, plist)  # allocate and initialise
    lib = _lib.lib()
    h = obj.ptr
    n_total = sum(npg)
    n_obs = w["times"].size
    n_groups = len(npg)
    particle_steps = n_total * n_obs * STEPS_PER_OBS
    ll = np.empty(n_groups)

    stream_ptr = ctypes.c_void_p()
    _lib.check(lib.dust2_gb300_filter_stream(h, ctypes.byref(stream_ptr)))
    ext = torch.cuda.ExternalStream(stream_ptr.value)
    flush = torch.empty(256 * 1024 * 1024, dtype=torch.uint8, device="cuda")

    def run_once():
        _lib.check(lib.dust2_gb300_filter_run_async(h, None, 0))

    for _ in range(args.warmup):
        run_once()
        _lib.check(lib.dust2_gb300_filter_last_log_likelihood(h,
                                                              _lib.dptr(ll)))

    # the timed runs replay the run's plain graph (captured by the first
    # run above); the step kernel's own times come from separate runs
    # below, because the CUDA events recorded around every step launch
    # lengthen a run (by ~7 us per data time for the 1000-particle filter)
    clocks = ClockSampler(local)
    clocks.start()
    time.sleep(0.5)
    if world > 1:
        dist.barrier()
    torch.cuda.synchronize()
    elapsed = []
    for _ in range(args.steps):
        flush.zero_()
        torch.cuda.synchronize()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(ext)
        run_once()
        e1.record(ext)
        _lib.check(lib.dust2_gb300_filter_last_log_likelihood(
            h, _lib.dptr(ll)))
        elapsed.append(e0.elapsed_time(e1))
    torch.cuda.synchronize()
    if world > 1:
        dist.barrier()
    clock_info = clocks.stop()

    # the same runs with events around each step launch inside the graph
    _lib.check(lib.dust2_gb300_filter_set_timing(h, 1))
    run_once()  # capture the instrumented graph
    _lib.check(lib.dust2_gb300_filter_last_log_likelihood(h, _lib.dptr(ll)))
    _lib.check(lib.dust2_gb300_filter_set_timing(h, 1))  # reset the sums
    for _ in range(args.steps):
        flush.zero_()
        torch.cuda.synchronize()
        run_once()
        _lib.check(lib.dust2_gb300_filter_last_log_likelihood(
            h, _lib.dptr(ll)))
    step_ms = ctypes.c_double()
    run_ms = ctypes.c_double()
    n_step = ctypes.c_int64()
    n_run = ctypes.c_int64()
    _lib.check(lib.dust2_gb300_filter_kernel_times(
        h, ctypes.byref(step_ms), ctypes.byref(n_step), ctypes.byref(run_ms),
        ctypes.byref(n_run)))
    reorder_ms = ctypes.c_double()
    n_reorder = ctypes.c_int64()
    _lib.check(lib.dust2_gb300_filter_reorder_times(
        h, ctypes.byref(reorder_ms), ctypes.byref(n_reorder)))
    _lib.check(lib.dust2_gb300_filter_set_timing(h, 0))
    ms = float(np.mean(elapsed))
    ms_max = max_over_ranks(ms, world, "cuda")
    value = whole_job_rate(particle_steps, world, ms_max * 1e-3)

    # end to end through the public API: host parameters in, host
    # log-likelihoods out, every step (after one untimed run that
    # re-captures the plain graph, which switching timing off discarded)
    d.dust_likelihood_run(obj, plist)
    e2e_times = []
    for _ in range(args.steps):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        res = d.dust_likelihood_run(obj, plist)
        e2e_times.append(time.perf_counter() - t0)
    assert np.all(np.isfinite(res))
    e2e_s = float(np.mean(e2e_times))
    e2e_max = max_over_ranks(e2e_s, world, "cuda")
    h2d = n_groups * gen.n_pars * 8
    d2h = n_groups * 8 + n_groups * 4 + 4

    step_launch_ms = step_ms.value / max(1, n_step.value)
    roofline = None
    if rank == 0:
        peak = fp64_peak_tflops()
        ps_per_launch = n_total * STEPS_PER_OBS
        achieved = None
        frac = None
        ops = FP64_OPS_PER_PARTICLE_STEP.get(args.workload)
        if ops is not None:
            achieved = (ops * ps_per_launch / (step_launch_ms * 1e-3) / 1e12)
            frac = achieved / peak
        roofline = {
            "bound": "fp64", "kernel": f"k_step_compare<{w['system']}>",
            "achieved": achieved, "peak": peak, "unit": "TFLOP/s",
            "frac": frac,
            "traffic": traffic_per_launch(args.workload, ps_per_launch),
            "traffic_source": "ncu dram__bytes_read.sum + "
                              "dram__bytes_write.sum per particle-step of "
                              "this kernel (DRAM_BYTES_PER_UNIT), times the "
                              "particle-steps of one launch",
            "peak_source": "measured in-process: DFMA-chain microbenchmark "
                           "(dust2_gb300_fp64_peak); MEASURED_PEAKS.json has no FP64 entry",
            "step_launch_ms": step_launch_ms,
            "fp64_pipe": pipe_roofline(
                args.workload, ps_per_launch / (step_launch_ms * 1e-3), peak),
            "fp64_formulation": formulation_roofline(
                args.workload, ps_per_launch / (step_launch_ms * 1e-3), peak),
            "fp64_algorithmic": algorithmic_roofline(
                args.workload, ps_per_launch / (step_launch_ms * 1e-3), peak),
            "step_share_of_run": step_ms.value / max(run_ms.value, 1e-12),
            "flops_basis": "executed FP64 ops per particle-step (ncu SASS "
                           "dadd+dmul+2*dfma)"}

    if rank == 0:
        line = {
            "metric": "filter particle-steps/s",
            "value": value, "unit": "particle-steps/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": ms_max, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic (simulated by the model, seeded)",
            "config": filter_config(args, w, world),
            "e2e": {"value": particle_steps * world / e2e_max,
                    "unit": "particle-steps/s", "h2d_bytes_per_step": h2d,
                    "d2h_bytes_per_step": d2h, "seconds_per_step": e2e_max},
            # per observation: the step kernel and the tail, which is one
            # cluster launch when every group has <= 1024 particles, else
            # weights, group, resample, fallback and reorder
            "gpu_launches": args.steps * (
                2 + (2 if max(npg) <= 1024 else 6) * n_obs),
            "clocks": clock_info,
            "roofline": roofline,
            "serial_fallbacks": d.dust_likelihood_serial_fallbacks(obj),
            # the step kernel's launch shape chosen by the autotuner
            "step_shape": d.dust_likelihood_step_shape(obj),
            "reorder_roofline": reorder_roofline(
                n_total, w["n_state"], reorder_ms.value, n_reorder.value),
        }
        if world == 1 and not args.no_cpu_baseline:
            line["cpu_baseline"] = cpu_baseline(w, args.cpu_seconds)
        print(json.dumps(line), flush=True)
    if world > 1:
        dist.destroy_process_group()


def percentile(x, q):
    return float(np.percentile(np.asarray(x, dtype=float), q))


# A step of the serving benchmark is this many likelihood requests; they
# are spread over the clients in turn, so 20 steps give each of the 64
# clients 5 requests.
REQUESTS_PER_STEP = 16
SERVE_METRIC = ("filter particle-steps/s and p50/p99 latency, served vs "
                "plain GPU")


def serve_workload(simulate, steps, packer=None):
    """The serving workload with REQUESTS_PER_STEP * steps requests:
    client i makes counts[i] of them (the first clients one more when
    they do not divide evenly)."""
    from dust2_gb300 import workloads
    n_clients = 64
    base, extra = divmod(REQUESTS_PER_STEP * steps, n_clients)
    counts = [base + (1 if i < extra else 0) for i in range(n_clients)]
    w = workloads.serving_clients(simulate, n_clients=n_clients,
                                  rounds=max(1, max(counts)), packer=packer)
    w["counts"] = counts
    w["particle_steps"] = sum(n * c["particle_steps"]
                              for n, c in zip(counts, w["clients"]))
    return w


def serve_config(args, w, world=1):
    """The config object of both arms of the serving benchmark (with
    `world` replicas, one server per GPU)."""
    clients = w["clients"]
    return {"workload": "serve_seir", "system": "seir_age (16 ages, 96 "
            "states, dt 0.25, negative-binomial compare)",
            "clients": len(clients), "requests": sum(w["counts"]),
            "requests_per_step": REQUESTS_PER_STEP,
            "requests_per_client": [min(w["counts"]), max(w["counts"])],
            "arrival_rate_per_s": w["rate"],
            "particles": [c["n_particles"] for c in clients],
            "days": [int(c["data"]["time"].size) for c in clients],
            "particle_steps": w["particle_steps"],
            "hbm_budget_bytes": args.hbm_budget,
            "l2": "not flushed: a continuous request stream; each "
                  "request's state (0.4-50 MB) is resident between requests",
            "parallelism": f"replicas x{world}, one server per GPU"}


def seir_device_rate(simulate, n_obs=365):
    """Particle-steps/s of the plain filter when it fills the device: 32
    SEIR groups x 8192 particles (the batched SEIR workload) over its
    whole 365 observations (the cost of a step depends on the epidemic's
    phase, so a prefix would overstate it), through
    dust_likelihood_run."""
    import dust2_gb300 as d
    from dust2_gb300 import workloads
    w = workloads.seir_batched(simulate, n_obs=n_obs)
    w["system"] = "seir_age"
    obj = d.dust_filter_create(d.seir_age(), 0, data_columns(w),
                               n_particles=w["n_particles"], dt=w["dt"],
                               seed=w["seed"])
    d.dust_likelihood_run(obj, w["plist"])
    t0 = time.perf_counter()
    d.dust_likelihood_run(obj, w["plist"])
    seconds = time.perf_counter() - t0
    ps = sum(w["n_particles"]) * n_obs * STEPS_PER_OBS
    return {"value": ps / seconds, "unit": "particle-steps/s",
            "workload": f"seir_age 32 groups x 8192 particles, "
                        f"{n_obs} observations, dust_likelihood_run"}


def serve_arm(args, rank, world, local):
    """Served likelihoods vs the plain path on the serving workload.

    64 clients (MCMC chains) each keep one request outstanding: the first
    requests arrive as a Poisson stream at 200/s, and after each result a
    client waits an exponential think time before its next request.  A
    benchmark step is REQUESTS_PER_STEP requests.

    Served: every client's session is open on one likelihood server, and
    each client thread submits and waits in real time.  Plain: the same
    requests, submitted in real time by the same client threads, run one
    by one in arrival order by a single executor thread through
    dust_likelihood_run on one-group filters (one per client).  Latency
    is submit to result on both arms, and both include host parameters
    in and host log-likelihoods out.  The plain arm's per-request rate is
    compared with the device's full rate on this system (the batched SEIR
    filter) to bound what any batching can gain over it.

    Under torchrun every rank is an independent replica (its own server
    and plain executor on its own GPU, the same request stream): both
    arms start after a barrier, their times are the slowest rank's, and
    rates count the requests of all ranks."""
    import queue

    import torch
    import torch.distributed as dist
    torch.cuda.set_device(local)
    if world > 1:
        dist.init_process_group("nccl")
    import __graft_entry__
    __graft_entry__.build()
    import dust2_gb300 as d

    simulate = gpu_simulate_factory()
    w = serve_workload(simulate, args.steps)
    clients = w["clients"]
    counts = w["counts"]
    C = len(clients)
    total_ps = w["particle_steps"]
    gen = d.seir_age()
    c0 = clients[0]

    clocks = ClockSampler(local)
    clocks.start()

    # served arm
    server = d.dust_likelihood_server(gen, hbm_budget=args.hbm_budget,
                                      max_sessions=2 * C)
    warm = server.open(c0["pars"][0], c0["data"], 512, dt=w["dt"], seed=1)
    for _ in range(args.warmup):
        server.likelihood(warm, c0["pars"][0])
    server.close(warm)
    ids = [server.open(c["pars"][0], c["data"], c["n_particles"], dt=w["dt"],
                       seed=c["seed"]) for c in clients]
    server.set_timing(True)
    st0 = server.stats()
    served_ll = [[None] * n for n in counts]
    served_lat = []
    lock = threading.Lock()
    torch.cuda.synchronize()
    if world > 1:
        dist.barrier()
    t0 = time.perf_counter()
    t_end = [t0] * C

    def served_client(i):
        c = clients[i]
        delay = t0 + w["first_arrival"][i] - time.perf_counter()
        if delay > 0:
            time.sleep(delay)
        for r in range(counts[i]):
            ticket = server.submit(ids[i], c["pars"][r])
            ll, lat = server.wait(ticket)
            with lock:
                served_ll[i][r] = ll
                served_lat.append(lat)
            t_end[i] = time.perf_counter()
            if r + 1 < counts[i]:
                time.sleep(w["think"][i, r])

    threads = [threading.Thread(target=served_client, args=(i,))
               for i in range(C)]
    for th in threads:
        th.start()
    for th in threads:
        th.join()
    served_s = max_over_ranks(max(t_end) - t0, world, "cuda")
    st = server.stats()
    served_value = world * total_ps / served_s
    step_ms = st["step_kernel_ms"] - st0["step_kernel_ms"]
    launches = int(st["kernel_launches"] - st0["kernel_launches"])
    server_info = {k: st[k] for k in ("device_steps", "requests_done",
                                      "max_running", "particle_capacity")}
    server.free()

    # plain arm: one filter per client, one executor
    objs = [d.dust_filter_create(gen, 0, c["data"],
                                 n_particles=c["n_particles"], dt=w["dt"],
                                 seed=c["seed"]) for c in clients]
    wobj = d.dust_filter_create(gen, 0, c0["data"], n_particles=512,
                                dt=w["dt"], seed=1)
    for _ in range(args.warmup):
        d.dust_likelihood_run(wobj, c0["pars"][0])
    for i, c in enumerate(clients):
        if counts[i] > 0:
            # allocate each filter and capture its graph before the timed
            # region, then put its generators back where they started, so
            # that its requests see the streams the served session sees
            words = d.dust_likelihood_rng_state(objs[i])
            d.dust_likelihood_run(objs[i], c["pars"][0])
            d.dust_likelihood_set_rng_state(objs[i], words)
    plain_ll = [[None] * n for n in counts]
    plain_lat = []
    service = []  # (particle-steps, seconds) per request
    todo = queue.Queue()
    n_requests = sum(counts)
    torch.cuda.synchronize()
    if world > 1:
        dist.barrier()
    t0 = time.perf_counter()
    t_end = [t0] * C

    def executor():
        for _ in range(n_requests):
            i, r, box = todo.get()
            a = time.perf_counter()
            ll = d.dust_likelihood_run(objs[i], clients[i]["pars"][r])
            b = time.perf_counter()
            box["ll"] = float(np.ravel(ll)[0])
            service.append((clients[i]["particle_steps"], b - a))
            box["done"].set()

    def plain_client(i):
        delay = t0 + w["first_arrival"][i] - time.perf_counter()
        if delay > 0:
            time.sleep(delay)
        for r in range(counts[i]):
            box = {"done": threading.Event()}
            submitted = time.perf_counter()
            todo.put((i, r, box))
            box["done"].wait()
            done = time.perf_counter()
            with lock:
                plain_ll[i][r] = box["ll"]
                plain_lat.append(done - submitted)
            t_end[i] = done
            if r + 1 < counts[i]:
                time.sleep(w["think"][i, r])

    ex = threading.Thread(target=executor)
    ex.start()
    threads = [threading.Thread(target=plain_client, args=(i,))
               for i in range(C)]
    for th in threads:
        th.start()
    for th in threads:
        th.join()
    ex.join()
    plain_s = max_over_ranks(max(t_end) - t0, world, "cuda")
    clock_info = clocks.stop()
    plain_value = world * total_ps / plain_s
    same = all(np.array_equal(np.array(a, dtype=float),
                              np.array(b, dtype=float))
               for a, b in zip(served_ll, plain_ll))

    # the device's full rate on this system, and each plain request's
    # share of it
    dev = seir_device_rate(simulate)
    rate = np.array([ps / s for ps, s in service])
    util = rate / dev["value"]
    busy = sum(ps for ps, _ in service) / sum(s for _, s in service)
    weighted = busy / dev["value"]

    ops = FP64_OPS_PER_PARTICLE_STEP.get("seir_batched")
    peak = fp64_peak_tflops()
    in_kernel_rate = total_ps / (step_ms * 1e-3) if step_ms > 0 else None
    achieved = (ops * in_kernel_rate / 1e12
                if ops is not None and in_kernel_rate else None)
    n_par = gen.n_pars
    line = {
        "metric": SERVE_METRIC,
        "value": served_value, "unit": "particle-steps/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": served_s * 1e3 / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f64",
        "data": "synthetic (simulated by the model, seeded)",
        "config": serve_config(args, w, world),
        "latency_s": {"served": {"p50": percentile(served_lat, 50),
                                 "p99": percentile(served_lat, 99)},
                      "plain": {"p50": percentile(plain_lat, 50),
                                "p99": percentile(plain_lat, 99)}},
        "plain": {"value": plain_value, "unit": "particle-steps/s",
                  "seconds": plain_s, "busy_rate": busy,
                  "mean_service_s": float(np.mean([s for _, s in service]))},
        "served": {"value": served_value, "seconds": served_s,
                   "in_step_kernel_rate": in_kernel_rate},
        "served_over_plain": served_value / plain_value,
        "results_equal_plain": bool(same),
        "device_rate": dev,
        "plain_utilisation": {
            "weighted": weighted,
            "p10": percentile(util, 10), "p50": percentile(util, 50),
            "p90": percentile(util, 90),
            "note": "each plain request's particle-steps/s over the "
                    "device rate; weighted = all plain particle-steps "
                    "over all plain service time, over the device rate"},
        "served_over_plain_bound": 1.0 / weighted,
        "served_over_device_rate": served_value / dev["value"],
        "server": server_info,
        "e2e": {"value": served_value, "unit": "particle-steps/s",
                "h2d_bytes_per_step": REQUESTS_PER_STEP * n_par * 8,
                "d2h_bytes_per_step": REQUESTS_PER_STEP * 8,
                "note": "the served value is already end to end: clients "
                        "submit host parameters and read host "
                        "log-likelihoods through the server's C ABI"},
        "gpu_launches": launches,
        "clocks": clock_info,
        "roofline": {
            "bound": "fp64", "kernel": "k_served_step_compare<seir_age>",
            "achieved": achieved, "peak": peak, "unit": "TFLOP/s",
            "frac": None if achieved is None else achieved / peak,
            "traffic": traffic_per_launch(
                "seir_batched",
                total_ps / max(1, server_info["device_steps"])),
            "traffic_source": "ncu dram bytes per particle-step of the SEIR "
                              "step kernel (batched SEIR filter) times the "
                              "mean particle-steps of one tick",
            "peak_source": "measured in-process: DFMA-chain microbenchmark "
                           "(dust2_gb300_fp64_peak); MEASURED_PEAKS.json "
                           "has no FP64 entry",
            "step_kernel_share": step_ms * 1e-3 / served_s,
            "fp64_pipe": pipe_roofline("seir_batched", in_kernel_rate, peak),
            "fp64_formulation": formulation_roofline("seir_batched",
                                                     in_kernel_rate, peak),
            "fp64_algorithmic": algorithmic_roofline("seir_batched",
                                                     in_kernel_rate, peak),
            "flops_basis": "executed FP64 ops per particle-step of the "
                           "SEIR step kernel (ncu SASS dadd+dmul+2*dfma)"},
    }
    if world == 1 and not args.no_cpu_baseline:
        line["cpu_baseline"] = serve_cpu_baseline(w, args.cpu_seconds)
    if rank == 0:
        print(json.dumps(line), flush=True)
    if world > 1:
        dist.destroy_process_group()


def ode_alloc(w, seed=1):
    """The batched sirode system through the C ABI (one group per
    instance, rtol = atol = 1e-6)."""
    import ctypes
    from dust2_gb300 import _lib
    ctl = _lib.OdeControl(10000, 1e-6, 1e-6, float(np.finfo(float).eps),
                          float("inf"), None, 0, 0)
    pars = _lib.as_f64(w["pars"])
    words = np.array([seed], dtype=np.uint64)
    h = ctypes.c_void_p()
    _lib.check(_lib.lib().dust2_gb300_system_alloc(
        b"sirode", _lib.dptr(pars), w["n_groups"], 1, 0.0, 1.0,
        ctypes.byref(ctl), _lib.uptr(words), 1, 0, ctypes.byref(h)))
    return h


def ode_cpu(w, n_inst, threads):
    from oracle import pyoracle
    port = pyoracle.port_timing()
    gen_pars = 4
    pars = np.asarray(w["pars"]).reshape(-1, gen_pars)[:n_inst].ravel()
    t0 = time.perf_counter()
    _, stats = port.ode_simulate("sirode", pars, n_inst, 1, 0.0, w["times"],
                                 5, n_threads=threads)
    dt = time.perf_counter() - t0
    return dt, int(stats[:, 0].sum())


def ode_cpu_baseline(w, target_seconds):
    from oracle import pyoracle
    threads = pyoracle.port_timing().max_threads()
    n = 1024
    t, steps = ode_cpu(w, n, threads)
    while t < target_seconds / 4 and n < w["n_groups"]:
        n = min(w["n_groups"], n * 4)
        t, steps = ode_cpu(w, n, threads)
    return {"value": steps / t, "unit": "dopri5 steps/s", "cores": threads,
            "kind": "port", "math": CPU_MATH,
            "sample": f"instances 1-{n} of {w['n_groups']}, integrated "
                      f"0..200 with {w['times'].size} outputs",
            "seconds": t, "instances": n}


def ode_config(w, world=1):
    """The config object of both arms of the dopri5 benchmark."""
    return {"workload": "ode_batched", "system": "sirode",
            "instances": w["n_groups"], "outputs": int(w["times"].size),
            "rtol": 1e-6, "atol": 1e-6,
            "l2": "flushed (256 MB write) between timed steps; outputs "
                  f"{w['n_groups'] * w['times'].size * 40 / 1e9:.1f} GB",
            "parallelism": f"replicas x{world}"}


def ode_arm(args, rank, world, local):
    """Batched dopri5: 262,144 sirode instances integrated 0..200 with
    output at every integer time (rtol = atol = 1e-6).  A step of the
    benchmark is one simulate of every instance from t = 0; the metric
    counts attempted dopri5 steps (accepted + rejected) per second.
    Under torchrun every rank integrates its own copy (replicas): timed
    steps start after a barrier and the slowest rank's time counts."""
    import ctypes

    import torch
    import torch.distributed as dist
    torch.cuda.set_device(local)
    if world > 1:
        dist.init_process_group("nccl")
    import __graft_entry__
    __graft_entry__.build()
    from dust2_gb300 import _lib, workloads

    lib = _lib.lib()
    w = workloads.sirode_batched(n_instances=args.ode_instances)
    G = w["n_groups"]
    times = _lib.as_f64(w["times"])
    h = ode_alloc(w)
    n_out = times.size * G * 5
    out = torch.empty(n_out, dtype=torch.float64, device="cuda")
    stream_ptr = ctypes.c_void_p()
    _lib.check(lib.dust2_gb300_system_stream(h, ctypes.byref(stream_ptr)))
    ext = torch.cuda.ExternalStream(stream_ptr.value)
    flush = torch.empty(256 * 1024 * 1024, dtype=torch.uint8, device="cuda")

    def run_once(device=True, host_out=None):
        _lib.check(lib.dust2_gb300_system_set_time(h, 0.0))
        _lib.check(lib.dust2_gb300_system_set_state_initial(h))
        if device:
            _lib.check(lib.dust2_gb300_system_simulate_device(
                h, _lib.dptr(times), times.size,
                ctypes.c_void_p(out.data_ptr())))
        else:
            _lib.check(lib.dust2_gb300_system_simulate(
                h, _lib.dptr(times), times.size, None, 0,
                _lib.dptr(host_out)))

    for _ in range(args.warmup):
        run_once()
    ns = np.zeros(G, dtype=np.int64)
    na = np.zeros(G, dtype=np.int64)
    nr = np.zeros(G, dtype=np.int64)
    ss = np.zeros(G)
    er = np.zeros(G)
    _lib.check(lib.dust2_gb300_system_internals(
        h, _lib.dptr(ss), _lib.dptr(er), ns.ctypes.data_as(_lib.c_i64_p),
        na.ctypes.data_as(_lib.c_i64_p), nr.ctypes.data_as(_lib.c_i64_p)))
    steps = int(ns.sum())
    clocks = ClockSampler(local)
    clocks.start()
    time.sleep(0.5)
    elapsed = []
    if world > 1:
        dist.barrier()
    for _ in range(args.steps):
        flush.zero_()
        torch.cuda.synchronize()
        _lib.check(lib.dust2_gb300_system_set_time(h, 0.0))
        _lib.check(lib.dust2_gb300_system_set_state_initial(h))
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(ext)
        _lib.check(lib.dust2_gb300_system_simulate_device(
            h, _lib.dptr(times), times.size, ctypes.c_void_p(out.data_ptr())))
        e1.record(ext)
        torch.cuda.synchronize()
        elapsed.append(e0.elapsed_time(e1))
    clock_info = clocks.stop()
    ms = max_over_ranks(float(np.mean(elapsed)), world, "cuda")
    # the caller's output buffer: pinned host memory, as the timing
    # contract's host<->device copies are
    host_t = torch.empty(n_out, dtype=torch.float64, pin_memory=True)
    host = host_t.numpy()
    # one untimed call first, as on the other arms: the first copies into
    # a fresh 2.1 GB host buffer run at 30-45 GB/s (its pages are mapped
    # on first touch) against ~190 GB/s afterwards
    run_once(device=False, host_out=host)
    e2e = []
    for _ in range(args.steps):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        run_once(device=False, host_out=host)
        e2e.append(time.perf_counter() - t0)
    e2e_s = max_over_ranks(float(np.mean(e2e)), world, "cuda")
    peak = fp64_peak_tflops()
    ops = FP64_OPS_PER_PARTICLE_STEP.get("ode_batched")
    achieved = None if ops is None else ops * steps / (ms * 1e-3) / 1e12
    _lib.check(lib.dust2_gb300_system_free(h))
    line = {
        "metric": "dopri5 steps/s", "value": world * steps / (ms * 1e-3),
        "unit": "dopri5 steps/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (seeded parameters)",
        "config": ode_config(w, world),
        "dopri5": {"steps_per_step": steps, "accepted": int(na.sum()),
                   "rejected": int(nr.sum()),
                   "steps_per_instance": [int(ns.min()), int(ns.max())]},
        "e2e": {"value": world * steps / e2e_s, "unit": "dopri5 steps/s",
                "h2d_bytes_per_step": times.size * 8,
                "d2h_bytes_per_step": n_out * 8, "seconds_per_step": e2e_s},
        "gpu_launches": 2 * args.steps,
        "clocks": clock_info,
        "roofline": {"bound": "fp64", "kernel": "k_ode_run<sirode>",
                     "achieved": achieved, "peak": peak, "unit": "TFLOP/s",
                     "frac": None if achieved is None else achieved / peak,
                     "traffic": traffic_per_launch("ode_batched", steps),
                     "fp64_pipe": pipe_roofline("ode_batched",
                                                steps / (ms * 1e-3), peak),
                     "fp64_algorithmic": algorithmic_roofline(
                         "ode_batched", steps / (ms * 1e-3), peak),
                     "flops_basis": "executed FP64 ops per attempted "
                                    "dopri5 step (ncu SASS)"},
    }
    if world == 1 and not args.no_cpu_baseline:
        line["cpu_baseline"] = ode_cpu_baseline(w, args.cpu_seconds)
    if rank == 0:
        print(json.dumps(line), flush=True)
    if world > 1:
        dist.destroy_process_group()


def reference_arm(args, rank, world):
    """The CPU implementation of the path on the host cores (the oracle
    port of dust2's engine; dust2's own sources are not present on the
    benchmark machine).  Inputs are built, packed and seeded by the
    oracle: this arm never loads the CUDA library."""
    if rank != 0:
        return
    from oracle import build as oracle_build
    oracle_build.build_port()
    from oracle import pyoracle

    port = pyoracle.port_timing()
    threads = port.max_threads()
    unit = "particle-steps/s"
    # each of the warmup + steps runs is one sample of about a third of
    # the CPU-baseline target, so that 25 runs take a couple of minutes
    step_seconds = args.cpu_seconds / 3
    if args.workload == "ode_batched":
        from dust2_gb300 import workloads
        w = workloads.sirode_batched(n_instances=args.ode_instances)
        base = ode_cpu_baseline(w, step_seconds)
        n_inst = base["instances"]

        def one():
            return ode_cpu(w, n_inst, threads)
        metric, unit = "dopri5 steps/s", "dopri5 steps/s"
        config = ode_config(w, world)
    elif args.workload == "serve_seir":
        w = serve_workload(oracle_simulate(), args.steps,
                           packer=pyoracle.pack_pars)
        picks, base = serve_cpu_sample(w, step_seconds, threads)

        def one():
            return serve_cpu_run(w, picks, threads)
        metric = SERVE_METRIC
        config = serve_config(args, w, world)
    else:
        w = build_workload(args.workload, oracle_simulate(),
                           packer=pyoracle.pack_pars)
        n_groups = cpu_sample_groups(w, step_seconds, threads)
        base = {"sample": cpu_sample_text(w, n_groups)}

        def one():
            return run_cpu(w, n_groups, threads)
        metric = "filter particle-steps/s"
        config = filter_config(args, w, world)
    for _ in range(args.warmup):
        one()
    times = []
    ps = None
    for _ in range(args.steps):
        t, ps = one()
        times.append(t)
    t = float(np.mean(times))
    value = ps / t
    line = {
        "impl": "reference", "metric": metric,
        "value": value, "unit": unit, "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": t * 1e3,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f64", "data": "synthetic (simulated by the model, seeded)",
        "config": config,
        "cpu_baseline": {"value": value, "unit": unit,
                         "cores": threads, "kind": "port",
                         "sample": base["sample"], "math": CPU_MATH},
        "e2e": {"value": value, "unit": unit,
                "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "native_so_loaded": native_library_loaded(),
    }
    print(json.dumps(line), flush=True)


def native_library_loaded():
    """Whether this process has mapped the CUDA engine's library."""
    try:
        with open("/proc/self/maps") as f:
            return "libdust2_gb300" in f.read()
    except OSError:
        return None


def serve_cpu_inputs(w, picks):
    """Packed parameters, data and generator words of requests (client,
    request) of the serving workload, built by the oracle."""
    from oracle import pyoracle
    out = []
    for i, r in picks:
        c = w["clients"][i]
        n = c["n_particles"]
        out.append((pyoracle.pack_pars("seir_age", c["pars"][r]),
                    np.asarray(c["data"]["incidence"], dtype=float),
                    c["data"]["time"], n,
                    pyoracle.rng_streams(n + 2, c["seed"]),
                    c["particle_steps"]))
    return out


def serve_cpu_run(w, picks, threads):
    """Requests (client, request) of the serving workload, one by one, on
    the CPU oracle (the reference's engine restated; OpenMP over
    particles); returns (seconds, particle-steps)."""
    from oracle import pyoracle
    port = pyoracle.port_timing()
    inputs = serve_cpu_inputs(w, picks)
    total = 0
    t0 = time.perf_counter()
    for pars, data, times, n, rng, ps in inputs:
        port.filter_run("seir_age", pars, [n], 0.0, times, data, 1, w["dt"],
                        rng, n_runs=1, n_state=96, n_threads=threads)
        total += ps
    return time.perf_counter() - t0, total


def serve_cpu_sample(w, target_seconds, threads):
    """The first requests of the clients, in order, that take about
    target_seconds on the CPU (calibrated on the first)."""
    t, ps = serve_cpu_run(w, [(0, 0)], threads)
    rate = ps / max(t, 1e-9)
    picks, total = [(0, 0)], ps
    for i in range(1, len(w["clients"])):
        if total / rate >= target_seconds:
            break
        picks.append((i, 0))
        total += w["clients"][i]["particle_steps"]
    base = {"sample": f"first requests of clients 1-{len(picks)} of "
                      f"{len(w['clients'])}, one by one"}
    return picks, base


def serve_cpu_baseline(w, target_seconds):
    from oracle import pyoracle
    threads = pyoracle.port_timing().max_threads()
    picks, base = serve_cpu_sample(w, target_seconds, threads)
    t, ps = serve_cpu_run(w, picks, threads)
    return {"value": ps / t, "unit": "particle-steps/s", "cores": threads,
            "kind": "port", "sample": base["sample"], "seconds": t,
            "math": CPU_MATH}


def oracle_simulate():
    from oracle import pyoracle

    def simulate(name, flat, n_groups, n_particles, dt, seed, times):
        rng = pyoracle.rng_streams(n_groups * n_particles, seed)
        out, _ = pyoracle.port().discrete_simulate(
            name, flat, n_groups, n_particles, 0.0, dt, rng, times)
        n_state = N_STATE[name]
        return out[:times.size * n_groups * n_particles * n_state]
    return simulate


def main():
    args = parse_args()
    rank, world, local = dist_info()
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        reference_arm(args, rank, world)
    elif args.workload == "serve_seir":
        serve_arm(args, rank, world, local)
    elif args.workload == "ode_batched":
        ode_arm(args, rank, world, local)
    else:
        gpu_arm(args, rank, world, local)


if __name__ == "__main__":
    main()
