"""The reference arm of bench.py on CPU: the oracle's timing build runs the
default workload's metric on a bounded sample and prints the one JSON line
of the benchmark contract, with `impl`, `cpu_baseline` and a zero-copy
`e2e`."""
import json
import pathlib
import subprocess
import sys

import numpy as np

import bench
from oracle import pyoracle

ROOT = pathlib.Path(__file__).resolve().parent.parent


def test_reference_arm_prints_contract_line():
    res = subprocess.run(
        [sys.executable, str(ROOT / "bench.py"), "--impl", "reference",
         "--steps", "1", "--warmup", "3", "--cpu-seconds", "0.3"],
        capture_output=True, text=True, timeout=600, cwd=ROOT)
    assert res.returncode == 0, res.stderr[-2000:]
    lines = [x for x in res.stdout.splitlines() if x.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference"
    assert d["metric"] == bench.SERVE_METRIC
    assert d["unit"] == "particle-steps/s"
    assert d["higher_is_better"] is True
    assert d["steps"] == 1 and d["warmup"] == 3 and d["n_gpus"] == 1
    assert d["value"] > 0
    assert d["config"]["workload"] == "serve_seir"
    assert d["config"]["requests"] == bench.REQUESTS_PER_STEP
    # the CPU arm builds its inputs with the oracle alone
    assert d["native_so_loaded"] is False
    cb = d["cpu_baseline"]
    assert cb["kind"] in ("port", "reference") and cb["cores"] >= 1
    assert cb["value"] == d["value"]
    assert d["e2e"] == {"value": d["value"], "unit": d["unit"],
                        "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}


def test_serving_config_is_the_same_for_both_arms():
    # the GPU arm packs parameters with the library's parameter tables,
    # the CPU arm with the oracle's; the workloads (and so the config
    # objects the two lines print) must be identical
    class Args:
        hbm_budget = 16e9

    sim = bench.oracle_simulate()
    a = bench.serve_workload(sim, 3)
    b = bench.serve_workload(sim, 3, packer=pyoracle.pack_pars)
    assert bench.serve_config(Args, a) == bench.serve_config(Args, b)
    for ca, cb in zip(a["clients"], b["clients"]):
        for pa, pb in zip(ca["pars"], cb["pars"]):
            assert pa.keys() == pb.keys()
    assert sum(a["counts"]) == 3 * bench.REQUESTS_PER_STEP
    # 20 steps give every client 5 requests
    c20 = bench.serve_workload(sim, 20, packer=pyoracle.pack_pars)["counts"]
    assert c20 == [5] * 64


def test_oracle_packing_and_seeding_match_the_library():
    import dust2_gb300 as d
    from dust2_gb300 import workloads
    p = workloads.seir_plist([1.7])[0]
    assert np.array_equal(pyoracle.pack_pars("seir_age", p),
                          d.Generator("seir_age").pack_pars(p),
                          equal_nan=True)
    want = np.frombuffer(d.rng_streams(300, 11005), dtype="<u8")
    assert np.array_equal(pyoracle.rng_streams(300, 11005), want)
