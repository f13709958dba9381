"""The reference arm of bench.py on CPU: the oracle's timing build runs the
default workload's metric on a bounded sample and prints the one JSON line
of the benchmark contract, with `impl`, `cpu_baseline` and a zero-copy
`e2e`."""
import json
import pathlib
import subprocess
import sys

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
    assert d["metric"] == "filter particle-steps/s"
    assert d["unit"] == "particle-steps/s"
    assert d["higher_is_better"] is True
    assert d["steps"] == 1 and d["warmup"] == 3 and d["n_gpus"] == 1
    assert d["value"] > 0
    assert d["config"]["workload"] == "sir_batched"
    cb = d["cpu_baseline"]
    assert cb["kind"] in ("port", "reference") and cb["cores"] >= 1
    assert cb["value"] == d["value"]
    assert d["e2e"] == {"value": d["value"], "unit": d["unit"],
                        "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}
