"""The exact parallel running sum of the serial resampling fallback
(dust2gpu/exact_sum.hpp, kernel exact_running_sums): its window algorithm,
emulated on the CPU over the same integer helpers, reproduces the plain
left-to-right FP64 loop of filter_details.hpp:45-74 bit for bit on 2,000
weight vectors (filter-like, equal, halfway cases, powers of two down to
subnormals, sparse, 10^+-300, overflow to Inf, negative)."""
import pathlib
import shutil
import subprocess

import pytest

ROOT = pathlib.Path(__file__).resolve().parent.parent


def test_exact_running_sum_matches_plain_loop(tmp_path):
    cxx = shutil.which("g++")
    if cxx is None:
        pytest.skip("g++ not available")
    exe = tmp_path / "exact_sum_check"
    subprocess.run(
        [cxx, "-O2", "-std=c++17", "-ffp-contract=off",
         "-I", str(ROOT / "dust2_gb300" / "csrc"),
         str(ROOT / "tests" / "exact_sum_check.cpp"), "-o", str(exe)],
        check=True)
    res = subprocess.run([str(exe)], capture_output=True, text=True,
                         timeout=300)
    assert res.returncode == 0, res.stdout + res.stderr
    fields = res.stdout.split()
    assert fields[0] == "cases" and int(fields[1]) == 2000
    assert fields[2] == "bad" and int(fields[3]) == 0
    # the windows stay few: about one per 128..1024 weights plus the
    # binade crossings
    assert float(fields[5]) < 20


def test_integer_pipe_replacements_match_fp64(tmp_path):
    """The FP64 operations of the samplers done on the integer pipe give
    the FP64 bits: random::centered_uniform (U - 1/2 and 1/2 - |U - 1/2|
    of the BTRS and PTRS attempts), math::floor_bits (std::floor) and
    math::twice_normal (2 x)."""
    cxx = shutil.which("g++")
    if cxx is None:
        pytest.skip("g++ not available")
    exe = tmp_path / "integer_pipe_check"
    subprocess.run(
        [cxx, "-O2", "-std=c++17", "-ffp-contract=off",
         "-I", str(ROOT / "dust2_gb300" / "csrc"),
         str(ROOT / "tests" / "integer_pipe_check.cpp"), "-o", str(exe)],
        check=True)
    res = subprocess.run([str(exe)], capture_output=True, text=True,
                         timeout=300)
    assert res.returncode == 0, res.stdout + res.stderr
    fields = res.stdout.split()
    assert fields[:1] == ["cases"] and int(fields[1]) > 12000000
    assert fields[2] == "bad" and int(fields[3]) == 0
