"""System classes written for dust2 run on this engine unchanged apart
from DUST2_HD on their device functions (compat/dust2/common.hpp and
compat/plugin.hpp).

On the CPU: dust2's own example (inst/examples/sir.cpp, read in place from
the reference checkout, where there is one) is compiled against the
compat headers with only DUST2_HD inserted, and its trajectories and
compare values are the bits of the engine's native sir system, which
restates that model against the engine's contract.  The same transformed
source also compiles as device code for sm_103a.  The dust2-shaped sirs
system compiled into the library is checked on the GPU in
test_gpu_compat.py."""

import os
import re
import shutil
import subprocess
from pathlib import Path

import numpy as np
import pytest

import __graft_entry__
from oracle import pyoracle

ROOT = Path(__file__).resolve().parent.parent
CSRC = ROOT / "dust2_gb300" / "csrc"


def reference_example(name):
    inc = Path(__graft_entry__.REFERENCE_INCLUDE)
    path = inc.parent / "examples" / name
    if not path.exists():
        pytest.skip("the reference's examples are not present")
    return path.read_text()


def with_device_functions(src):
    """The one change a dust2 class needs: DUST2_HD on the functions the
    engine runs on the device."""
    out, n = re.subn(
        r"\bstatic (void|real_type) (initial|update|compare_data|"
        r"adjoint_\w+)\(", r"DUST2_HD static \1 \2(", src)
    assert n >= 3
    return out


DRIVER = r"""
#include <cstdio>
#include <cstdlib>
#include <vector>
#include "compat/plugin.hpp"
#include "example.cpp"

struct example_spec {
  using system = ::sir;
  static constexpr const char* name = "sir_example";
  static constexpr int n_state_max = 5;
  static constexpr double default_dt = 1;
  static constexpr dust2gpu::parameter_info parameters[] = {
    {"I0", 1, NAN, false, false}, {"N", 1, NAN, false, true},
    {"beta", 1, NAN, false, false}, {"gamma", 1, NAN, false, false},
    {"exp_noise", 1, NAN, false, true}};
  static constexpr const char* data_names[] = {"incidence"};
};
using P = dust2gpu::compat::plugin<example_spec>;

// argv: n_particles n_times steps_per_time dt, then on stdin the
// parameter row (5 doubles), one observed incidence, and 4 generator
// words per particle.  Prints the state after each time and one compare
// value per particle, as 64-bit patterns.
int main(int argc, char** argv) {
  const int np = std::atoi(argv[1]);
  const int nt = std::atoi(argv[2]);
  const int spt = std::atoi(argv[3]);
  const double dt = std::atof(argv[4]);
  double row[5];
  for (auto& x : row) {
    if (std::scanf("%lf", &x) != 1) return 1;
  }
  double obs;
  if (std::scanf("%lf", &obs) != 1) return 1;
  const auto shared = P::build_shared(row);
  const auto z = P::zero_every(shared);
  const double drow[1] = {obs};
  const auto data = dust2gpu::build_data_of<P>(drow, shared);
  const int ns = P::n_state(shared);
  for (int k = 0; k < np; ++k) {
    P::rng_state_type rng{};
    for (int w = 0; w < 4; ++w) {
      unsigned long long v;
      if (std::scanf("%llu", &v) != 1) return 1;
      rng.state[w] = v;
    }
    P::internal_state internal{};
    std::vector<double> x(ns), y(ns);
    P::initial(0, shared, internal, rng, x.data());
    double t = 0;
    for (int i = 0; i < nt; ++i) {
      for (int s = 0; s < spt; ++s) {
        for (int e = 0; e < z.n; ++e) {
          if (std::fmod(t, z.period[e]) == 0) {
            for (int j = 0; j < ns; ++j) {
              if (z.has(e, j)) x[j] = 0;
            }
          }
        }
        P::update(t, dt, x.data(), shared, internal, rng, y.data());
        x.swap(y);
        t = t + dt;
      }
      for (int j = 0; j < ns; ++j) {
        double v = x[j];
        unsigned long long b;
        std::memcpy(&b, &v, 8);
        std::printf("%llu\n", b);
      }
    }
    const double ll = P::compare_data(t, x.data(), data, shared, internal,
                                      rng);
    unsigned long long b;
    std::memcpy(&b, &ll, 8);
    std::printf("c %llu\n", b);
  }
  return 0;
}
"""


@pytest.fixture(scope="module")
def example_binary(tmp_path_factory):
    src = with_device_functions(reference_example("sir.cpp"))
    d = tmp_path_factory.mktemp("compat")
    (d / "example.cpp").write_text(src)
    (d / "driver.cpp").write_text(DRIVER)
    exe = d / "driver"
    res = subprocess.run(
        ["g++", "-std=c++17", "-O2", "-ffp-contract=off", "-include",
         "cstring", "-I", str(d), "-I", str(CSRC), "-I",
         str(CSRC / "compat"), str(d / "driver.cpp"), "-o", str(exe)],
        capture_output=True, text=True)
    assert res.returncode == 0, res.stderr[-3000:]
    return exe


def run_example(exe, pars, n, n_times, dt, obs, words):
    inp = " ".join(repr(float(x)) for x in pars) + f" {obs!r} " + \
        " ".join(str(int(x)) for x in words)
    res = subprocess.run([str(exe), str(n), str(n_times),
                          str(int(round(1 / dt))), repr(dt)], input=inp,
                         capture_output=True, text=True, check=True)
    states, compares = [], []
    for ln in res.stdout.splitlines():
        if ln.startswith("c "):
            compares.append(int(ln[2:]))
        else:
            states.append(int(ln))
    st = np.array(states, dtype=np.uint64).view(np.float64)
    ns = st.size // (n * n_times)
    return (st.reshape(n, n_times, ns).transpose(1, 0, 2),
            np.array(compares, dtype=np.uint64).view(np.float64))


def test_dust2_example_runs_unchanged_and_matches_native_sir(example_binary):
    port = pyoracle.port()
    pars = {"I0": 10, "N": 1000, "beta": 0.3, "gamma": 0.1,
            "exp_noise": 1e6}
    row = pyoracle.pack_pars("sir", pars)
    n, n_times, dt = 40, 30, 0.25
    words = pyoracle.rng_streams(n, 77)
    got, got_cmp = run_example(example_binary, row, n, n_times, dt, 17.0,
                               words)
    times = np.arange(1, n_times + 1, dtype=float)
    want, rng_after = port.discrete_simulate("sir", row, 1, n, 0.0, dt,
                                             words, times)
    want = want[:n_times * n * 5].reshape(n_times, n, 5)
    np.testing.assert_array_equal(got, want)
    # the compare value of each particle after the run, from the same
    # generator state (the example's compare draws exponential noise)
    want_cmp, _ = port.compare("sir", row, 1, n, times[-1],
                               want[-1].ravel(), np.array([17.0]), 1,
                               rng_after)
    np.testing.assert_array_equal(got_cmp, np.ravel(want_cmp))


def test_dust2_example_compiles_as_device_code(tmp_path):
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(nvcc):
        pytest.skip("nvcc not available")
    src = with_device_functions(reference_example("sir.cpp"))
    (tmp_path / "example.cpp").write_text(src)
    (tmp_path / "k.cu").write_text(DRIVER.split("int main")[0] + r"""
__global__ void k_step(const P::shared_state* shared, double* x,
                       unsigned long long* words) {
  P::rng_state_type rng{};
  for (int w = 0; w < 4; ++w) rng.state[w] = words[w];
  P::internal_state internal{};
  double y[5];
  P::update(0, 0.25, x, *shared, internal, rng, y);
  P::data_type d{1};
  x[0] = P::compare_data(0.25, y, d, *shared, internal, rng);
}
""")
    res = subprocess.run(
        [nvcc, "-gencode", "arch=compute_103a,code=sm_103a", "-std=c++17",
         "--expt-relaxed-constexpr", "-fmad=false", "-include", "cstring",
         "-I", str(tmp_path), "-I", str(CSRC), "-I", str(CSRC / "compat"),
         "-c", str(tmp_path / "k.cu"), "-o", str(tmp_path / "k.o")],
        capture_output=True, text=True)
    assert res.returncode == 0, res.stderr[-3000:]
