// The engine's dopri5 solver (dust2_gb300/csrc/engine/dopri5.cuh, host and
// device code) compiled for the host, so that a CPU test can compare the
// GPU's arithmetic -- fused stage sums, controller powers through the
// engine's exp and log, reciprocals for the divisions -- with the
// oracle's restatement of dust2's solver.  host_ode integrates n
// instances of a system from time 0 through `times`, as k_ode_run does
// for one particle each: initialise, then one solver run per output time.
#include <cstdint>
#include <string>

#include "engine/dopri5.cuh"
#include "systems/logistic.hpp"
#include "systems/sirode.hpp"

namespace {

namespace dp = dust2gpu::engine::dopri5;

template <typename T>
int run(const double* pars, int n_pars, int n, const double* times,
        int n_times, double* out, std::int64_t* stats, double ssmin,
        double ssmax, const double* critical, int n_critical) {
  constexpr int NV = T::n_state_max - T::n_output;
  dp::control_dev c{};
  c.max_steps = 10000;
  c.atol = 1e-6;
  c.rtol = 1e-6;
  c.step_size_min = ssmin;
  c.step_size_max = ssmax;
  c.factor_safe = 0.9;
  c.facc1 = 1 / 0.2;
  c.facc2 = 1 / 10.0;
  c.beta = 0.04;
  c.constant = 0.2 - 0.04 * 0.75;
  c.critical = critical;
  c.n_critical = n_critical;
  for (int k = 0; k < n; ++k) {
    const auto sh = T::build_shared(pars + static_cast<long>(k) * n_pars);
    typename T::internal_state internal{};
    const auto z = T::zero_every(sh);
    const int ns = T::n_state(sh);
    double y[T::n_state_max];
    dust2gpu::random::rng_state r{};
    T::initial(0.0, sh, internal, r, y);
    dp::state<NV> st{};
    dp::scratch<NV> s{};
    dp::solver<T, NV> sol{c, sh, internal, ns - T::n_output, k};
    sol.initialise(0.0, y, st, s);
    if (st.err != 0) {
      return st.err;
    }
    double t = 0;
    for (int i = 0; i < n_times; ++i) {
      sol.run(t, times[i], y, z, st, s);
      t = times[i];
      for (int q = 0; q < ns; ++q) {
        out[(static_cast<long>(i) * n + k) * ns + q] = y[q];
      }
    }
    stats[3 * k] = st.n_steps;
    stats[3 * k + 1] = st.n_steps_accepted;
    stats[3 * k + 2] = st.n_steps_rejected;
  }
  return 0;
}

}  // namespace

// The solver's helpers for the CPU tests: t / period as the zero_every
// check computes it, and 1/x as the error norm and controller compute it.
extern "C" double host_div_period(double t, double period) {
  return dp::div_period(t, period);
}

extern "C" double host_recip(double x) {
  return dp::recip(x);
}

extern "C" int host_ode(const char* name, const double* pars, int n_pars,
                        int n, const double* times, int n_times, double* out,
                        std::int64_t* stats, double ssmin, double ssmax,
                        const double* critical, int n_critical) {
  const std::string s(name);
  if (s == "sirode") {
    return run<dust2gpu::systems::sirode>(pars, n_pars, n, times, n_times,
                                          out, stats, ssmin, ssmax, critical,
                                          n_critical);
  }
  if (s == "logistic") {
    return run<dust2gpu::systems::logistic>(pars, n_pars, n, times, n_times,
                                            out, stats, ssmin, ssmax,
                                            critical, n_critical);
  }
  return -1;
}
