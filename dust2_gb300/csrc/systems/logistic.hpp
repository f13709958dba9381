// Multi-species logistic growth ODE with an output variable: the GPU
// restatement of dust2's bundled example inst/examples/logistic.cpp
// (packing x[n] + total, where total is an `output` computed from x).
// The vector parameters r and K have a fixed capacity of 8 species.
#pragma once

#include "../dust2gpu/system.hpp"

namespace dust2gpu {
namespace systems {

struct logistic {
  static constexpr const char* name = "logistic";
  using real_type = double;
  using rng_state_type = random::rng_state;
  static constexpr int n_max = 8;

  struct shared_state {
    int n;
    real_type r[n_max];
    real_type K[n_max];
  };
  struct internal_state {};
  struct data_type {};

  static constexpr int n_state_max = n_max + 1;
  static constexpr int n_output = 1;

  static constexpr parameter_info parameters[] = {
    {"n", 1, NAN, true, true},
    {"r", n_max, NAN, true, false},
    {"K", n_max, NAN, true, false}};

  static shared_state build_shared(const double* pars) {
    shared_state s{};
    const double n = read_par<logistic>(pars, 0);
    if (!(n >= 1) || n > n_max || n != std::floor(n)) {
      throw std::runtime_error("'n' must be an integer in [1, 8]");
    }
    s.n = static_cast<int>(n);
    read_par_array<logistic>(pars, 1, s.r, s.n, true);
    read_par_array<logistic>(pars, 2, s.K, s.n, true);
    return s;
  }

  static void update_shared(const double* pars, shared_state& s) {
    read_par_array<logistic>(pars, 1, s.r, s.n, false);
    read_par_array<logistic>(pars, 2, s.K, s.n, false);
  }

  static std::vector<packing_entry> packing_state(const shared_state& s) {
    return {{"x", {s.n}}, {"total", {}}};
  }

  static int n_state(const shared_state& s) {
    return s.n + 1;
  }

  static zero_every_spec zero_every(const shared_state&) {
    return zero_every_none();
  }

  DUST2_HD static void initial(real_type time, const shared_state& shared,
                               internal_state& internal,
                               rng_state_type& rng_state,
                               real_type* state) {
    for (int i = 0; i < shared.n; ++i) {
      state[i] = 1;
    }
  }

  DUST2_HD static void rhs(real_type time, const real_type* state,
                           const shared_state& shared,
                           internal_state& internal,
                           real_type* state_deriv) {
    for (int i = 0; i < shared.n; ++i) {
      state_deriv[i] = shared.r[i] * state[i] * (1 - state[i] / shared.K[i]);
    }
  }

  DUST2_HD static void output(real_type time, real_type* state,
                              const shared_state& shared,
                              internal_state& internal) {
    real_type tot = 0;
    for (int i = 0; i < shared.n; ++i) {
      tot += state[i];
    }
    state[shared.n] = tot;
  }
};

}  // namespace systems
}  // namespace dust2gpu
