// Deterministic SIR ODE: the GPU restatement of dust2's bundled example
// inst/examples/sirode.cpp (same packing, parameters, rhs, zero_every and
// Poisson compare).
#pragma once

#include "../dust2gpu/system.hpp"

namespace dust2gpu {
namespace systems {

struct sirode {
  static constexpr const char* name = "sirode";
  using real_type = double;
  using rng_state_type = random::rng_state;

  struct shared_state {
    real_type N;
    real_type I0;
    real_type beta;
    real_type gamma;
  };
  struct internal_state {};
  struct data_type {
    real_type incidence;
  };

  static constexpr int n_state_max = 5;
  static constexpr int n_output = 0;

  static constexpr parameter_info parameters[] = {
    {"I0", 1, 10, false, false},
    {"N", 1, 1000, false, true},
    {"beta", 1, 0.2, false, false},
    {"gamma", 1, 0.1, false, false}};
  static constexpr const char* data_names[] = {"incidence"};

  static shared_state build_shared(const double* pars) {
    shared_state s;
    s.I0 = read_par<sirode>(pars, 0);
    s.N = read_par<sirode>(pars, 1);
    s.beta = read_par<sirode>(pars, 2);
    s.gamma = read_par<sirode>(pars, 3);
    return s;
  }

  static void update_shared(const double* pars, shared_state& s) {
    s.I0 = read_par_update<sirode>(pars, 0, s.I0);
    s.beta = read_par_update<sirode>(pars, 2, s.beta);
    s.gamma = read_par_update<sirode>(pars, 3, s.gamma);
  }

  static std::vector<packing_entry> packing_state(const shared_state&) {
    return {{"S", {}}, {"I", {}}, {"R", {}}, {"cases_cumul", {}},
            {"cases_inc", {}}};
  }

  static int n_state(const shared_state&) {
    return 5;
  }

  static zero_every_spec zero_every(const shared_state&) {
    auto z = zero_every_none();
    zero_every_add(z, 1, {4});
    return z;
  }

  static data_type build_data(const double* d) {
    return data_type{d[0]};
  }

  DUST2_HD static void initial(real_type time, const shared_state& shared,
                               internal_state& internal,
                               rng_state_type& rng_state,
                               real_type* state_next) {
    state_next[0] = shared.N - shared.I0;
    state_next[1] = shared.I0;
    state_next[2] = 0;
    state_next[3] = 0;
    state_next[4] = 0;
  }

  DUST2_HD static void rhs(real_type time, const real_type* state,
                           const shared_state& shared,
                           internal_state& internal,
                           real_type* state_deriv) {
    const auto S = state[0];
    const auto I = state[1];
    const auto rate_SI = shared.beta * S * I / shared.N;
    const auto rate_IR = shared.gamma * I;
    state_deriv[0] = -rate_SI;
    state_deriv[1] = rate_SI - rate_IR;
    state_deriv[2] = rate_IR;
    state_deriv[3] = rate_SI;
    state_deriv[4] = rate_SI;
  }

  DUST2_HD static real_type compare_data(const real_type time,
                                         const real_type* state,
                                         const data_type& data,
                                         const shared_state& shared,
                                         internal_state& internal,
                                         rng_state_type& rng_state) {
    if (math::is_nan(data.incidence)) {
      return 0;
    }
    return density::poisson(data.incidence, state[4], true);
  }
};

}  // namespace systems
}  // namespace dust2gpu
