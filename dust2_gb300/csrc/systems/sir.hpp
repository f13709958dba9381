// Stochastic SIR with exponential observation noise: the GPU restatement
// of dust2's bundled example inst/examples/sir.cpp (same state packing,
// parameters, defaults, draw order and compare).
#pragma once

#include "../dust2gpu/system.hpp"

namespace dust2gpu {
namespace systems {

struct sir {
  static constexpr const char* name = "sir";
  using real_type = double;
  using rng_state_type = random::rng_state;

  struct shared_state {
    real_type N;
    real_type I0;
    real_type beta;
    real_type gamma;
    real_type exp_noise;
  };
  struct internal_state {};
  struct data_type {
    real_type incidence;
  };

  static constexpr int n_state_max = 5;
  static constexpr real_type default_dt = 1;
  // state entries and the gradient of beta, gamma, I0 (sir.cpp:122-124)
  static constexpr int n_adjoint_max = 8;

  // inst/examples/sir.cpp:7-11 (parameter annotations) and :74-81.
  static constexpr parameter_info parameters[] = {
    {"I0", 1, 10, false, false},
    {"N", 1, 1000, false, true},
    {"beta", 1, 0.2, false, false},
    {"gamma", 1, 0.1, false, false},
    {"exp_noise", 1, 1e6, false, true}};
  static constexpr const char* data_names[] = {"incidence"};

  static shared_state build_shared(const double* pars) {
    shared_state s;
    s.I0 = read_par<sir>(pars, 0);
    s.N = read_par<sir>(pars, 1);
    s.beta = read_par<sir>(pars, 2);
    s.gamma = read_par<sir>(pars, 3);
    s.exp_noise = read_par<sir>(pars, 4);
    return s;
  }

  // sir.cpp:89-93: only I0, beta and gamma can change.
  static void update_shared(const double* pars, shared_state& s) {
    s.I0 = read_par_update<sir>(pars, 0, s.I0);
    s.beta = read_par_update<sir>(pars, 2, s.beta);
    s.gamma = read_par_update<sir>(pars, 3, s.gamma);
  }

  static std::vector<packing_entry> packing_state(const shared_state&) {
    return {{"S", {}}, {"I", {}}, {"R", {}}, {"cases_cumul", {}},
            {"cases_inc", {}}};
  }

  static int n_state(const shared_state&) {
    return 5;
  }

  // sir.cpp:122-124
  static std::vector<packing_entry> packing_gradient(const shared_state&) {
    return {{"beta", {}}, {"gamma", {}}, {"I0", {}}};
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

  DUST2_HD static void update(real_type time, real_type dt,
                              const real_type* state,
                              const shared_state& shared,
                              internal_state& internal,
                              rng_state_type& rng_state,
                              real_type* state_next) {
    const auto S = state[0];
    const auto I = state[1];
    const auto R = state[2];
    const auto cases_cumul = state[3];
    const auto cases_inc = state[4];
    const auto p_SI = 1 - math::exp(-shared.beta * I / shared.N * dt);
    const auto p_IR = 1 - math::exp(-shared.gamma * dt);
    const auto n_SI = random::binomial(rng_state, S, p_SI);
    const auto n_IR = random::binomial(rng_state, I, p_IR);
    state_next[0] = S - n_SI;
    state_next[1] = I + n_SI - n_IR;
    state_next[2] = R + n_IR;
    state_next[3] = cases_cumul + n_SI;
    state_next[4] = cases_inc + n_SI;
  }

  DUST2_HD static real_type compare_data(const real_type time,
                                         const real_type* state,
                                         const data_type& data,
                                         const shared_state& shared,
                                         internal_state& internal,
                                         rng_state_type& rng_state) {
    const auto incidence_observed = data.incidence;
    if (math::is_nan(data.incidence)) {
      return 0;
    }
    const auto noise = random::exponential_rate(rng_state, shared.exp_noise);
    const auto incidence_modelled = state[4];
    const auto lambda = incidence_modelled + noise;
    return density::poisson(incidence_observed, lambda, true);
  }

  // The adjoint equations of the deterministic model (sir.cpp:126-210),
  // term for term: the reverse-mode derivatives of update, compare and
  // initial with respect to state and to beta, gamma, I0.
  DUST2_HD static void adjoint_initial(real_type time,
                                       const real_type* state,
                                       const real_type* adjoint,
                                       const shared_state& shared,
                                       internal_state& internal,
                                       real_type* adjoint_next) {
    const real_type adj_I = adjoint[1];
    for (int i = 0; i < 7; ++i) {
      adjoint_next[i] = adjoint[i];
    }
    adjoint_next[7] = adjoint[7] + adj_I;
  }

  DUST2_HD static void adjoint_update(real_type time, real_type dt,
                                      const real_type* state,
                                      const real_type* adjoint,
                                      const shared_state& shared,
                                      internal_state& internal,
                                      real_type* adjoint_next) {
    const auto S = state[0];
    const auto I = state[1];
    const auto adj_S = adjoint[0];
    const auto adj_I = adjoint[1];
    const auto adj_R = adjoint[2];
    const auto adj_cases_cumul = adjoint[3];
    const auto adj_cases_inc = adjoint[4];
    const auto adj_beta = adjoint[5];
    const auto adj_gamma = adjoint[6];
    const auto adj_I0 = adjoint[7];
    const auto p_SI = 1 - math::exp(-shared.beta * I / shared.N * dt);
    const auto p_IR = 1 - math::exp(-shared.gamma * dt);
    const auto adj_n_IR = -adj_I + adj_R;
    const auto adj_n_SI = adj_cases_inc + adj_cases_cumul + adj_I + -adj_S;
    const auto adj_p_IR = adj_n_IR * I;
    const auto adj_p_SI = adj_n_SI * S;
    const auto e_SI = math::exp(-shared.beta * I * dt / shared.N);
    adjoint_next[0] = adj_n_SI * p_SI + adj_S;
    adjoint_next[1] = adj_n_IR * p_IR +
      adj_p_SI * (shared.beta * dt) * e_SI / shared.N + adj_I;
    adjoint_next[2] = adj_R;
    adjoint_next[3] = adj_cases_cumul;
    adjoint_next[4] = adj_cases_inc;
    adjoint_next[5] = adj_beta + adj_p_SI * I * dt * e_SI / shared.N;
    adjoint_next[6] = adj_gamma + adj_p_IR * math::exp(-shared.gamma);
    adjoint_next[7] = adj_I0;
  }

  DUST2_HD static void adjoint_compare_data(real_type time,
                                            const real_type* state,
                                            const real_type* adjoint,
                                            const data_type& data,
                                            const shared_state& shared,
                                            internal_state& internal,
                                            real_type* adjoint_next) {
    const real_type cases_inc = state[4];
    const real_type noise = 1 / shared.exp_noise;
    const real_type lambda = cases_inc + noise;
    const real_type adj_lambda = data.incidence / lambda - 1;
    for (int i = 0; i < 8; ++i) {
      adjoint_next[i] = adjoint[i];
    }
    adjoint_next[4] = adjoint[4] + adj_lambda;
  }
};

}  // namespace systems
}  // namespace dust2gpu
