// Stochastic SIR with a Poisson observation of daily incidence: the
// model of the benchmark workloads (state S, I, R, cases_inc; binomial
// transitions with p = 1 - exp(-rate dt); daily reset of cases_inc;
// compare log Poisson(observed | cases_inc + 1e-6)).  Same structure and
// draw order as dust2's example inst/examples/sir.cpp:51-72, without the
// cumulative-cases entry and without the random noise draw in compare.
#pragma once

#include "../dust2gpu/system.hpp"

namespace dust2gpu {
namespace systems {

struct sir_cases {
  static constexpr const char* name = "sir_cases";
  using real_type = double;
  using rng_state_type = random::rng_state;

  struct shared_state {
    real_type N;
    real_type I0;
    real_type beta;
    real_type gamma;
  };
  // Per-thread scratch (dust2's internal_state): the recovery
  // probability 1 - exp(-gamma dt) and the terms of its binomial draws
  // that depend on p alone (random::binomial_prepare) are the same at
  // every step while gamma and dt are, so they are kept here and
  // recomputed only when either changes.  The draws are exactly those of
  // binomial(rng, I, p_IR).
  struct internal_state {
    std::uint64_t key_gamma;
    std::uint64_t key_dt;
    bool ready;
    random::binomial_prob b_IR;
  };
  struct data_type {
    real_type incidence;
  };

  static constexpr int n_state_max = 4;
  static constexpr real_type default_dt = 0.25;

  static constexpr parameter_info parameters[] = {
    {"I0", 1, 10, false, false},
    {"N", 1, 1000, false, true},
    {"beta", 1, 0.2, false, false},
    {"gamma", 1, 0.1, false, false}};
  static constexpr const char* data_names[] = {"incidence"};

  static shared_state build_shared(const double* pars) {
    shared_state s;
    s.I0 = read_par<sir_cases>(pars, 0);
    s.N = read_par<sir_cases>(pars, 1);
    s.beta = read_par<sir_cases>(pars, 2);
    s.gamma = read_par<sir_cases>(pars, 3);
    return s;
  }

  static void update_shared(const double* pars, shared_state& s) {
    s.I0 = read_par_update<sir_cases>(pars, 0, s.I0);
    s.beta = read_par_update<sir_cases>(pars, 2, s.beta);
    s.gamma = read_par_update<sir_cases>(pars, 3, s.gamma);
  }

  static std::vector<packing_entry> packing_state(const shared_state&) {
    return {{"S", {}}, {"I", {}}, {"R", {}}, {"cases_inc", {}}};
  }

  static int n_state(const shared_state&) {
    return 4;
  }

  static zero_every_spec zero_every(const shared_state&) {
    auto z = zero_every_none();
    zero_every_add(z, 1, {3});
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
    const auto cases_inc = state[3];
    const auto p_SI = 1 - math::exp(-shared.beta * I / shared.N * dt);
    const auto key_gamma = math::bits_of(shared.gamma);
    const auto key_dt = math::bits_of(dt);
    if (!internal.ready || internal.key_gamma != key_gamma ||
        internal.key_dt != key_dt) {
      internal.b_IR =
        random::binomial_prepare(1 - math::exp(-shared.gamma * dt));
      internal.key_gamma = key_gamma;
      internal.key_dt = key_dt;
      internal.ready = true;
    }
    const auto n_SI = random::binomial(rng_state, S, p_SI);
    const auto n_IR = random::binomial(rng_state, I, internal.b_IR);
    state_next[0] = S - n_SI;
    state_next[1] = I + n_SI - n_IR;
    state_next[2] = R + n_IR;
    state_next[3] = cases_inc + n_SI;
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
    const auto lambda = state[3] + 1e-6;
    return density::poisson(data.incidence, lambda, true);
  }
};

}  // namespace systems
}  // namespace dust2gpu
