// SIRS with waning immunity and a negative-binomial observation of daily
// incidence, written as a dust2 system class (the shape of dust2's
// inst/examples/*.cpp: cpp11::list readers, monty samplers,
// dust2::packing, dust2::zero_every_type) rather than against this
// engine's own contract.  It compiles through compat/dust2/common.hpp and
// is adapted by compat/plugin.hpp; the only change a dust2 class needs is
// DUST2_HD on the functions that run on the device.
//
// Per step of length dt, in this order:
//   n_SI ~ Bin(S, 1 - exp(-beta I / N dt))
//   n_IR ~ Bin(I, 1 - exp(-gamma dt))
//   n_RS ~ Bin(R, 1 - exp(-omega dt))
// and incidence (n_SI) accumulates between daily resets.
// compare: log NegBin(cases | size = kappa, mu = incidence + 1e-6).
#pragma once

#include <dust2/common.hpp>

#include "../compat/plugin.hpp"

// [[dust2::class(sirs)]]
// [[dust2::time_type(discrete)]]
// [[dust2::has_compare()]]
// [[dust2::parameter(N, constant = TRUE)]]
// [[dust2::parameter(I0, constant = FALSE)]]
// [[dust2::parameter(beta, constant = FALSE)]]
// [[dust2::parameter(gamma, constant = FALSE)]]
// [[dust2::parameter(omega, constant = FALSE)]]
// [[dust2::parameter(kappa, constant = TRUE)]]
class sirs {
public:
  sirs() = delete;

  using real_type = double;

  struct shared_state {
    real_type N;
    real_type I0;
    real_type beta;
    real_type gamma;
    real_type omega;
    real_type kappa;
  };

  struct internal_state {};

  struct data_type {
    real_type cases;
  };

  using rng_state_type = monty::random::generator<real_type>;

  static dust2::packing packing_state(const shared_state& shared) {
    return dust2::packing{{"S", {}}, {"I", {}}, {"R", {}}, {"incidence", {}}};
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
    const real_type S = state[0];
    const real_type I = state[1];
    const real_type R = state[2];
    const real_type lambda = shared.beta * I / shared.N;
    const real_type p_SI = 1 - monty::math::exp(-lambda * dt);
    const real_type p_IR = 1 - monty::math::exp(-shared.gamma * dt);
    const real_type p_RS = 1 - monty::math::exp(-shared.omega * dt);
    const real_type n_SI = monty::random::binomial<real_type>(rng_state, S,
                                                              p_SI);
    const real_type n_IR = monty::random::binomial<real_type>(rng_state, I,
                                                              p_IR);
    const real_type n_RS = monty::random::binomial<real_type>(rng_state, R,
                                                              p_RS);
    state_next[0] = S - n_SI + n_RS;
    state_next[1] = I + n_SI - n_IR;
    state_next[2] = R + n_IR - n_RS;
    state_next[3] = state[3] + n_SI;
  }

  static shared_state build_shared(cpp11::list pars) {
    shared_state s;
    s.N = dust2::r::read_real(pars, "N", 10000);
    s.I0 = dust2::r::read_real(pars, "I0", 10);
    s.beta = dust2::r::read_real(pars, "beta");
    s.gamma = dust2::r::read_real(pars, "gamma", 0.1);
    s.omega = dust2::r::read_real(pars, "omega", 0.01);
    s.kappa = dust2::r::read_real(pars, "kappa", 10);
    return s;
  }

  static void update_shared(cpp11::list pars, shared_state& shared) {
    shared.I0 = dust2::r::read_real(pars, "I0", shared.I0);
    shared.beta = dust2::r::read_real(pars, "beta", shared.beta);
    shared.gamma = dust2::r::read_real(pars, "gamma", shared.gamma);
    shared.omega = dust2::r::read_real(pars, "omega", shared.omega);
  }

  static auto zero_every(const shared_state& shared) {
    return dust2::zero_every_type<real_type>{{1, {3}}};
  }

  static data_type build_data(cpp11::list r_data, const shared_state& shared) {
    return data_type{dust2::r::read_real(r_data, "cases", NA_REAL)};
  }

  DUST2_HD static real_type compare_data(const real_type time,
                                         const real_type* state,
                                         const data_type& data,
                                         const shared_state& shared,
                                         internal_state& internal,
                                         rng_state_type& rng_state) {
    if (std::isnan(data.cases)) {
      return 0;
    }
    return monty::density::negative_binomial_mu(data.cases, shared.kappa,
                                                state[3] + 1e-6, true);
  }
};

namespace dust2gpu {
namespace systems {

// What dust2 would generate from the annotations above: the parameter
// table (names and lengths; defaults stay in build_shared) and the data
// fields, plus the engine's bound on the state size.
struct sirs_spec {
  using system = ::sirs;
  static constexpr const char* name = "sirs";
  static constexpr int n_state_max = 4;
  static constexpr double default_dt = 1;
  static constexpr parameter_info parameters[] = {
    {"N", 1, NAN, false, true},
    {"I0", 1, NAN, false, false},
    {"beta", 1, NAN, true, false},
    {"gamma", 1, NAN, false, false},
    {"omega", 1, NAN, false, false},
    {"kappa", 1, NAN, false, true}};
  static constexpr const char* data_names[] = {"cases"};
};

using sirs = compat::plugin<sirs_spec>;

}  // namespace systems
}  // namespace dust2gpu
