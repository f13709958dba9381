// Mixed-time malaria transmission model: the GPU restatement of dust2's
// bundled example inst/examples/malaria.cpp.  Humans (Sh, Ih) and vectors
// (Sv, Iv, and n_rates exposed compartments Ev) follow an ODE; the vector
// birth rate beta is "special" state that the rhs reads but does not
// integrate, and that the discrete-time update moves as a log-normal
// random walk every dt.  Data are tested/positive counts compared with a
// binomial on the human prevalence Ih.
#pragma once

#include <string>

#include "../dust2gpu/system.hpp"

namespace dust2gpu {
namespace systems {

struct malaria {
  static constexpr const char* name = "malaria";
  using real_type = double;
  using rng_state_type = random::rng_state;

  struct shared_state {
    real_type a;      // biting rate
    real_type bh;     // Pr(transmission vector to human)
    real_type bv;     // Pr(transmission human to vector)
    int n_rates;      // number of exposed compartments
    real_type mu;     // -log(Pr(vector survival))
    real_type r;      // recovery rate
    real_type tau;    // mosquito latency
    real_type initial_Ih;
    real_type initial_Iv;
    real_type initial_Sv;
    real_type beta_volatility;
  };
  struct internal_state {};
  struct data_type {
    real_type tested;
    real_type positive;
  };

  // State: [Sh, Ih, Sv, Iv, Ev[n_rates], beta]; n_rates is bounded so
  // that the state fits a thread's registers and local memory.
  static constexpr int n_rates_max = 19;
  static constexpr int n_state_max = 4 + n_rates_max + 1;
  static constexpr int n_output = 0;
  static constexpr int n_special = 1;

  static constexpr parameter_info parameters[] = {
    {"a", 1, 1.0 / 3.0, false, false},
    {"n_rates", 1, 15, false, true},
    {"r", 1, 0.01, false, false},
    {"tau", 1, 12, false, false},
    {"initial_Ih", 1, 0.8, false, true},
    {"initial_Iv", 1, 18, false, true},
    {"initial_Sv", 1, 100, false, true},
    {"beta_volatility", 1, 0.5, false, true}};
  static constexpr const char* data_names[] = {"tested", "positive"};

  // malaria.cpp build_shared: bh = bv = 0.05, daily vector survival 0.9
  static shared_state build_shared(const double* pars) {
    shared_state s;
    s.a = read_par<malaria>(pars, 0);
    const double n_rates = read_par<malaria>(pars, 1);
    if (!(n_rates >= 1 && n_rates <= n_rates_max) ||
        n_rates != static_cast<double>(static_cast<int>(n_rates))) {
      throw std::runtime_error("'n_rates' must be an integer in [1, " +
                               std::to_string(n_rates_max) + "]");
    }
    s.n_rates = static_cast<int>(n_rates);
    s.r = read_par<malaria>(pars, 2);
    s.tau = read_par<malaria>(pars, 3);
    s.initial_Ih = read_par<malaria>(pars, 4);
    s.initial_Iv = read_par<malaria>(pars, 5);
    s.initial_Sv = read_par<malaria>(pars, 6);
    s.beta_volatility = read_par<malaria>(pars, 7);
    s.bh = 0.05;
    s.bv = 0.05;
    s.mu = -math::log(0.9);
    return s;
  }

  static void update_shared(const double* pars, shared_state& s) {
    s.a = read_par_update<malaria>(pars, 0, s.a);
    s.r = read_par_update<malaria>(pars, 2, s.r);
    s.tau = read_par_update<malaria>(pars, 3, s.tau);
  }

  static std::vector<packing_entry> packing_state(const shared_state& s) {
    return {{"Sh", {}}, {"Ih", {}}, {"Sv", {}}, {"Iv", {}},
            {"Ev", {s.n_rates}}, {"beta", {}}};
  }

  static int n_state(const shared_state& s) {
    return 4 + s.n_rates + 1;
  }

  static zero_every_spec zero_every(const shared_state&) {
    return zero_every_none();
  }

  static data_type build_data(const double* d) {
    return data_type{d[0], d[1]};
  }

  DUST2_HD static void initial(real_type time, const shared_state& shared,
                               internal_state& internal,
                               rng_state_type& rng_state,
                               real_type* state_next) {
    state_next[0] = 1 - shared.initial_Ih;
    state_next[1] = shared.initial_Ih;
    state_next[2] = shared.initial_Sv;
    state_next[3] = shared.initial_Iv;
    for (int i = 4; i < 4 + shared.n_rates; ++i) {
      state_next[i] = 0;
    }
    state_next[4 + shared.n_rates] = shared.mu;
  }

  DUST2_HD static void rhs(real_type time, const real_type* state,
                           const shared_state& shared,
                           internal_state& internal,
                           real_type* state_deriv) {
    const real_type Sh = state[0];
    const real_type Ih = state[1];
    const real_type Sv = state[2];
    const real_type Iv = state[3];
    const real_type* Ev = state + 4;
    const int n = shared.n_rates;
    const real_type beta = state[4 + n];
    const real_type foi_h = shared.a * shared.bh * Iv;
    const real_type foi_v = shared.a * shared.bv * Ih;
    const real_type rate = n / shared.tau;
    state_deriv[4] = foi_v * Sv - rate * Ev[0] - shared.mu * Ev[0];
    for (int i = 1; i < n; ++i) {
      state_deriv[4 + i] = rate * Ev[i - 1] - rate * Ev[i] -
        shared.mu * Ev[i];
    }
    state_deriv[0] = -foi_h * Sh + shared.r * Ih;
    state_deriv[1] = foi_h * Sh - shared.r * Ih;
    state_deriv[2] = beta * shared.initial_Sv - foi_v * Sv - shared.mu * Sv;
    state_deriv[3] = rate * Ev[n - 1] - shared.mu * Iv;
  }

  // Only the special entry changes; the engine has copied the rest of the
  // state into state_next before the call (continuous/system.hpp:568).
  DUST2_HD static void update(real_type time, real_type dt,
                              const real_type* state,
                              const shared_state& shared,
                              internal_state& internal,
                              rng_state_type& rng_state,
                              real_type* state_next) {
    const int i = 4 + shared.n_rates;
    const real_type beta = state[i];
    state_next[i] = beta * math::exp(
      random::normal(rng_state, 0, shared.beta_volatility));
  }

  DUST2_HD static real_type compare_data(const real_type time,
                                         const real_type* state,
                                         const data_type& data,
                                         const shared_state& shared,
                                         internal_state& internal,
                                         rng_state_type& rng_state) {
    if (math::is_nan(data.positive) || math::is_nan(data.tested)) {
      return 0;
    }
    return density::binomial(data.positive, data.tested, state[1], true);
  }
};

}  // namespace systems
}  // namespace dust2gpu
