// Gaussian random walk: the GPU restatement of dust2's bundled example
// inst/examples/walk.cpp (parameters sd, len, random_initial; no compare).
#pragma once

#include "../dust2gpu/system.hpp"

namespace dust2gpu {
namespace systems {

struct walk {
  static constexpr const char* name = "walk";
  using real_type = double;
  using rng_state_type = random::rng_state;

  struct shared_state {
    int len;
    real_type sd;
    bool random_initial;
  };
  struct internal_state {};
  struct data_type {};

  static constexpr int n_state_max = 16;
  static constexpr real_type default_dt = 1;

  static constexpr parameter_info parameters[] = {
    {"sd", 1, NAN, true, false},
    {"len", 1, 1, false, true},
    {"random_initial", 1, 0, false, true}};

  static shared_state build_shared(const double* pars) {
    shared_state s;
    s.sd = read_par<walk>(pars, 0);
    const double len = read_par<walk>(pars, 1);
    if (!(len >= 1) || len > n_state_max || len != std::floor(len)) {
      throw std::runtime_error("'len' must be an integer in [1, 16]");
    }
    s.len = static_cast<int>(len);
    s.random_initial = read_par<walk>(pars, 2) != 0;
    return s;
  }

  static void update_shared(const double* pars, shared_state& s) {
    s.sd = read_par_update<walk>(pars, 0, s.sd);
  }

  static std::vector<packing_entry> packing_state(const shared_state& s) {
    return {{"x", {s.len}}};
  }

  static int n_state(const shared_state& s) {
    return s.len;
  }

  static zero_every_spec zero_every(const shared_state&) {
    return zero_every_none();
  }

  DUST2_HD static void initial(real_type time, const shared_state& shared,
                               internal_state& internal,
                               rng_state_type& rng_state,
                               real_type* state_next) {
    for (int i = 0; i < shared.len; ++i) {
      state_next[i] = shared.random_initial ?
        random::normal(rng_state, 0, shared.sd) : 0;
    }
  }

  DUST2_HD static void update(real_type time, real_type dt,
                              const real_type* state,
                              const shared_state& shared,
                              internal_state& internal,
                              rng_state_type& rng_state,
                              real_type* state_next) {
    for (int i = 0; i < shared.len; ++i) {
      state_next[i] = random::normal(rng_state, state[i], shared.sd * dt);
    }
  }
};

}  // namespace systems
}  // namespace dust2gpu
