// Age-structured stochastic SEIR with a negative-binomial observation of
// total daily incidence (16 age groups; state S, E, I, R, cases_cumul and
// cases_inc per age, 96 entries).  Written against dust2's plugin
// contract (vignettes/writing.Rmd; structure as inst/examples/sir.cpp):
//   lambda_a = beta sum_b C[a][b] I_b / N_b,   beta = R0 gamma / rho(C)
//   per age a, in this order: n_SE ~ Bin(S_a, 1 - exp(-lambda_a dt)),
//   n_EI ~ Bin(E_a, 1 - exp(-sigma dt)), n_IR ~ Bin(I_a, 1 - exp(-gamma dt))
//   incidence counts n_EI and resets daily;
//   compare: log NegBin(observed | size, mu = sum_a cases_inc_a + 1e-6).
// rho(C) is the spectral radius of the contact matrix, found on the host
// by power iteration when parameters are read.
#pragma once

#include "../dust2gpu/system.hpp"

namespace dust2gpu {
namespace systems {

struct seir_age {
  static constexpr const char* name = "seir_age";
  // update() reads the entries of age a (and, before its loop, every I)
  // before it writes the same entries of state_next, and reads nothing
  // it has written: it is correct in place, so a particle keeps one
  // state array.
  static constexpr bool update_in_place = true;
  // The 96 doubles stay in a per-thread array (local memory, cached),
  // with 4 blocks of 128 threads per SM (128 registers).  Measured on
  // the batched SEIR filter (particle-steps/s): this 149.5M; 3 blocks
  // 144.3M; 5 blocks 147.3M.  Earlier builds: two arrays with copies
  // (before in-place updates) 116.0M against 118.2M in place; the state
  // in rows of shared memory instead (2 blocks of 99 KB per SM) 107.7M --
  // occupancy hides the FP64 pipe's latency better than shared memory
  // saves local-memory traffic.
  static constexpr int min_blocks_per_sm = 4;
  using real_type = double;
  using rng_state_type = random::rng_state;
  static constexpr int n_age = 16;

  struct shared_state {
    real_type beta;
    real_type sigma;
    real_type gamma;
    real_type size;
    real_type R0;
    real_type I0;
    real_type N[n_age];
    real_type inv_N[n_age];
    real_type contact[n_age][n_age];
  };
  struct internal_state {};
  struct data_type {
    real_type incidence;
  };

  static constexpr int n_state_max = 6 * n_age;
  static constexpr real_type default_dt = 0.25;

  static constexpr parameter_info parameters[] = {
    {"R0", 1, 2, false, false},
    {"sigma", 1, 0.2, false, false},
    {"gamma", 1, 0.1, false, false},
    {"size", 1, 20, false, true},
    {"I0", 1, 1, false, false},
    {"N", n_age, 62500, false, true},
    {"contact", n_age * n_age, NAN, true, true}};
  static constexpr const char* data_names[] = {"incidence"};

  static real_type spectral_radius(const real_type (&c)[n_age][n_age]) {
    // power iteration; the contact matrix is non-negative
    std::vector<double> x(n_age, 1.0), y(n_age);
    double rho = 0;
    for (int it = 0; it < 1000; ++it) {
      double norm = 0;
      for (int a = 0; a < n_age; ++a) {
        double acc = 0;
        for (int b = 0; b < n_age; ++b) {
          acc += c[a][b] * x[b];
        }
        y[a] = acc;
        norm = std::max(norm, std::fabs(acc));
      }
      if (!(norm > 0)) {
        return 0;
      }
      for (int a = 0; a < n_age; ++a) {
        x[a] = y[a] / norm;
      }
      if (std::fabs(norm - rho) < 1e-14 * norm) {
        rho = norm;
        break;
      }
      rho = norm;
    }
    return rho;
  }

  static void derive(shared_state& s) {
    const double rho = spectral_radius(s.contact);
    s.beta = rho > 0 ? s.R0 * s.gamma / rho : 0;
    for (int a = 0; a < n_age; ++a) {
      s.inv_N[a] = 1.0 / s.N[a];
    }
  }

  static shared_state build_shared(const double* pars) {
    shared_state s{};
    s.R0 = read_par<seir_age>(pars, 0);
    s.sigma = read_par<seir_age>(pars, 1);
    s.gamma = read_par<seir_age>(pars, 2);
    s.size = read_par<seir_age>(pars, 3);
    s.I0 = read_par<seir_age>(pars, 4);
    const double* n = pars + parameter_offset<seir_age>(5);
    for (int a = 0; a < n_age; ++a) {
      s.N[a] = std::isnan(n[0]) ? parameters[5].default_value : n[a];
    }
    read_par_array<seir_age>(pars, 6, &s.contact[0][0], n_age * n_age, true);
    derive(s);
    return s;
  }

  static void update_shared(const double* pars, shared_state& s) {
    s.R0 = read_par_update<seir_age>(pars, 0, s.R0);
    s.sigma = read_par_update<seir_age>(pars, 1, s.sigma);
    s.gamma = read_par_update<seir_age>(pars, 2, s.gamma);
    s.I0 = read_par_update<seir_age>(pars, 4, s.I0);
    derive(s);
  }

  static std::vector<packing_entry> packing_state(const shared_state&) {
    return {{"S", {n_age}}, {"E", {n_age}}, {"I", {n_age}}, {"R", {n_age}},
            {"cases_cumul", {n_age}}, {"cases_inc", {n_age}}};
  }

  static int n_state(const shared_state&) {
    return 6 * n_age;
  }

  static zero_every_spec zero_every(const shared_state&) {
    auto z = zero_every_none();
    std::vector<int> idx;
    for (int a = 0; a < n_age; ++a) {
      idx.push_back(5 * n_age + a);
    }
    zero_every_add(z, 1, idx);
    return z;
  }

  static data_type build_data(const double* d) {
    return data_type{d[0]};
  }

  DUST2_HD static void initial(real_type time, const shared_state& shared,
                               internal_state& internal,
                               rng_state_type& rng_state,
                               real_type* state_next) {
    for (int a = 0; a < n_age; ++a) {
      state_next[a] = shared.N[a] - shared.I0;
      state_next[n_age + a] = 0;
      state_next[2 * n_age + a] = shared.I0;
      state_next[3 * n_age + a] = 0;
      state_next[4 * n_age + a] = 0;
      state_next[5 * n_age + a] = 0;
    }
  }

  DUST2_HD static void update(real_type time, real_type dt,
                              const real_type* state,
                              const shared_state& shared,
                              internal_state& internal,
                              rng_state_type& rng_state,
                              real_type* state_next) {
    const real_type* S = state;
    const real_type* E = state + n_age;
    const real_type* I = state + 2 * n_age;
    const real_type* R = state + 3 * n_age;
    const real_type* cum = state + 4 * n_age;
    const real_type* inc = state + 5 * n_age;
    // Every age's infection probability depends on the state at the
    // start of the step only, so all 16 are computed before the draws;
    // the prevalences x are then dead while the samplers run.
    real_type p_SE[n_age];
    {
      real_type x[n_age];
      for (int b = 0; b < n_age; ++b) {
        x[b] = I[b] * shared.inv_N[b];
      }
#pragma unroll 1
      for (int a = 0; a < n_age; ++a) {
        real_type acc = 0;
        for (int b = 0; b < n_age; ++b) {
          acc = std::fma(shared.contact[a][b], x[b], acc);
        }
        const real_type lambda = shared.beta * acc;
        p_SE[a] = 1 - math::exp(-lambda * dt);
      }
    }
    const real_type p_EI = 1 - math::exp(-shared.sigma * dt);
    const real_type p_IR = 1 - math::exp(-shared.gamma * dt);
    // the same two probabilities serve every age: prepare them once
    const auto b_EI = random::binomial_prepare(p_EI);
    const auto b_IR = random::binomial_prepare(p_IR);
    // one age per iteration, not unrolled: the body holds three samplers
#pragma unroll 1
    for (int a = 0; a < n_age; ++a) {
      const real_type n_SE = random::binomial(rng_state, S[a], p_SE[a]);
      const real_type n_EI = random::binomial(rng_state, E[a], b_EI);
      const real_type n_IR = random::binomial(rng_state, I[a], b_IR);
      state_next[a] = S[a] - n_SE;
      state_next[n_age + a] = E[a] + n_SE - n_EI;
      state_next[2 * n_age + a] = I[a] + n_EI - n_IR;
      state_next[3 * n_age + a] = R[a] + n_IR;
      state_next[4 * n_age + a] = cum[a] + n_EI;
      state_next[5 * n_age + a] = inc[a] + n_EI;
    }
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
    real_type mu = 0;
    for (int a = 0; a < n_age; ++a) {
      mu += state[5 * n_age + a];
    }
    return density::negative_binomial_mu(data.incidence, shared.size,
                                         mu + 1e-6, true);
  }
};

}  // namespace systems
}  // namespace dust2gpu
