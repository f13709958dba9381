// TEST INFRASTRUCTURE (oracle).  Drives dust2's own C++ engine --
// dust2::dust_discrete, dust2::filter, dust2::dust_continuous and the
// filter_details helpers, compiled unmodified from the reference tree
// (inst/include/dust2/...) -- on the project's system classes, and
// exposes it through a small C interface for the tests and for fixture
// generation.  Built by oracle/Makefile into oracle/_ref/ only where the
// reference sources are present; never part of the product.
//
// The project's systems (dust2_gb300/csrc/systems/*.hpp) are written to
// the GPU plugin contract; the adapters below present them to the
// reference engine in its own plugin contract (vignettes/writing.Rmd;
// detection in inst/include/dust2/properties.hpp): `packing_state`
// returns a dust2::packing, `zero_every` a dust2::zero_every_type, and a
// sampler error recorded in the generator becomes the exception the
// reference engine expects to catch (discrete/system.hpp:82-84).
#include <cstdint>
#include <cstring>
#include <limits>
#include <stdexcept>
#include <string>
#include <vector>

#include <dust2/continuous/system.hpp>
#include <dust2/discrete/system.hpp>
#include <dust2/filter.hpp>
#include <dust2/filter_details.hpp>
#include <dust2/unfilter.hpp>

#include "engine/error_text.hpp"
#include "systems/logistic.hpp"
#include "systems/malaria.hpp"
#include "systems/seir_age.hpp"
#include "systems/sir.hpp"
#include "systems/sir_cases.hpp"
#include "systems/sirode.hpp"
#include "systems/walk.hpp"

namespace {

using rng_state_type = dust2gpu::random::rng_state;

void raise_if_error(rng_state_type& rng) {
  if (rng.err != 0) {
    dust2gpu::particle_error e{rng.err, rng.err_v0, rng.err_v1};
    rng.err = 0;
    throw std::runtime_error(dust2gpu::error_text(e));
  }
}

template <typename S>
dust2::zero_every_type<double> zero_every_of(
    const typename S::shared_state& shared) {
  const auto z = S::zero_every(shared);
  dust2::zero_every_type<double> ret;
  for (int i = 0; i < z.n; ++i) {
    std::vector<size_t> idx;
    for (int s = 0; s < 64 * dust2gpu::ZERO_EVERY_WORDS; ++s) {
      if (z.has(i, s)) {
        idx.push_back(s);
      }
    }
    ret.push_back({z.period[i], idx});
  }
  return ret;
}

template <typename S>
struct ref_discrete {
  using real_type = double;
  using rng_state_type = ::rng_state_type;
  using shared_state = typename S::shared_state;
  using internal_state = typename S::internal_state;
  using data_type = typename S::data_type;

  static dust2::packing packing_state(const shared_state& shared) {
    return dust2::packing{
      {"state", {static_cast<size_t>(S::n_state(shared))}}};
  }
  static void initial(real_type time, const shared_state& shared,
                      internal_state& internal, rng_state_type& rng,
                      real_type* state_next) {
    S::initial(time, shared, internal, rng, state_next);
    raise_if_error(rng);
  }
  static void update(real_type time, real_type dt, const real_type* state,
                     const shared_state& shared, internal_state& internal,
                     rng_state_type& rng, real_type* state_next) {
    S::update(time, dt, state, shared, internal, rng, state_next);
    raise_if_error(rng);
  }
  static real_type compare_data(const real_type time, const real_type* state,
                                const data_type& data,
                                const shared_state& shared,
                                internal_state& internal,
                                rng_state_type& rng) {
    const auto ret = S::compare_data(time, state, data, shared, internal, rng);
    raise_if_error(rng);
    return ret;
  }
  static dust2::zero_every_type<real_type> zero_every(
      const shared_state& shared) {
    return zero_every_of<S>(shared);
  }
};

// The same system with its adjoint methods forwarded, so that
// dust2::properties sees packing_gradient (properties.hpp:19-21, 121-129)
// and unfilter::last_gradient runs compute_gradient_.
template <typename S>
struct ref_discrete_adjoint : ref_discrete<S> {
  using real_type = double;
  using shared_state = typename S::shared_state;
  using internal_state = typename S::internal_state;
  using data_type = typename S::data_type;

  // dust2::packing is built from an initializer list only; the systems
  // with adjoints here have three scalar gradient entries.
  static dust2::packing packing_gradient(const shared_state& shared) {
    const auto e = S::packing_gradient(shared);
    if (e.size() != 3 || !e[0].dims.empty() || !e[1].dims.empty() ||
        !e[2].dims.empty()) {
      throw std::runtime_error("expected three scalar gradient entries");
    }
    return dust2::packing{{e[0].name, {}}, {e[1].name, {}}, {e[2].name, {}}};
  }
  static void adjoint_initial(real_type time, const real_type* state,
                              const real_type* adjoint,
                              const shared_state& shared,
                              internal_state& internal,
                              real_type* adjoint_next) {
    S::adjoint_initial(time, state, adjoint, shared, internal, adjoint_next);
  }
  static void adjoint_update(real_type time, real_type dt,
                             const real_type* state,
                             const real_type* adjoint,
                             const shared_state& shared,
                             internal_state& internal,
                             real_type* adjoint_next) {
    S::adjoint_update(time, dt, state, adjoint, shared, internal,
                      adjoint_next);
  }
  static void adjoint_compare_data(real_type time, const real_type* state,
                                   const real_type* adjoint,
                                   const data_type& data,
                                   const shared_state& shared,
                                   internal_state& internal,
                                   real_type* adjoint_next) {
    S::adjoint_compare_data(time, state, adjoint, data, shared, internal,
                            adjoint_next);
  }
};

template <typename S>
struct ref_continuous {
  using real_type = double;
  using rng_state_type = ::rng_state_type;
  using shared_state = typename S::shared_state;
  using internal_state = typename S::internal_state;
  using data_type = typename S::data_type;

  static dust2::packing packing_state(const shared_state& shared) {
    return dust2::packing{
      {"state", {static_cast<size_t>(S::n_state(shared))}}};
  }
  static void initial(real_type time, const shared_state& shared,
                      internal_state& internal, rng_state_type& rng,
                      real_type* state_next) {
    S::initial(time, shared, internal, rng, state_next);
  }
  static void rhs(real_type time, const real_type* state,
                  const shared_state& shared, internal_state& internal,
                  real_type* deriv) {
    S::rhs(time, state, shared, internal, deriv);
  }
  static real_type compare_data(const real_type time, const real_type* state,
                                const data_type& data,
                                const shared_state& shared,
                                internal_state& internal,
                                rng_state_type& rng) {
    return S::compare_data(time, state, data, shared, internal, rng);
  }
  static dust2::zero_every_type<real_type> zero_every(
      const shared_state& shared) {
    return zero_every_of<S>(shared);
  }
};

// A mixed-time system (rhs + update) for dust_continuous: the special
// entries are the last packing block, counted by size_special
// (properties.hpp:130-153).
template <typename S>
struct ref_mixed : ref_continuous<S> {
  using real_type = double;
  using rng_state_type = ::rng_state_type;
  using shared_state = typename S::shared_state;
  using internal_state = typename S::internal_state;

  static dust2::packing packing_state(const shared_state& shared) {
    const size_t n = S::n_state(shared);
    return dust2::packing{
      {"state", {n - S::n_special}},
      {"special", {static_cast<size_t>(S::n_special)}}};
  }
  static size_t size_special() {
    return 1;
  }
  static void update(real_type time, real_type dt, const real_type* state,
                     const shared_state& shared, internal_state& internal,
                     rng_state_type& rng, real_type* state_next) {
    S::update(time, dt, state, shared, internal, rng, state_next);
    raise_if_error(rng);
  }
};

// logistic: an ODE with one output variable (size_output / output).
struct ref_logistic {
  using S = dust2gpu::systems::logistic;
  using real_type = double;
  using rng_state_type = ::rng_state_type;
  using shared_state = S::shared_state;
  using internal_state = S::internal_state;
  using data_type = S::data_type;

  static dust2::packing packing_state(const shared_state& shared) {
    return dust2::packing{{"x", {static_cast<size_t>(shared.n)}},
                          {"total", {}}};
  }
  static size_t size_output() {
    return 1;
  }
  static void initial(real_type time, const shared_state& shared,
                      internal_state& internal, rng_state_type& rng,
                      real_type* state_next) {
    S::initial(time, shared, internal, rng, state_next);
  }
  static void rhs(real_type time, const real_type* state,
                  const shared_state& shared, internal_state& internal,
                  real_type* deriv) {
    S::rhs(time, state, shared, internal, deriv);
  }
  static void output(real_type time, real_type* state,
                     const shared_state& shared, internal_state& internal) {
    S::output(time, state, shared, internal);
  }
};

template <typename T>
struct tag {
  using type = T;
};

template <typename F>
bool dispatch_discrete(const std::string& name, F f) {
  using namespace dust2gpu::systems;
  if (name == "sir") {
    f(tag<ref_discrete<sir>>{}, tag<sir>{});
  } else if (name == "sir_cases") {
    f(tag<ref_discrete<sir_cases>>{}, tag<sir_cases>{});
  } else if (name == "walk") {
    f(tag<ref_discrete<walk>>{}, tag<walk>{});
  } else if (name == "seir_age") {
    f(tag<ref_discrete<seir_age>>{}, tag<seir_age>{});
  } else {
    return false;
  }
  return true;
}

template <typename S>
std::vector<typename S::shared_state> shared_of(const double* pars,
                                                int n_groups) {
  const int np = dust2gpu::parameter_length<S>();
  std::vector<typename S::shared_state> ret;
  for (int g = 0; g < n_groups; ++g) {
    ret.push_back(S::build_shared(pars + static_cast<size_t>(g) * np));
  }
  return ret;
}

void set_err(char* err, int err_len, const std::string& msg) {
  if (err != nullptr && err_len > 0) {
    std::strncpy(err, msg.c_str(), err_len - 1);
    err[err_len - 1] = '\0';
  }
}

}  // namespace

extern "C" {

// dust_discrete: set initial state (or `initial`), then run_to_time for
// each of `times`, recording the full state after each.  out:
// [n_times][group][particle][state]; rng_out: final generator state.
int ref_discrete_simulate(const char* name, const double* pars, int n_groups,
                          int n_particles, double time, double dt,
                          const uint64_t* rng, int deterministic,
                          const double* initial, const double* times,
                          int n_times, double* out, uint64_t* rng_out,
                          char* err, int err_len) {
  try {
    bool ok = dispatch_discrete(name, [&](auto t, auto s) {
      using T = typename decltype(t)::type;
      using S = typename decltype(s)::type;
      auto shared = shared_of<S>(pars, n_groups);
      std::vector<typename T::internal_state> internal(n_groups);
      const size_t n_total = static_cast<size_t>(n_particles) * n_groups;
      std::vector<uint64_t> seed(rng, rng + 4 * n_total);
      dust2::dust_discrete<T> sys(shared, internal, time, dt, n_particles,
                                  seed, deterministic != 0, 1);
      if (initial == nullptr) {
        sys.set_state_initial(sys.all_groups());
      } else {
        sys.set_state(initial, {}, {}, {}, false, false);
      }
      const size_t len = sys.state().size();
      for (int i = 0; i < n_times; ++i) {
        sys.run_to_time(times[i], sys.all_groups());
        std::copy(sys.state().begin(), sys.state().end(), out + i * len);
      }
      const auto r = sys.rng_state();
      std::copy(r.begin(), r.end(), rng_out);
    });
    if (!ok) {
      throw std::runtime_error(std::string("unknown system ") + name);
    }
    return 0;
  } catch (const std::exception& e) {
    set_err(err, err_len, e.what());
    return 1;
  }
}

// dust_discrete::compare_data on a given state.
int ref_compare(const char* name, const double* pars, int n_groups,
                int n_particles, double time, const double* state,
                const double* data, int n_groups_data, const uint64_t* rng,
                double* out, uint64_t* rng_out, char* err, int err_len) {
  try {
    bool ok = dispatch_discrete(name, [&](auto t, auto s) {
      using T = typename decltype(t)::type;
      using S = typename decltype(s)::type;
      if constexpr (dust2gpu::has_compare_data<S>::value) {
        auto shared = shared_of<S>(pars, n_groups);
        std::vector<typename T::internal_state> internal(n_groups);
        const size_t n_total = static_cast<size_t>(n_particles) * n_groups;
        std::vector<uint64_t> seed(rng, rng + 4 * n_total);
        dust2::dust_discrete<T> sys(shared, internal, time, 1.0, n_particles,
                                    seed, false, 1);
        sys.set_state(state, {}, {}, {}, false, false);
        std::vector<typename S::data_type> d;
        const int nd = sizeof(typename S::data_type) / sizeof(double);
        for (int g = 0; g < n_groups_data; ++g) {
          d.push_back(S::build_data(data + g * nd));
        }
        std::vector<double> o(n_total);
        sys.compare_data(d.begin(), n_groups_data, sys.all_groups(),
                         o.begin());
        std::copy(o.begin(), o.end(), out);
        const auto r = sys.rng_state();
        std::copy(r.begin(), r.end(), rng_out);
      } else {
        throw std::runtime_error("system has no compare_data");
      }
    });
    if (!ok) {
      throw std::runtime_error(std::string("unknown system ") + name);
    }
    return 0;
  } catch (const std::exception& e) {
    set_err(err, err_len, e.what());
    return 1;
  }
}

// dust2::filter over dust_discrete, following dust2_discrete_filter_alloc
// (r/discrete/filter.hpp:13-88) for the stream split.  Runs the filter
// n_runs times (the object persists between runs, as
// dust_likelihood_run does); ll_out: [n_runs][n_groups].  initial (may be
// null) is applied before every run in place of the initial conditions.
int ref_filter_run(const char* name, const double* pars, int n_groups,
                   int n_particles, double time_start, const double* times,
                   int n_times, const double* data, int n_groups_data,
                   double dt, const uint64_t* rng, int n_runs,
                   const double* initial, double* ll_out, double* state_out,
                   uint64_t* rng_out, char* err, int err_len) {
  try {
    bool ok = dispatch_discrete(name, [&](auto t, auto s) {
      using T = typename decltype(t)::type;
      using S = typename decltype(s)::type;
      if constexpr (dust2gpu::has_compare_data<S>::value) {
        auto shared = shared_of<S>(pars, n_groups);
        std::vector<typename T::internal_state> internal(n_groups);
        std::vector<uint64_t> seed_filter, seed_system;
        for (int g = 0; g < n_groups; ++g) {
          const uint64_t* it = rng + static_cast<size_t>(g) * 4 *
            (n_particles + 2);
          seed_filter.insert(seed_filter.end(), it, it + 8);
          seed_system.insert(seed_system.end(), it + 8,
                             it + 4 * (n_particles + 2));
        }
        dust2::dust_discrete<T> sys(shared, internal, time_start, dt,
                                    n_particles, seed_system, false, 1);
        std::vector<double> tt(times, times + n_times);
        std::vector<typename S::data_type> d;
        const int nd = sizeof(typename S::data_type) / sizeof(double);
        for (int i = 0; i < n_times * n_groups_data; ++i) {
          d.push_back(S::build_data(data + static_cast<size_t>(i) * nd));
        }
        dust2::filter<dust2::dust_discrete<T>> obj(sys, time_start, tt, d,
                                                   seed_filter);
        for (int r = 0; r < n_runs; ++r) {
          if (initial != nullptr) {
            obj.sys.set_state(initial, {}, {}, {}, false, false);
          }
          obj.run(initial == nullptr, false, {}, {}, obj.sys.all_groups());
          const auto& ll = obj.last_log_likelihood();
          std::copy(ll.begin(), ll.end(), ll_out + r * n_groups);
        }
        std::copy(obj.sys.state().begin(), obj.sys.state().end(), state_out);
        // the raw layout of r/filter.hpp:273-298
        const auto sf = obj.rng_state();
        const auto ss = obj.sys.rng_state();
        size_t pos = 0;
        for (int g = 0; g < n_groups; ++g) {
          for (int w = 0; w < 8; ++w) {
            rng_out[pos++] = sf[g * 8 + w];
          }
          for (int w = 0; w < 4 * n_particles; ++w) {
            rng_out[pos++] = ss[static_cast<size_t>(g) * 4 * n_particles + w];
          }
        }
      } else {
        throw std::runtime_error("system has no compare_data");
      }
    });
    if (!ok) {
      throw std::runtime_error(std::string("unknown system ") + name);
    }
    return 0;
  } catch (const std::exception& e) {
    set_err(err, err_len, e.what());
    return 1;
  }
}

// dust_continuous: initial conditions, then run_to_time through `times`,
// recording state; stats_out: [particle][3] n_steps, accepted, rejected.
int ref_ode_simulate(const char* name, const double* pars, int n_groups,
                     int n_particles, double time, int max_steps,
                     double atol, double rtol, double step_size_min,
                     double step_size_max, const double* critical,
                     int n_critical, const double* times, int n_times,
                     double* out, int64_t* stats_out, char* err,
                     int err_len) {
  try {
    auto body = [&](auto t, auto s) {
      using T = typename decltype(t)::type;
      using S = typename decltype(s)::type;
      auto shared = shared_of<S>(pars, n_groups);
      std::vector<typename T::internal_state> internal(n_groups);
      std::vector<double> crit(critical, critical + n_critical);
      dust2::ode::control<double> ctl(max_steps, atol, rtol, step_size_min,
                                      step_size_max, crit, false, false);
      std::vector<uint64_t> seed{42};
      dust2::dust_continuous<T> sys(shared, internal, time, 0, ctl,
                                    n_particles, seed, true, 1);
      sys.set_state_initial(sys.all_groups());
      const size_t len = sys.state().size();
      for (int i = 0; i < n_times; ++i) {
        sys.run_to_time(times[i], sys.all_groups());
        const auto& st = sys.state();
        std::copy(st.begin(), st.end(), out + i * len);
      }
      const auto& oi = sys.ode_internals();
      for (size_t k = 0; k < oi.size(); ++k) {
        stats_out[3 * k] = oi[k].n_steps;
        stats_out[3 * k + 1] = oi[k].n_steps_accepted;
        stats_out[3 * k + 2] = oi[k].n_steps_rejected;
      }
    };
    const std::string nm(name);
    if (nm == "sirode") {
      using S = dust2gpu::systems::sirode;
      body(tag<ref_continuous<S>>{}, tag<S>{});
    } else if (nm == "logistic") {
      body(tag<ref_logistic>{}, tag<dust2gpu::systems::logistic>{});
    } else {
      throw std::runtime_error("unknown system " + nm);
    }
    return 0;
  } catch (const std::exception& e) {
    set_err(err, err_len, e.what());
    return 1;
  }
}

// dust_continuous over a mixed-time system (continuous/system.hpp:80-106,
// 544-585): initial conditions, then run_to_time through `times`
// recording state.  dt = 0 runs the ODE alone.  rng: 4 words per particle
// (the particles' streams).  stats_out: [particle][3] n_steps, accepted,
// rejected.
int ref_mixed_simulate(const char* name, const double* pars, int n_groups,
                       int n_particles, double time, double dt,
                       int max_steps, double atol, double rtol,
                       double step_size_min, double step_size_max,
                       const uint64_t* rng, const double* times, int n_times,
                       double* out, int64_t* stats_out, char* err,
                       int err_len) {
  try {
    const std::string nm(name);
    if (nm != "malaria") {
      throw std::runtime_error("unknown system " + nm);
    }
    using S = dust2gpu::systems::malaria;
    using T = ref_mixed<S>;
    auto shared = shared_of<S>(pars, n_groups);
    std::vector<typename T::internal_state> internal(n_groups);
    dust2::ode::control<double> ctl(max_steps, atol, rtol, step_size_min,
                                    step_size_max, {}, false, false);
    const size_t n_total = static_cast<size_t>(n_particles) * n_groups;
    std::vector<uint64_t> seed(rng, rng + 4 * n_total);
    dust2::dust_continuous<T> sys(shared, internal, time, dt, ctl,
                                  n_particles, seed, false, 1);
    sys.set_state_initial(sys.all_groups());
    const size_t len = sys.state().size();
    for (int i = 0; i < n_times; ++i) {
      sys.run_to_time(times[i], sys.all_groups());
      const auto& st = sys.state();
      std::copy(st.begin(), st.end(), out + i * len);
    }
    const auto& oi = sys.ode_internals();
    for (size_t k = 0; k < oi.size(); ++k) {
      stats_out[3 * k] = oi[k].n_steps;
      stats_out[3 * k + 1] = oi[k].n_steps_accepted;
      stats_out[3 * k + 2] = oi[k].n_steps_rejected;
    }
    return 0;
  } catch (const std::exception& e) {
    set_err(err, err_len, e.what());
    return 1;
  }
}

// dust2::filter over dust_continuous for a mixed-time system, following
// dust2_continuous_filter_alloc (r/continuous/filter.hpp:13-86) for the
// stream split; otherwise as ref_filter_run (n_runs runs of the same
// object; ll_out [n_runs][n_groups]; state_out; rng_out in the raw layout
// of r/filter.hpp:273-298).
int ref_mixed_filter_run(const char* name, const double* pars, int n_groups,
                         int n_particles, double time_start,
                         const double* times, int n_times, const double* data,
                         int n_groups_data, double dt, int max_steps,
                         double atol, double rtol, double step_size_min,
                         double step_size_max, const uint64_t* rng,
                         int n_runs, double* ll_out, double* state_out,
                         uint64_t* rng_out, char* err, int err_len) {
  try {
    const std::string nm(name);
    if (nm != "malaria") {
      throw std::runtime_error("unknown system " + nm);
    }
    using S = dust2gpu::systems::malaria;
    using T = ref_mixed<S>;
    auto shared = shared_of<S>(pars, n_groups);
    std::vector<typename T::internal_state> internal(n_groups);
    dust2::ode::control<double> ctl(max_steps, atol, rtol, step_size_min,
                                    step_size_max, {}, false, false);
    std::vector<uint64_t> seed_filter, seed_system;
    for (int g = 0; g < n_groups; ++g) {
      const uint64_t* it = rng + static_cast<size_t>(g) * 4 *
        (n_particles + 2);
      seed_filter.insert(seed_filter.end(), it, it + 8);
      seed_system.insert(seed_system.end(), it + 8,
                         it + 4 * (n_particles + 2));
    }
    dust2::dust_continuous<T> sys(shared, internal, time_start, dt, ctl,
                                  n_particles, seed_system, false, 1);
    std::vector<double> tt(times, times + n_times);
    std::vector<typename S::data_type> d;
    const int nd = sizeof(typename S::data_type) / sizeof(double);
    for (int i = 0; i < n_times * n_groups_data; ++i) {
      d.push_back(S::build_data(data + static_cast<size_t>(i) * nd));
    }
    dust2::filter<dust2::dust_continuous<T>> obj(sys, time_start, tt, d,
                                                 seed_filter);
    for (int r = 0; r < n_runs; ++r) {
      obj.run(true, false, {}, {}, obj.sys.all_groups());
      const auto& ll = obj.last_log_likelihood();
      std::copy(ll.begin(), ll.end(), ll_out + r * n_groups);
    }
    std::copy(obj.sys.state().begin(), obj.sys.state().end(), state_out);
    const auto sf = obj.rng_state();
    const auto ss = obj.sys.rng_state();
    size_t pos = 0;
    for (int g = 0; g < n_groups; ++g) {
      for (int w = 0; w < 8; ++w) {
        rng_out[pos++] = sf[g * 8 + w];
      }
      for (int w = 0; w < 4 * n_particles; ++w) {
        rng_out[pos++] = ss[static_cast<size_t>(g) * 4 * n_particles + w];
      }
    }
    return 0;
  } catch (const std::exception& e) {
    set_err(err, err_len, e.what());
    return 1;
  }
}

// dust2::filter::run with save_trajectories and snapshots
// (filter.hpp:42-104) and the export of both with reordering
// (trajectories.hpp:135-268, as r/filter.hpp:55-137 calls it);
// select_random draws one particle per group from the filter's second
// streams (filter.hpp:130-138).  out: [time][group][particle][state];
// snap_out: [snapshot][group][particle][state]
int ref_filter_trajectories(const char* name, const double* pars,
                            int n_groups, int n_particles, double time_start,
                            const double* times, int n_times,
                            const double* data, int n_groups_data,
                            double dt, const uint64_t* rng,
                            const int* index_state, int n_index_state,
                            const double* snapshots, int n_snapshots,
                            int select_random, double* ll_out, double* out,
                            double* snap_out, int* select_out, char* err,
                            int err_len) {
  try {
    bool ok = dispatch_discrete(name, [&](auto t, auto s) {
      using T = typename decltype(t)::type;
      using S = typename decltype(s)::type;
      if constexpr (dust2gpu::has_compare_data<S>::value) {
        auto shared = shared_of<S>(pars, n_groups);
        std::vector<typename T::internal_state> internal(n_groups);
        std::vector<uint64_t> seed_filter, seed_system;
        for (int g = 0; g < n_groups; ++g) {
          const uint64_t* it = rng + static_cast<size_t>(g) * 4 *
            (n_particles + 2);
          seed_filter.insert(seed_filter.end(), it, it + 8);
          seed_system.insert(seed_system.end(), it + 8,
                             it + 4 * (n_particles + 2));
        }
        dust2::dust_discrete<T> sys(shared, internal, time_start, dt,
                                    n_particles, seed_system, false, 1);
        std::vector<double> tt(times, times + n_times);
        std::vector<typename S::data_type> d;
        const int nd = sizeof(typename S::data_type) / sizeof(double);
        for (int i = 0; i < n_times * n_groups_data; ++i) {
          d.push_back(S::build_data(data + static_cast<size_t>(i) * nd));
        }
        dust2::filter<dust2::dust_discrete<T>> obj(sys, time_start, tt, d,
                                                   seed_filter);
        std::vector<size_t> is(index_state, index_state + n_index_state);
        std::vector<double> snaps(snapshots, snapshots + n_snapshots);
        obj.run(true, true, snaps, is, obj.sys.all_groups());
        const auto& ll = obj.last_log_likelihood();
        std::copy(ll.begin(), ll.end(), ll_out);
        std::vector<size_t> select;
        if (select_random) {
          select = obj.select_random_particle(obj.sys.all_groups());
          for (int g = 0; g < n_groups; ++g) {
            select_out[g] = static_cast<int>(select[g]);
          }
        }
        obj.last_trajectories().export_state(out, true, select);
        if (n_snapshots > 0) {
          obj.last_trajectories().export_snapshots(snap_out, true, select);
        }
      } else {
        throw std::runtime_error("system has no compare_data");
      }
    });
    if (!ok) {
      throw std::runtime_error(std::string("unknown system ") + name);
    }
    return 0;
  } catch (const std::exception& e) {
    set_err(err, err_len, e.what());
    return 1;
  }
}

// dust2::unfilter (unfilter.hpp:42-73) on a deterministic system seeded
// 42, as r/discrete/unfilter.hpp and r/continuous/unfilter.hpp build it;
// n_runs runs at the same parameters.  ll_out: [n_runs][group][particle];
// state_out: the state after the last run.
int ref_unfilter_run(const char* name, const double* pars, int n_groups,
                     int n_particles, double time_start, const double* times,
                     int n_times, const double* data, int n_groups_data,
                     double dt, int max_steps, double atol, double rtol,
                     double step_size_min, double step_size_max, int n_runs,
                     double* ll_out, double* state_out, char* err,
                     int err_len) {
  try {
    std::vector<double> tt(times, times + n_times);
    std::vector<uint64_t> seed{42};
    auto finish = [&](auto& obj) {
      for (int r = 0; r < n_runs; ++r) {
        obj.run(true, false, {}, {}, obj.sys.all_groups());
        const auto& ll = obj.last_log_likelihood();
        std::copy(ll.begin(), ll.end(),
                  ll_out + static_cast<size_t>(r) * n_groups * n_particles);
      }
      const auto& st = obj.sys.state();
      std::copy(st.begin(), st.end(), state_out);
    };
    // one data entry per group and time (r/helpers.hpp:406-424); shared
    // data is repeated for each group
    auto data_of = [&](auto s) {
      using S = typename decltype(s)::type;
      std::vector<typename S::data_type> d;
      const int nd = sizeof(typename S::data_type) / sizeof(double);
      for (int i = 0; i < n_times; ++i) {
        for (int g = 0; g < n_groups; ++g) {
          const int gd = n_groups_data == 1 ? 0 : g;
          d.push_back(S::build_data(
            data + (static_cast<size_t>(i) * n_groups_data + gd) * nd));
        }
      }
      return d;
    };
    const std::string nm(name);
    if (nm == "sirode") {
      using S = dust2gpu::systems::sirode;
      using T = ref_continuous<S>;
      auto shared = shared_of<S>(pars, n_groups);
      std::vector<typename T::internal_state> internal(n_groups);
      dust2::ode::control<double> ctl(max_steps, atol, rtol, step_size_min,
                                      step_size_max, {}, false, false);
      dust2::dust_continuous<T> sys(shared, internal, time_start, 0, ctl,
                                    n_particles, seed, true, 1);
      dust2::unfilter<dust2::dust_continuous<T>> obj(sys, time_start, tt,
                                                     data_of(tag<S>{}));
      finish(obj);
      return 0;
    }
    if (nm == "malaria") {
      // mixed time: dt is the update interval (0: none)
      using S = dust2gpu::systems::malaria;
      using T = ref_mixed<S>;
      auto shared = shared_of<S>(pars, n_groups);
      std::vector<typename T::internal_state> internal(n_groups);
      dust2::ode::control<double> ctl(max_steps, atol, rtol, step_size_min,
                                      step_size_max, {}, false, false);
      dust2::dust_continuous<T> sys(shared, internal, time_start, dt, ctl,
                                    n_particles, seed, true, 1);
      dust2::unfilter<dust2::dust_continuous<T>> obj(sys, time_start, tt,
                                                     data_of(tag<S>{}));
      finish(obj);
      return 0;
    }
    bool ok = dispatch_discrete(name, [&](auto t, auto s) {
      using T = typename decltype(t)::type;
      using S = typename decltype(s)::type;
      if constexpr (dust2gpu::has_compare_data<S>::value) {
        auto shared = shared_of<S>(pars, n_groups);
        std::vector<typename T::internal_state> internal(n_groups);
        dust2::dust_discrete<T> sys(shared, internal, time_start, dt,
                                    n_particles, seed, true, 1);
        dust2::unfilter<dust2::dust_discrete<T>> obj(sys, time_start, tt,
                                                     data_of(s));
        finish(obj);
      } else {
        throw std::runtime_error("system has no compare_data");
      }
    });
    if (!ok) {
      throw std::runtime_error("unknown system " + nm);
    }
    return 0;
  } catch (const std::exception& e) {
    set_err(err, err_len, e.what());
    return 1;
  }
}

// One unfilter run (run, or run_adjoint when adjoint != 0) saving
// trajectories of the entries index_state (n_index_state 0 = all) and
// snapshots at the data times `snapshots` (unfilter.hpp:42-110), then the
// exports of r/unfilter.hpp:64-125 (no reordering).  traj_out:
// [time][group][particle][entry]; snap_out: [snapshot][group][particle]
// [state]; ll_out: [group][particle].
int ref_unfilter_trajectories(const char* name, const double* pars,
                              int n_groups, int n_particles,
                              double time_start, const double* times,
                              int n_times, const double* data,
                              int n_groups_data, double dt,
                              const int* index_state, int n_index_state,
                              const double* snapshots, int n_snapshots,
                              int adjoint, double* ll_out, double* traj_out,
                              double* snap_out, char* err, int err_len) {
  try {
    std::vector<double> tt(times, times + n_times);
    std::vector<uint64_t> seed{42};
    std::vector<size_t> is(index_state, index_state + n_index_state);
    std::vector<double> snaps(snapshots, snapshots + n_snapshots);
    auto finish = [&](auto& obj, bool use_adjoint) {
      if (use_adjoint) {
        obj.run_adjoint(true, true, snaps, is, obj.sys.all_groups());
      } else {
        obj.run(true, true, snaps, is, obj.sys.all_groups());
      }
      const auto& ll = obj.last_log_likelihood();
      std::copy(ll.begin(), ll.end(), ll_out);
      const auto& tr = obj.last_trajectories();
      tr.export_state(traj_out, false, {});
      if (n_snapshots > 0) {
        tr.export_snapshots(snap_out, false, {});
      }
    };
    auto data_of = [&](auto s) {
      using S = typename decltype(s)::type;
      std::vector<typename S::data_type> d;
      const int nd = sizeof(typename S::data_type) / sizeof(double);
      for (int i = 0; i < n_times; ++i) {
        for (int g = 0; g < n_groups; ++g) {
          const int gd = n_groups_data == 1 ? 0 : g;
          d.push_back(S::build_data(
            data + (static_cast<size_t>(i) * n_groups_data + gd) * nd));
        }
      }
      return d;
    };
    const std::string nm(name);
    if (nm == "sirode") {
      using S = dust2gpu::systems::sirode;
      using T = ref_continuous<S>;
      auto shared = shared_of<S>(pars, n_groups);
      std::vector<typename T::internal_state> internal(n_groups);
      dust2::ode::control<double> ctl(10000, 1e-6, 1e-6,
                                      std::numeric_limits<double>::epsilon(),
                                      std::numeric_limits<double>::infinity(),
                                      {}, false, false);
      dust2::dust_continuous<T> sys(shared, internal, time_start, 0, ctl,
                                    n_particles, seed, true, 1);
      dust2::unfilter<dust2::dust_continuous<T>> obj(sys, time_start, tt,
                                                     data_of(tag<S>{}));
      finish(obj, false);
      return 0;
    }
    if (nm != "sir") {
      throw std::runtime_error("unsupported system " + nm);
    }
    using S = dust2gpu::systems::sir;
    using T = ref_discrete_adjoint<S>;
    auto shared = shared_of<S>(pars, n_groups);
    std::vector<typename T::internal_state> internal(n_groups);
    dust2::dust_discrete<T> sys(shared, internal, time_start, dt, n_particles,
                                seed, true, 1);
    dust2::unfilter<dust2::dust_discrete<T>> obj(sys, time_start, tt,
                                                 data_of(tag<S>{}));
    finish(obj, adjoint != 0);
    return 0;
  } catch (const std::exception& e) {
    set_err(err, err_len, e.what());
    return 1;
  }
}

// unfilter::run_adjoint then last_gradient (unfilter.hpp:77-110,
// 135-142, 188-229) for the sir system, seeded 42, n_particles 1 per
// group; ll_out: [group]; gradient_out: [group][n_gradient]; state_out:
// the state after the run.  The reference copies gradients correctly for
// one particle per group only (adjoint_data.hpp:75-83).
int ref_unfilter_adjoint(const char* name, const double* pars, int n_groups,
                         double time_start, const double* times, int n_times,
                         const double* data, int n_groups_data, double dt,
                         double* ll_out, double* gradient_out,
                         double* state_out, char* err, int err_len) {
  try {
    const std::string nm(name);
    if (nm != "sir") {
      throw std::runtime_error("no adjoint for system " + nm);
    }
    using S = dust2gpu::systems::sir;
    using T = ref_discrete_adjoint<S>;
    std::vector<double> tt(times, times + n_times);
    std::vector<uint64_t> seed{42};
    auto shared = shared_of<S>(pars, n_groups);
    std::vector<typename T::internal_state> internal(n_groups);
    dust2::dust_discrete<T> sys(shared, internal, time_start, dt, 1, seed,
                                true, 1);
    // The reference holds one data entry per group and time
    // (r/helpers.hpp:406-424); shared data is repeated for each group.
    std::vector<typename S::data_type> d;
    const int nd = sizeof(typename S::data_type) / sizeof(double);
    for (int i = 0; i < n_times; ++i) {
      for (int g = 0; g < n_groups; ++g) {
        const int gd = n_groups_data == 1 ? 0 : g;
        d.push_back(S::build_data(
          data + (static_cast<size_t>(i) * n_groups_data + gd) * nd));
      }
    }
    dust2::unfilter<dust2::dust_discrete<T>> obj(sys, time_start, tt, d);
    obj.run_adjoint(true, false, {}, {}, obj.sys.all_groups());
    const auto& ll = obj.last_log_likelihood();
    std::copy(ll.begin(), ll.end(), ll_out);
    obj.last_gradient(gradient_out);
    const auto& st = obj.sys.state();
    std::copy(st.begin(), st.end(), state_out);
    return 0;
  } catch (const std::exception& e) {
    set_err(err, err_len, e.what());
    return 1;
  }
}

// inst/include/dust2/filter_details.hpp:11-39 (w updated in place)
double ref_scale_log_weights(int n, double* w) {
  std::vector<double> v(w, w + n);
  const double ret = dust2::details::scale_log_weights<double>(n, v.begin());
  std::copy(v.begin(), v.end(), w);
  return ret;
}

// inst/include/dust2/filter_details.hpp:45-74
void ref_resample_weight(int n, const double* w, double u, int64_t* idx) {
  std::vector<double> v(w, w + n);
  std::vector<size_t> i(n);
  dust2::details::resample_weight<double>(n, v.cbegin(), u, i.begin());
  for (int k = 0; k < n; ++k) {
    idx[k] = static_cast<int64_t>(i[k]);
  }
}

}  // extern "C"
