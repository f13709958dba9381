// Per-system factory: builds shared state from the flat parameter table,
// data from the flat data table, and the device engine.  Each system's
// translation unit (systems_*.cu) instantiates this once and registers
// it at load time.
#pragma once

#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

#include "continuous.cuh"
#include "discrete.cuh"
#include "filter.cuh"
#include "lf_table.hpp"
#include "registry.hpp"
#include "served.cuh"
#include "unfilter.cuh"

namespace dust2gpu {
namespace engine {

template <typename T>
std::vector<typename T::shared_state> build_shared_groups(const double* pars,
                                                          int n_groups) {
  const int np = parameter_length<T>();
  std::vector<typename T::shared_state> shared;
  shared.reserve(n_groups);
  int n_state = -1;
  for (int g = 0; g < n_groups; ++g) {
    shared.push_back(T::build_shared(pars + static_cast<std::size_t>(g) * np));
    const int n_g = T::n_state(shared.back());
    // inst/include/dust2/r/helpers.hpp:333-369
    if (g > 0 && n_g != n_state) {
      throw std::runtime_error(
        "State length for group " + std::to_string(g + 1) +
        " was different to previous groups; total length was expected to "
        "be " + std::to_string(n_state) + " but it was " +
        std::to_string(n_g));
    }
    n_state = n_g;
  }
  return shared;
}

template <typename T>
system_api* create_system(const double* pars, int n_groups,
                          const std::vector<int>& n_particles, double time,
                          double dt, const ode_control& control,
                          const std::vector<std::uint64_t>& rng_words,
                          bool deterministic, int tile_size) {
  bind_lf_table();
  auto shared = build_shared_groups<T>(pars, n_groups);
  if constexpr (is_continuous<T>()) {
    // dt is the update interval of a mixed-time system (0: none)
    return new continuous_system<T>(std::move(shared), time, control,
                                    n_particles, rng_words, deterministic,
                                    tile_size, is_mixed_time<T>() ? dt : 0);
  } else {
    return new discrete_system<T>(std::move(shared), time, dt, n_particles,
                                  rng_words, deterministic, tile_size);
  }
}

// The system under a filter: discrete, or mixed time (r/continuous/
// filter.hpp builds a dust_continuous with the dt of the time control).
template <typename T>
auto make_filter_system(std::vector<typename T::shared_state> shared,
                        double time_start, double dt,
                        const ode_control& control,
                        const std::vector<int>& n_particles,
                        const std::vector<std::uint64_t>& words,
                        int tile_size) {
  if constexpr (is_continuous<T>()) {
    return std::make_unique<continuous_system<T>>(
      std::move(shared), time_start, control, n_particles, words, false,
      tile_size, dt);
  } else {
    (void)control;
    return std::make_unique<discrete_system<T>>(
      std::move(shared), time_start, dt, n_particles, words, false,
      tile_size);
  }
}

template <typename T>
filter_api* create_filter(const double* pars, int n_groups,
                          const std::vector<int>& n_particles,
                          double time_start, const double* times, int n_times,
                          const double* data, int n_groups_data, double dt,
                          const ode_control& control,
                          const std::vector<std::uint64_t>& rng_words,
                          int tile_size) {
  if constexpr ((is_continuous<T>() && !is_mixed_time<T>()) ||
                !has_compare_data<T>::value) {
    // R/interface-filter.R:59-65 refuses pure continuous-time systems
    throw std::runtime_error(
      is_continuous<T>() ?
      "Can't use 'dust_filter_create()' with continuous-time models" :
      std::string("Can't create filter; the '") + T::name +
      "' system does not have 'compare_data' support");
  } else {
    bind_lf_table();
    auto shared = build_shared_groups<T>(pars, n_groups);
    // data rows, [time][group] (one group's row when data are shared)
    const int nd = static_cast<int>(sizeof(typename T::data_type) /
                                    sizeof(double));
    std::vector<typename T::data_type> d;
    d.reserve(static_cast<std::size_t>(n_times) * n_groups_data);
    for (int i = 0; i < n_times * n_groups_data; ++i) {
      d.push_back(build_data_of<T>(data + static_cast<std::size_t>(i) * nd,
                                   shared[i % n_groups_data]));
    }
    // Split the stream block (r/discrete/filter.hpp:63-75): per group the
    // first 2 streams go to the filter, the rest to the particles.
    std::vector<std::uint64_t> sys_words;
    std::size_t pos = 0;
    for (int g = 0; g < n_groups; ++g) {
      pos += 8;
      for (int w = 0; w < 4 * n_particles[g]; ++w) {
        sys_words.push_back(rng_words[pos++]);
      }
    }
    auto sys = make_filter_system<T>(std::move(shared), time_start, dt,
                                     control, n_particles, sys_words,
                                     tile_size);
    std::vector<double> t(times, times + n_times);
    return new filter_engine<T>(std::move(sys), time_start, std::move(t),
                                std::move(d), n_groups_data, rng_words);
  }
}

template <typename T>
server_api* create_server(double hbm_budget_bytes, int max_sessions) {
  if constexpr (is_continuous<T>() || !has_compare_data<T>::value) {
    throw std::runtime_error(
      std::string("Can't serve likelihoods of the '") + T::name +
      "' system: it has no discrete-time filter");
  } else {
    bind_lf_table();
    return new served_engine<T>(hbm_budget_bytes, max_sessions);
  }
}

// r/discrete/unfilter.hpp:14-56, r/continuous/unfilter.hpp:14-56: a
// deterministic system (the streams of seed 42, never advanced).
template <typename T>
unfilter_api* create_unfilter(const double* pars, int n_groups,
                              const std::vector<int>& n_particles,
                              double time_start, const double* times,
                              int n_times, const double* data,
                              int n_groups_data, double dt,
                              const ode_control& control) {
  if constexpr (!has_compare_data<T>::value) {
    throw std::runtime_error(
      std::string("Can't create unfilter; the '") + T::name +
      "' system does not have 'compare_data' support");
  } else {
    bind_lf_table();
    auto shared = build_shared_groups<T>(pars, n_groups);
    long n_total = 0;
    for (int n : n_particles) {
      n_total += n;
    }
    const auto words = make_streams_from_seed(42, n_total);
    std::vector<typename T::data_type> d;
    const int nd = static_cast<int>(sizeof(typename T::data_type) /
                                    sizeof(double));
    for (int i = 0; i < n_times * n_groups_data; ++i) {
      d.push_back(build_data_of<T>(data + static_cast<std::size_t>(i) * nd,
                                   shared[i % n_groups_data]));
    }
    std::vector<double> t(times, times + n_times);
    if constexpr (is_continuous<T>()) {
      auto sys = std::make_unique<continuous_system<T>>(
        std::move(shared), time_start, control, n_particles, words, true, 0,
        is_mixed_time<T>() ? dt : 0);
      return new unfilter_engine<T>(std::move(sys), time_start, std::move(t),
                                    std::move(d), n_groups_data);
    } else {
      auto sys = std::make_unique<discrete_system<T>>(
        std::move(shared), time_start, dt, n_particles, words, true);
      return new unfilter_engine<T>(std::move(sys), time_start, std::move(t),
                                    std::move(d), n_groups_data);
    }
  }
}

template <typename T>
struct registrar {
  system_factory factory;
  explicit registrar() {
    factory.name = T::name;
    factory.continuous = is_continuous<T>();
    factory.has_compare = has_compare_data<T>::value;
    factory.info_json = &system_info_json<T>;
    factory.create_system = &create_system<T>;
    factory.create_filter = &create_filter<T>;
    factory.create_server = &create_server<T>;
    factory.create_unfilter = &create_unfilter<T>;
    register_system(&factory);
  }
};

}  // namespace engine
}  // namespace dust2gpu

// One system per translation unit.
#define DUST2_REGISTER_SYSTEM(T)                                          \
  static ::dust2gpu::engine::registrar<T> dust2_registrar_instance
