// Registry of the systems compiled into the library.  dust2 generates one
// set of `dust2_<component>_<system>_<verb>` entry points per system
// (inst/template/*.cpp, src/cpp11.cpp); here each system registers one
// factory and the C ABI dispatches on the system name at allocation.
#pragma once

#include <cstdint>
#include <memory>
#include <sstream>
#include <string>
#include <vector>

#include "../dust2gpu/system.hpp"
#include "api.hpp"
#include "seeding.hpp"
#include "server_api.hpp"

namespace dust2gpu {
namespace engine {

struct system_factory {
  const char* name;
  bool continuous;
  bool has_compare;
  std::string (*info_json)();
  system_api* (*create_system)(const double* pars, int n_groups,
                               const std::vector<int>& n_particles,
                               double time, double dt,
                               const ode_control& control,
                               const std::vector<std::uint64_t>& rng_words,
                               bool deterministic, int tile_size);
  filter_api* (*create_filter)(const double* pars, int n_groups,
                               const std::vector<int>& n_particles,
                               double time_start, const double* times,
                               int n_times, const double* data,
                               int n_groups_data, double dt,
                               const ode_control& control,
                               const std::vector<std::uint64_t>& rng_words,
                               int tile_size);
  // nullptr for systems without a filter (continuous time, no compare).
  server_api* (*create_server)(double hbm_budget_bytes, int max_sessions);
  unfilter_api* (*create_unfilter)(const double* pars, int n_groups,
                                   const std::vector<int>& n_particles,
                                   double time_start, const double* times,
                                   int n_times, const double* data,
                                   int n_groups_data, double dt,
                                   const ode_control& control);
};

void register_system(const system_factory* f);
const system_factory* find_system(const char* name);
std::vector<const system_factory*> all_systems();

// JSON description of a system's parameter table and packing, used by
// the host-side mirror of dust2's R layer.
template <typename T>
std::string system_info_json() {
  std::ostringstream s;
  s.precision(17);
  s << "{\"name\": \"" << T::name << "\", \"time_type\": \""
    << (is_mixed_time<T>() ? "mixed" :
        is_continuous<T>() ? "continuous" : "discrete") << "\""
    << ", \"has_compare\": "
    << (has_compare_data<T>::value ? "true" : "false")
    << ", \"has_adjoint\": "
    << (has_adjoint<T>::value && !is_continuous<T>() ? "true" : "false")
    << ", \"n_state_max\": " << T::n_state_max;
  if constexpr (!is_continuous<T>()) {
    s << ", \"default_dt\": " << T::default_dt;
  }
  s << ", \"parameters\": [";
  for (std::size_t i = 0; i < std::size(T::parameters); ++i) {
    const auto& p = T::parameters[i];
    s << (i ? ", " : "") << "{\"name\": \"" << p.name << "\", \"length\": "
      << p.length << ", \"default\": ";
    if (std::isnan(p.default_value)) {
      s << "null";
    } else {
      s << p.default_value;
    }
    s << ", \"required\": " << (p.required ? "true" : "false")
      << ", \"constant\": " << (p.constant ? "true" : "false") << "}";
  }
  s << "], \"data\": [";
  if constexpr (has_compare_data<T>::value) {
    for (std::size_t i = 0; i < std::size(T::data_names); ++i) {
      s << (i ? ", " : "") << "\"" << T::data_names[i] << "\"";
    }
  }
  s << "]}";
  return s.str();
}

}  // namespace engine
}  // namespace dust2gpu
