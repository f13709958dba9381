// The system-class plugin contract, GPU edition.
//
// dust2's contract (documented in vignettes/writing.Rmd, examples in
// inst/examples/{sir,sirode,walk}.cpp, detection in
// inst/include/dust2/properties.hpp:13-107) is a class with types
// `real_type`, `shared_state`, `internal_state`, `data_type`,
// `rng_state_type` and static functions `initial`, `update` (discrete
// time) or `rhs` (continuous time), `compare_data`, `build_shared`,
// `update_shared`, `build_data`, `packing_state` and `zero_every`.
//
// The same contract is kept here.  What changes for the GPU:
//   * `initial`, `update`, `rhs`, `output` and `compare_data` are
//     `__host__ __device__` (DUST2_HD) and draw from
//     dust2gpu::random::rng_state;
//   * `shared_state`, `internal_state` and `data_type` must be
//     trivially copyable (they are copied to device memory);
//   * a compile-time bound `n_state_max` sizes the per-thread state
//     arrays, which then live in registers;
//   * `update` must write every element of `state_next` (the engine
//     keeps only two state vectors per particle);
//   * R lists are replaced by flat double arrays laid out by the
//     class's `parameters` table (NaN marks a value that was not given),
//     so the C ABI carries plain pointers;
//   * `zero_every` returns a fixed-size bit-mask table instead of a
//     std::vector of index vectors (inst/include/dust2/zero.hpp:9), so
//     the reset can be applied to register-resident state.
#pragma once

#include <cmath>
#include <cstdint>
#include <iterator>
#include <stdexcept>
#include <string>
#include <type_traits>
#include <vector>

#include "common.hpp"
#include "distributions.hpp"
#include "math.hpp"
#include "random.hpp"

namespace dust2gpu {

// One entry of a system's parameter table.  Array parameters occupy
// `length` consecutive slots of the flat parameter vector.
struct parameter_info {
  const char* name;
  int length;
  double default_value;  // NaN when there is no default
  bool required;
  bool constant;         // not changeable by update_pars
};

// One named block of state (inst/include/dust2/packing.hpp).
struct packing_entry {
  std::string name;
  std::vector<int> dims;
};

// Periodic reset of state entries: before a step starting at time t,
// every state index whose bit is set in mask[i] is zeroed when
// fmod(t, period[i]) == 0 (discrete/system.hpp:413-418).
constexpr int ZERO_EVERY_MAX = 4;
constexpr int ZERO_EVERY_WORDS = 2;  // up to 128 state entries
struct zero_every_spec {
  int n;
  double period[ZERO_EVERY_MAX];
  std::uint64_t mask[ZERO_EVERY_MAX][ZERO_EVERY_WORDS];

  DUST2_HD bool has(int i, int s) const {
    return (mask[i][s >> 6] >> (s & 63)) & 1;
  }
};

inline zero_every_spec zero_every_none() {
  zero_every_spec z{};
  z.n = 0;
  return z;
}

inline void zero_every_add(zero_every_spec& z, double period,
                           const std::vector<int>& index) {
  if (z.n >= ZERO_EVERY_MAX) {
    throw std::runtime_error("Too many zero_every entries");
  }
  z.period[z.n] = period;
  z.mask[z.n][0] = 0;
  z.mask[z.n][1] = 0;
  for (auto s : index) {
    if (s < 0 || s >= 64 * ZERO_EVERY_WORDS) {
      throw std::runtime_error("zero_every index out of range");
    }
    z.mask[z.n][s >> 6] |= static_cast<std::uint64_t>(1) << (s & 63);
  }
  z.n++;
}

// Read parameter `i` of table `T` from a flat vector, applying the
// default when absent and failing when a required value is missing
// (inst/include/dust2/r/helpers.hpp read_real; message as in
// tests/testthat/test-walk.R "A value is expected for 'sd'").
template <typename T>
int parameter_offset(int which) {
  int off = 0;
  for (int i = 0; i < which; ++i) {
    off += T::parameters[i].length;
  }
  return off;
}

template <typename T>
int parameter_length() {
  int len = 0;
  for (std::size_t i = 0; i < std::size(T::parameters); ++i) {
    len += T::parameters[i].length;
  }
  return len;
}

template <typename T>
double read_par(const double* pars, int which) {
  const auto& info = T::parameters[which];
  const double v = pars[parameter_offset<T>(which)];
  if (!std::isnan(v)) {
    return v;
  }
  if (info.required || std::isnan(info.default_value)) {
    throw std::runtime_error(std::string("A value is expected for '") +
                             info.name + "'");
  }
  return info.default_value;
}

// Value for update_pars: NaN keeps the current value.
template <typename T>
double read_par_update(const double* pars, int which, double current) {
  const double v = pars[parameter_offset<T>(which)];
  return std::isnan(v) ? current : v;
}

template <typename T>
void read_par_array(const double* pars, int which, double* dest, int n,
                    bool required) {
  const double* src = pars + parameter_offset<T>(which);
  if (std::isnan(src[0])) {
    if (required) {
      throw std::runtime_error(std::string("A value is expected for '") +
                               T::parameters[which].name + "'");
    }
    return;
  }
  for (int i = 0; i < n; ++i) {
    dest[i] = src[i];
  }
}

// Compile-time feature detection, as inst/include/dust2/properties.hpp.
template <class T, class = void>
struct has_compare_data : std::false_type {};
template <class T>
struct has_compare_data<T, std::void_t<decltype(&T::compare_data)>>
  : std::true_type {};

// Adjoint support (sir.cpp:6 has_adjoint(): adjoint_update,
// adjoint_compare_data, adjoint_initial and packing_gradient).
template <class T, class = void>
struct has_adjoint : std::false_type {};
template <class T>
struct has_adjoint<T, std::void_t<decltype(&T::adjoint_update)>>
  : std::true_type {};

template <class T, class = void>
struct has_output : std::false_type {};
template <class T>
struct has_output<T, std::void_t<decltype(&T::output)>> : std::true_type {};

template <class T, class = void>
struct has_rhs : std::false_type {};
template <class T>
struct has_rhs<T, std::void_t<decltype(&T::rhs)>> : std::true_type {};

template <class T, class = void>
struct has_update : std::false_type {};
template <class T>
struct has_update<T, std::void_t<decltype(&T::update)>> : std::true_type {};

template <typename T>
constexpr bool is_continuous() {
  return has_rhs<T>::value;
}

// Mixed time: an ODE (rhs) with a discrete-time update applied every dt
// (properties.hpp:99 is_mixed_time, continuous/system.hpp:544-585).
template <typename T>
constexpr bool is_mixed_time() {
  return has_rhs<T>::value && has_update<T>::value;
}

// "Special" state: entries after the ODE variables (and before any
// outputs) that the rhs reads but the solver does not integrate; only the
// update changes them (properties.hpp:130-153 size_special,
// do_n_state_special; malaria.cpp's beta).
template <class T, class = void>
struct has_special : std::false_type {};
template <class T>
struct has_special<T, std::void_t<decltype(T::n_special)>>
  : std::true_type {};

template <typename T>
constexpr int n_special() {
  if constexpr (has_special<T>::value) {
    return T::n_special;
  } else {
    return 0;
  }
}

// One data row of a system: `build_data(row)`, or `build_data(row,
// shared)` for systems that read the group's shared state (dust2's
// build_data takes it, e.g. for dimensions: inst/examples/sir.cpp).
template <class T, class = void>
struct build_data_takes_shared : std::false_type {};
template <class T>
struct build_data_takes_shared<T, std::void_t<decltype(T::build_data(
  std::declval<const double*>(),
  std::declval<const typename T::shared_state&>()))>> : std::true_type {};

template <typename T>
typename T::data_type build_data_of(const double* row,
                                    const typename T::shared_state& shared) {
  if constexpr (build_data_takes_shared<T>::value) {
    return T::build_data(row, shared);
  } else {
    return T::build_data(row);
  }
}

// Static checks every system must pass before the engine accepts it.
template <typename T>
constexpr bool check_system() {
  static_assert(std::is_trivially_copyable<typename T::shared_state>::value,
                "shared_state must be trivially copyable");
  static_assert(std::is_trivially_copyable<typename T::internal_state>::value,
                "internal_state must be trivially copyable");
  static_assert(std::is_trivially_copyable<typename T::data_type>::value,
                "data_type must be trivially copyable");
  static_assert(has_rhs<T>::value || has_update<T>::value,
                "a system has update (discrete), rhs (continuous) or both "
                "(mixed time)");
  return true;
}

}  // namespace dust2gpu
