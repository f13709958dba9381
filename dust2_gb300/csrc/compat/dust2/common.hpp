// dust2's system-authoring API over this engine, so that a system class
// written for dust2 compiles here with one change: `DUST2_HD` on its
// `initial`, `update`, `rhs`, `output` and `compare_data` functions (they
// run on the device).  A source that starts with
//   #include <dust2/common.hpp>
// finds this header when dust2_gb300/csrc/compat is on the include path.
//
// What a system class may use, by dust2's names (reference:
// inst/include/dust2/common.hpp, r/helpers.hpp:482-560, zero.hpp:10,
// packing.hpp; the monty calls of inst/examples/{sir,walk}.cpp):
//   cpp11::list                 the named parameter (or data) list given
//                               to build_shared / update_shared /
//                               build_data; here a view of one flat row
//                               laid out by the system's parameter table
//   dust2::r::read_real/int/size/bool (with or without default),
//   dust2::r::read_real_vector  read from such a list, with dust2's
//                               messages
//   dust2::packing, dust2::zero_every_type<real_type>,
//   dust2::no_data, dust2::no_internal_state
//   monty::random::generator<real_type> (the per-particle stream),
//   monty::random::{random_real, binomial, poisson, exponential_rate,
//   exponential, normal, uniform}, monty::math::{exp, log, lgamma, pow,
//   min, max}, monty::density::{poisson, negative_binomial_mu, binomial,
//   normal}: the engine's samplers and densities (same draws on the host
//   and the device)
//   NA_REAL                     NaN: "no value" for read_real defaults
//
// A compat system is registered through compat/plugin.hpp, which adds
// what dust2 generates from the class's annotations (the parameter
// table, data names) and the engine's compile-time state bound.
#pragma once

#include <cmath>
#include <cstddef>
#include <initializer_list>
#include <limits>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

#include "../../dust2gpu/distributions.hpp"
#include "../../dust2gpu/math.hpp"
#include "../../dust2gpu/random.hpp"
#include "../../dust2gpu/system.hpp"

#ifndef NA_REAL
#define NA_REAL (std::numeric_limits<double>::quiet_NaN())
#endif

namespace cpp11 {

// A named list of numbers: a view of a flat row of doubles laid out by a
// table of (name, length) entries.  An entry whose first value is NaN
// was not given (as a NULL element of dust2's R list).
class list {
public:
  struct entry {
    const char* name;
    int length;
  };

  list(const entry* table, int n_table, const double* row) :
    table_(table), n_table_(n_table), row_(row) {}

  // Values of `name` and their count; nullptr when absent or not given.
  const double* find(const char* name, int* length) const {
    int off = 0;
    for (int i = 0; i < n_table_; ++i) {
      if (std::string(table_[i].name) == name) {
        if (std::isnan(row_[off])) {
          return nullptr;
        }
        *length = table_[i].length;
        return row_ + off;
      }
      off += table_[i].length;
    }
    return nullptr;
  }

private:
  const entry* table_;
  int n_table_;
  const double* row_;
};

}  // namespace cpp11

namespace dust2 {

struct no_data {};
struct no_internal_state {};

// Named blocks of state (packing.hpp): {{"S", {}}, {"x", {n, m}}, ...},
// dimensions of any integer type.
class packing {
public:
  packing(std::initializer_list<
          std::pair<std::string, std::vector<std::size_t>>> blocks) {
    for (const auto& b : blocks) {
      dust2gpu::packing_entry e;
      e.name = b.first;
      for (auto d : b.second) {
        e.dims.push_back(static_cast<int>(d));
      }
      entries_.push_back(e);
    }
  }
  operator std::vector<dust2gpu::packing_entry>() const {
    return entries_;
  }
  // Number of state entries the blocks hold.
  int size() const {
    int n = 0;
    for (const auto& e : entries_) {
      int len = 1;
      for (int d : e.dims) {
        len *= d;
      }
      n += len;
    }
    return n;
  }

private:
  std::vector<dust2gpu::packing_entry> entries_;
};

template <typename real_type>
using zero_every_type =
  std::vector<std::pair<real_type, std::vector<std::size_t>>>;

namespace r {

inline std::string quoted(const char* name) {
  return std::string("'") + name + "'";
}

inline double scalar(cpp11::list pars, const char* name, bool* found) {
  int len = 0;
  const double* v = pars.find(name, &len);
  *found = v != nullptr;
  if (v == nullptr) {
    return 0;
  }
  if (len != 1) {
    throw std::runtime_error("Expected a scalar for " + quoted(name));
  }
  return v[0];
}

inline double read_real(cpp11::list pars, const char* name) {
  bool found;
  const double v = scalar(pars, name, &found);
  if (!found) {
    throw std::runtime_error("A value is expected for " + quoted(name));
  }
  return v;
}

inline double read_real(cpp11::list pars, const char* name,
                        double default_value) {
  bool found;
  const double v = scalar(pars, name, &found);
  return found ? v : default_value;
}

inline int to_int(double v, const char* name) {
  if (!(std::fabs(v - std::round(v)) < 1e-8)) {
    throw std::runtime_error("Expected " + quoted(name) +
                             " to be integer-like");
  }
  return static_cast<int>(std::round(v));
}

inline int read_int(cpp11::list pars, const char* name) {
  return to_int(read_real(pars, name), name);
}

inline int read_int(cpp11::list pars, const char* name, int default_value) {
  bool found;
  const double v = scalar(pars, name, &found);
  return found ? to_int(v, name) : default_value;
}

inline std::size_t to_size(double v, const char* name) {
  const int i = to_int(v, name);
  if (i < 0) {
    throw std::runtime_error("Expected " + quoted(name) +
                             " to be non-negative");
  }
  return static_cast<std::size_t>(i);
}

inline std::size_t read_size(cpp11::list pars, const char* name) {
  return to_size(read_real(pars, name), name);
}

inline std::size_t read_size(cpp11::list pars, const char* name,
                             std::size_t default_value) {
  bool found;
  const double v = scalar(pars, name, &found);
  return found ? to_size(v, name) : default_value;
}

inline bool read_bool(cpp11::list pars, const char* name) {
  return read_real(pars, name) != 0;
}

inline bool read_bool(cpp11::list pars, const char* name,
                      bool default_value) {
  bool found;
  const double v = scalar(pars, name, &found);
  return found ? v != 0 : default_value;
}

template <typename real_type>
void read_real_vector(cpp11::list pars, std::size_t len, real_type* dest,
                      const char* name, bool required) {
  int n = 0;
  const double* v = pars.find(name, &n);
  if (v == nullptr) {
    if (required) {
      throw std::runtime_error("A value is expected for " + quoted(name));
    }
    return;
  }
  if (static_cast<std::size_t>(n) < len) {
    throw std::runtime_error("Expected length " + std::to_string(len) +
                             " for " + quoted(name));
  }
  for (std::size_t i = 0; i < len; ++i) {
    dest[i] = static_cast<real_type>(v[i]);
  }
}

}  // namespace r
}  // namespace dust2

namespace monty {
namespace random {

template <typename real_type>
using generator = dust2gpu::random::rng_state;

template <typename real_type, typename rng_state_type>
DUST2_HD real_type random_real(rng_state_type& rng_state) {
  return dust2gpu::random::random_real(rng_state);
}

template <typename real_type, typename rng_state_type>
DUST2_HD real_type binomial(rng_state_type& rng_state, real_type n,
                            real_type p) {
  return dust2gpu::random::binomial(rng_state, n, p);
}

template <typename real_type, typename rng_state_type>
DUST2_HD real_type poisson(rng_state_type& rng_state, real_type lambda) {
  return dust2gpu::random::poisson(rng_state, lambda);
}

template <typename real_type, typename rng_state_type>
DUST2_HD real_type exponential_rate(rng_state_type& rng_state,
                                    real_type rate) {
  return dust2gpu::random::exponential_rate(rng_state, rate);
}

template <typename real_type, typename rng_state_type>
DUST2_HD real_type exponential(rng_state_type& rng_state, real_type rate) {
  return dust2gpu::random::exponential_rate(rng_state, rate);
}

template <typename real_type, typename rng_state_type>
DUST2_HD real_type normal(rng_state_type& rng_state, real_type mean,
                          real_type sd) {
  return dust2gpu::random::normal(rng_state, mean, sd);
}

template <typename real_type, typename rng_state_type>
DUST2_HD real_type uniform(rng_state_type& rng_state, real_type min,
                           real_type max) {
  return dust2gpu::random::uniform(rng_state, min, max);
}

}  // namespace random

namespace math {

template <typename T>
DUST2_HD T exp(T x) {
  return dust2gpu::math::exp(x);
}

template <typename T>
DUST2_HD T log(T x) {
  return dust2gpu::math::log(x);
}

template <typename T>
DUST2_HD T lgamma(T x) {
  return dust2gpu::math::lgamma(x);
}

template <typename T>
DUST2_HD T pow(T x, T y) {
  return ::pow(x, y);
}

template <typename T>
DUST2_HD T min(T a, T b) {
  return a < b ? a : b;
}

template <typename T>
DUST2_HD T max(T a, T b) {
  return a > b ? a : b;
}

}  // namespace math

namespace density {

template <typename T>
DUST2_HD T poisson(T x, T lambda, bool log) {
  return dust2gpu::density::poisson(x, lambda, log);
}

template <typename T>
DUST2_HD T negative_binomial_mu(T x, T size, T mu, bool log) {
  return dust2gpu::density::negative_binomial_mu(x, size, mu, log);
}

template <typename T>
DUST2_HD T binomial(T x, T size, T prob, bool log) {
  return dust2gpu::density::binomial(x, size, prob, log);
}

template <typename T>
DUST2_HD T normal(T x, T mu, T sd, bool log) {
  return dust2gpu::density::normal(x, mu, sd, log);
}

}  // namespace density
}  // namespace monty
