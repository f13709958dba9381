// A system class written for dust2 (against compat/dust2/common.hpp),
// adapted to this engine's plugin contract (dust2gpu/system.hpp).
//
// dust2 generates, from a class's `// [[dust2::...]]` annotations, its
// parameter table and the code that turns R lists into the class's
// inputs (inst/template/*.cpp, R/compile.R).  Here a short spec gives the
// same facts, plus the engine's compile-time bound on the state size:
//
//   struct my_spec {
//     using system = my_class;                 // the dust2 class, unchanged
//     static constexpr const char* name = "my_system";
//     static constexpr int n_state_max = 5;    // largest state it may have
//     static constexpr double default_dt = 1;  // discrete time
//     static constexpr dust2gpu::parameter_info parameters[] = {...};
//     static constexpr const char* data_names[] = {"incidence"};
//   };
//   using my_system = dust2gpu::compat::plugin<my_spec>;
//
// The adapter passes the class's build_shared / update_shared /
// build_data a cpp11::list view of the flat parameter (or data) row laid
// out by that table, converts its packing and zero_every, and inherits
// its initial / update / compare_data unchanged.  Entries of `parameters`
// only name and size the row: defaults and required values are the
// class's own (its read_real calls), as in dust2.
#pragma once

#include <iterator>
#include <type_traits>
#include <vector>

#include "dust2/common.hpp"

namespace dust2gpu {
namespace compat {

template <class S, class = void>
struct has_zero_every : std::false_type {};
template <class S>
struct has_zero_every<S, std::void_t<decltype(&S::zero_every)>>
  : std::true_type {};

template <typename Spec>
struct plugin : public Spec::system {
  using S = typename Spec::system;
  using real_type = typename S::real_type;
  using shared_state = typename S::shared_state;
  using internal_state = typename S::internal_state;
  using rng_state_type = random::rng_state;

  static constexpr const char* name = Spec::name;
  static constexpr int n_state_max = Spec::n_state_max;
  static constexpr double default_dt = Spec::default_dt;
  static constexpr const auto& parameters = Spec::parameters;
  static constexpr const auto& data_names = Spec::data_names;

  static_assert(std::is_same<typename S::rng_state_type,
                             random::rng_state>::value,
                "the system's rng_state_type must be "
                "monty::random::generator<real_type>");

  static std::vector<cpp11::list::entry> table(
      const parameter_info* p, std::size_t n) {
    std::vector<cpp11::list::entry> t;
    for (std::size_t i = 0; i < n; ++i) {
      t.push_back({p[i].name, p[i].length});
    }
    return t;
  }

  static const std::vector<cpp11::list::entry>& parameter_table() {
    static const auto t = table(parameters, std::size(parameters));
    return t;
  }

  static cpp11::list parameter_list(const double* row) {
    const auto& t = parameter_table();
    return cpp11::list(t.data(), static_cast<int>(t.size()), row);
  }

  static shared_state build_shared(const double* pars) {
    return S::build_shared(parameter_list(pars));
  }

  // update_pars: entries not given (NaN) keep their value, because the
  // class reads them with the current value as default (sir.cpp:90-94).
  static void update_shared(const double* pars, shared_state& shared) {
    S::update_shared(parameter_list(pars), shared);
  }

  static std::vector<packing_entry> packing_state(
      const shared_state& shared) {
    return S::packing_state(shared);
  }

  static int n_state(const shared_state& shared) {
    const dust2::packing p = S::packing_state(shared);
    return p.size();
  }

  static zero_every_spec zero_every(const shared_state& shared) {
    auto z = zero_every_none();
    if constexpr (has_zero_every<S>::value) {
      for (const auto& entry : S::zero_every(shared)) {
        std::vector<int> index(entry.second.begin(), entry.second.end());
        zero_every_add(z, static_cast<double>(entry.first), index);
      }
    }
    return z;
  }

  // dust2 passes build_data the group's shared state; the engine does
  // too (build_data_of in dust2gpu/system.hpp).
  template <typename D = S>
  static typename D::data_type build_data(const double* row,
                                          const shared_state& shared) {
    static const auto t = table(data_info(), std::size(data_names));
    return S::build_data(
      cpp11::list(t.data(), static_cast<int>(t.size()), row), shared);
  }

private:
  // data fields are scalars
  static const parameter_info* data_info() {
    static const auto info = [] {
      std::vector<parameter_info> v;
      for (const char* nm : data_names) {
        v.push_back(parameter_info{nm, 1, 0.0, false, false});
      }
      return v;
    }();
    return info.data();
  }
};

}  // namespace compat
}  // namespace dust2gpu
