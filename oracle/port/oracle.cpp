// TEST INFRASTRUCTURE (oracle).  A plain C++ restatement of dust2's CPU
// engine for the hot path, used only by tests/, the smoke check and the
// CPU-baseline leg of bench.py -- never by the product.  It is written
// independently of the CUDA engine, following the reference's code
// structure function by function (citations are to the dust2 source
// tree), and shares with the engine only what must be shared for
// bit-identical draws: the system classes (the plugin code a user
// writes) and the project's restatement of monty's generator and
// samplers (dust2_gb300/csrc/dust2gpu/).
//
// Parallelism mirrors the reference: an OpenMP loop over particles for
// stepping, initial conditions and compare (discrete/system.hpp:67-69),
// everything else serial.  Groups may have different particle counts
// (each group is then exactly a dust2 filter of its own size).
//
// Build: g++ -std=c++17 -O2 -fopenmp -ffp-contract=off (oracle/build.py).
#include <omp.h>

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <limits>
#include <numeric>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

#include "engine/error_text.hpp"
#include "systems/logistic.hpp"
#include "systems/malaria.hpp"
#include "systems/seir_age.hpp"
#include "systems/sir.hpp"
#include "systems/sir_cases.hpp"
#include "systems/sirode.hpp"
#include "systems/sirs.hpp"
#include "systems/walk.hpp"

namespace {

using rng_t = dust2gpu::random::rng_state;
using zero_list = std::vector<std::pair<double, std::vector<int>>>;

template <typename T>
struct tag {
  using type = T;
};

template <typename F>
bool dispatch_discrete(const std::string& name, F f) {
  using namespace dust2gpu::systems;
  if (name == "sir") {
    f(tag<sir>{});
  } else if (name == "sir_cases") {
    f(tag<sir_cases>{});
  } else if (name == "walk") {
    f(tag<walk>{});
  } else if (name == "seir_age") {
    f(tag<seir_age>{});
  } else if (name == "sirs") {
    f(tag<dust2gpu::systems::sirs>{});
  } else {
    return false;
  }
  return true;
}

template <typename S>
zero_list zero_every_of(const typename S::shared_state& shared) {
  const auto z = S::zero_every(shared);
  zero_list ret;
  for (int i = 0; i < z.n; ++i) {
    std::vector<int> idx;
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
std::vector<typename S::shared_state> shared_of(const double* pars,
                                                int n_groups) {
  const int np = dust2gpu::parameter_length<S>();
  std::vector<typename S::shared_state> ret;
  for (int g = 0; g < n_groups; ++g) {
    ret.push_back(S::build_shared(pars + static_cast<size_t>(g) * np));
  }
  return ret;
}

std::vector<rng_t> make_rng(const uint64_t* words, size_t n,
                            bool deterministic) {
  std::vector<rng_t> r(n);
  for (size_t k = 0; k < n; ++k) {
    for (int w = 0; w < 4; ++w) {
      r[k].state[w] = words[4 * k + w];
    }
    r[k].deterministic = deterministic;
    r[k].err = 0;
    r[k].err_v0 = 0;
    r[k].err_v1 = 0;
  }
  return r;
}

// Per-particle error capture and the summary of errors.hpp:29-54.
struct errors {
  std::vector<dust2gpu::particle_error> e;
  explicit errors(size_t n) : e(n, dust2gpu::particle_error{0, 0, 0}) {}
  void capture(size_t k, rng_t& r) {
    if (r.err != 0 && e[k].code == 0) {
      e[k] = dust2gpu::particle_error{r.err, r.err_v0, r.err_v1};
    }
    r.err = 0;
  }
  void report() const {
    size_t count = 0;
    for (auto& el : e) {
      count += el.code != 0;
    }
    if (count == 0) {
      return;
    }
    std::string msg = std::to_string(count) + " particles reported errors.";
    size_t j = 0;
    for (size_t i = 0; i < e.size() && j < 4; ++i) {
      if (e[i].code != 0) {
        msg += "\n  - " + std::to_string(i + 1) + ": " +
          dust2gpu::error_text(e[i]);
        ++j;
      }
    }
    if (j < count) {
      msg += "\n  - (and " + std::to_string(count - j) + " more)";
    }
    throw std::runtime_error(msg);
  }
};

// The stepping loop of discrete/system.hpp:404-423.
template <typename S>
void run_particle(double time, double dt, size_t n_steps,
                  const typename S::shared_state& shared,
                  typename S::internal_state& internal,
                  const zero_list& zero_every, double* state, rng_t& rng,
                  double* state_next) {
  for (size_t i = 0; i < n_steps; ++i) {
    const double time_i = time + i * dt;
    for (const auto& el : zero_every) {
      if (std::fmod(time_i, el.first) == 0) {
        for (const auto j : el.second) {
          state[j] = 0;
        }
      }
    }
    S::update(time_i, dt, state, shared, internal, rng, state_next);
    std::swap(state, state_next);
  }
}

// A set of groups with per-group particle counts, in dust2's AoS layout:
// particle k (global, group-major) owns state[k*n_state .. +n_state).
template <typename S>
struct discrete_sys {
  std::vector<typename S::shared_state> shared;
  std::vector<int> n_particles;
  std::vector<size_t> offset;
  size_t n_total;
  int n_state;
  double time;
  double dt;
  std::vector<double> state, state_next;
  std::vector<rng_t> rng;
  std::vector<zero_list> zero_every;
  int n_threads;
  errors err;

  discrete_sys(std::vector<typename S::shared_state> sh, std::vector<int> np,
               double time_, double dt_, const uint64_t* rng_words,
               bool deterministic, int threads) :
    shared(std::move(sh)), n_particles(std::move(np)),
    n_total(0), n_state(S::n_state(shared[0])), time(time_), dt(dt_),
    n_threads(threads), err(0) {
    for (int n : n_particles) {
      offset.push_back(n_total);
      n_total += n;
    }
    state.assign(n_total * n_state, 0.0);
    state_next.assign(n_total * n_state, 0.0);
    rng = make_rng(rng_words, n_total, deterministic);
    for (auto& s : shared) {
      zero_every.push_back(zero_every_of<S>(s));
    }
    err = errors(n_total);
  }

  int group_of(size_t k) const {
    return static_cast<int>(
      std::upper_bound(offset.begin(), offset.end(), k) - offset.begin()) - 1;
  }

  // discrete/system.hpp:130-152
  void set_state_initial() {
#pragma omp parallel for schedule(static) num_threads(n_threads)
    for (long k = 0; k < static_cast<long>(n_total); ++k) {
      const int g = group_of(k);
      typename S::internal_state internal{};
      S::initial(time, shared[g], internal, rng[k], state.data() + k * n_state);
      err.capture(k, rng[k]);
    }
    err.report();
  }

  // discrete/system.hpp:61-92, restricted to `active` groups
  void run_to_time(double t, const std::vector<char>& active) {
    const size_t n_steps = std::round(std::max(0.0, t - time) / dt);
#pragma omp parallel for schedule(static) num_threads(n_threads)
    for (long k = 0; k < static_cast<long>(n_total); ++k) {
      const int g = group_of(k);
      if (!active[g]) {
        continue;
      }
      typename S::internal_state internal{};
      run_particle<S>(time, dt, n_steps, shared[g], internal, zero_every[g],
                      state.data() + k * n_state, rng[k],
                      state_next.data() + k * n_state);
      err.capture(k, rng[k]);
    }
    err.report();
    if (n_steps % 2 == 1) {
      std::swap(state, state_next);
    }
    time = time + n_steps * dt;
  }

  // discrete/system.hpp:259-287
  template <typename D>
  void compare_data(const D* data, int n_groups_data,
                    const std::vector<char>& active, double* out) {
#pragma omp parallel for schedule(static) num_threads(n_threads)
    for (long k = 0; k < static_cast<long>(n_total); ++k) {
      const int g = group_of(k);
      if (!active[g]) {
        continue;
      }
      typename S::internal_state internal{};
      out[k] = S::compare_data(time, state.data() + k * n_state,
                               data[n_groups_data == 1 ? 0 : g], shared[g],
                               internal, rng[k]);
      err.capture(k, rng[k]);
    }
    err.report();
  }

  // discrete/system.hpp:169-181 (index is group-local)
  void reorder(const std::vector<size_t>& index,
               const std::vector<char>& active) {
    for (size_t k_to = 0; k_to < n_total; ++k_to) {
      const int g = group_of(k_to);
      const size_t k_from = active[g] ? offset[g] + index[k_to] : k_to;
      std::copy_n(state.begin() + k_from * n_state, n_state,
                  state_next.begin() + k_to * n_state);
    }
    std::swap(state, state_next);
  }
};

// filter_details.hpp:11-39
double scale_log_weights(size_t n, double* w) {
  if (n == 1) {
    return *w;
  }
  constexpr double neg_infinity = -std::numeric_limits<double>::infinity();
  double max_w = neg_infinity;
  for (size_t i = 0; i < n; ++i) {
    if (std::isnan(w[i])) {
      w[i] = neg_infinity;
    } else {
      max_w = std::max(max_w, w[i]);
    }
  }
  if (max_w == neg_infinity) {
    return max_w;
  }
  double tot = 0.0;
  for (size_t i = 0; i < n; ++i) {
    w[i] = std::exp(w[i] - max_w);
    tot += w[i];
  }
  return std::log(tot / n) + max_w;
}

// filter_details.hpp:45-74
void resample_weight(size_t n, const double* w, double u, size_t* idx) {
  double tot = 0.0;
  for (size_t i = 0; i < n; ++i) {
    tot += w[i];
  }
  const double uu0 = tot * u / n;
  const double du = tot / n;
  double ww = 0.0;
  size_t j = 0;
  for (size_t i = 0; i < n; ++i) {
    const double uu = uu0 + i * du;
    while (ww < uu && j < n) {
      ww += w[j];
      ++j;
    }
    idx[i] = j == 0 ? 0 : j - 1;
  }
}

// filter.hpp:42-104 for groups of (possibly) different sizes; each group
// owns the stream block [2 filter streams | n_g particle streams].
template <typename S>
struct filter_port {
  discrete_sys<S> sys;
  double time_start;
  std::vector<double> times;
  std::vector<typename S::data_type> data;
  int n_groups_data;
  std::vector<rng_t> frng;
  std::vector<double> ll;
  // trajectories (filter.hpp:89-100): per data time the post-reorder
  // state entries index_state of every particle, and the indices
  bool save = false;
  std::vector<int> index_state;
  std::vector<std::vector<double>> hist_state;
  std::vector<std::vector<size_t>> hist_order;
  std::vector<int> snap_obs;  // data time indices of snapshots
  std::vector<std::vector<double>> snaps;

  static std::vector<uint64_t> system_words(const uint64_t* rng,
                                            const std::vector<int>& np) {
    std::vector<uint64_t> ret;
    size_t pos = 0;
    for (int n : np) {
      pos += 8;
      ret.insert(ret.end(), rng + pos, rng + pos + 4 * n);
      pos += 4 * n;
    }
    return ret;
  }

  filter_port(std::vector<typename S::shared_state> shared,
              std::vector<int> np, double time_start_, const double* t,
              int n_times, const double* d, int n_groups_data_, double dt,
              const uint64_t* rng, int n_threads) :
    sys(std::move(shared), np, time_start_, dt,
        system_words(rng, np).data(), false, n_threads),
    time_start(time_start_), times(t, t + n_times),
    n_groups_data(n_groups_data_) {
    const int nd = sizeof(typename S::data_type) / sizeof(double);
    for (int i = 0; i < n_times * n_groups_data; ++i) {
      data.push_back(dust2gpu::build_data_of<S>(
        d + static_cast<size_t>(i) * nd, sys.shared[i % n_groups_data]));
    }
    size_t pos = 0;
    for (int n : np) {
      auto f = make_rng(rng + pos, 2, false);
      frng.insert(frng.end(), f.begin(), f.end());
      pos += 4 * (2 + n);
    }
    ll.assign(np.size(), 0);
  }

  void run(const double* initial, const std::vector<char>& active) {
    const size_t G = sys.n_particles.size();
    std::fill(ll.begin(), ll.end(), 0);
    sys.time = time_start;
    if (initial != nullptr) {
      std::copy_n(initial, sys.state.size(), sys.state.begin());
      sys.err = errors(sys.n_total);
    } else {
      const std::vector<char> all(G, 1);
      (void)all;
      sys.set_state_initial();
    }
    std::vector<double> w(sys.n_total);
    std::vector<size_t> index(sys.n_total);
    for (size_t it = 0; it < times.size(); ++it) {
      sys.run_to_time(times[it], active);
      sys.compare_data(data.data() + it * n_groups_data, n_groups_data,
                       active, w.data());
      for (size_t g = 0; g < G; ++g) {
        if (!active[g]) {
          continue;
        }
        const size_t n = sys.n_particles[g];
        double* wg = w.data() + sys.offset[g];
        size_t* idx = index.data() + sys.offset[g];
        const bool reorder_this_group =
          std::any_of(wg, wg + n, [](double v) { return v != 0; });
        if (reorder_this_group) {
          ll[g] += scale_log_weights(n, wg);
          const double u = dust2gpu::random::random_real(frng[2 * g]);
          resample_weight(n, wg, u, idx);
        } else {
          for (size_t j = 0; j < n; ++j) {
            idx[j] = j;
          }
        }
      }
      sys.reorder(index, active);
      if (save) {
        std::vector<double> st;
        for (size_t k = 0; k < sys.n_total; ++k) {
          for (int j : index_state) {
            st.push_back(sys.state[k * sys.n_state + j]);
          }
        }
        hist_state.push_back(st);
        hist_order.push_back(index);
      }
      if (std::find(snap_obs.begin(), snap_obs.end(),
                    static_cast<int>(it)) != snap_obs.end()) {
        snaps.push_back(sys.state);
      }
    }
  }

  // trajectories.hpp:199-268 with reorder: out [snapshot][group]
  // [particle][state]
  void export_snapshots(const int* select, double* out) const {
    const size_t n_t = hist_order.size();
    const size_t ns = sys.n_state;
    const size_t G = sys.n_particles.size();
    size_t n_out = select != nullptr ? 1 : sys.n_particles[0];
    for (size_t g = 0; g < G; ++g) {
      for (size_t jo = 0; jo < n_out; ++jo) {
        size_t j = select != nullptr ? select[g] : jo;
        long sn = static_cast<long>(snap_obs.size()) - 1;
        for (size_t irev = 0; irev < n_t && sn >= 0; ++irev) {
          const size_t i = n_t - 1 - irev;
          const size_t k = sys.offset[g] + j;
          if (snap_obs[sn] == static_cast<int>(i)) {
            double* dst = out + ((sn * G + g) * n_out + jo) * ns;
            for (size_t s2 = 0; s2 < ns; ++s2) {
              dst[s2] = snaps[sn][k * ns + s2];
            }
            --sn;
          }
          j = hist_order[i][k];
        }
      }
    }
  }

  // trajectories.hpp:135-190: each output particle of each group (all, or
  // select[g]) followed back through the saved indices.
  // out: [time][group][particle][state]
  void export_trajectories(const int* select, double* out) const {
    const size_t n_t = hist_state.size();
    const size_t ns = index_state.size();
    const size_t G = sys.n_particles.size();
    size_t n_out = select != nullptr ? 1 : sys.n_particles[0];
    for (size_t g = 0; g < G; ++g) {
      for (size_t jo = 0; jo < n_out; ++jo) {
        size_t j = select != nullptr ? select[g] : jo;
        for (size_t irev = 0; irev < n_t; ++irev) {
          const size_t i = n_t - 1 - irev;
          const size_t k = sys.offset[g] + j;
          double* dst = out + ((i * G + g) * n_out + jo) * ns;
          for (size_t s2 = 0; s2 < ns; ++s2) {
            dst[s2] = hist_state[i][k * ns + s2];
          }
          j = hist_order[i][k];
        }
      }
    }
  }
};

// ---- dopri5 (continuous/solver.hpp) ------------------------------------

struct ode_ctl {
  size_t max_steps;
  double atol, rtol, step_size_min, step_size_max;
  double factor_safe = 0.9, factor_min = 0.2, factor_max = 10.0;
  double beta = 0.04, constant = 0.2 - 0.04 * 0.75;
  std::vector<double> critical_times;
};

// ode::internals (solver.hpp:35-73), without history or events
struct ode_internals {
  double t0 = 0, t1 = 0, h = 0;
  std::vector<double> c1, c2, c3, c4, c5, dydt;
  double step_size = 0, error = 0;
  size_t n_steps = 0, n_steps_accepted = 0, n_steps_rejected = 0;
  explicit ode_internals(size_t n) :
    c1(n), c2(n), c3(n), c4(n), c5(n), dydt(n) {}
};

template <typename S>
struct dopri5_port {
  const ode_ctl& ctl;
  const typename S::shared_state& shared;
  size_t n;
  std::vector<double> y_next, y_stiff, k2, k3, k4, k5, k6;
  double facc1, facc2;

  dopri5_port(const ode_ctl& c, const typename S::shared_state& sh,
              size_t n_var) :
    ctl(c), shared(sh), n(n_var), y_next(n_var), y_stiff(n_var), k2(n_var),
    k3(n_var), k4(n_var), k5(n_var), k6(n_var),
    facc1(1 / c.factor_min), facc2(1 / c.factor_max) {}

  // special state (mixed-time systems) following the n ODE variables:
  // read by the rhs, constant through a run (solver.hpp:236-239)
  std::vector<double> special;

  void set_special(const double* y) {
    std::copy(y + n, y + n + special.size(), special.begin());
  }

  void rhs(double t, const double* y, double* dy) {
    typename S::internal_state internal{};
    // systems may read state beyond the ODE variables (specials,
    // outputs); pass a buffer large enough for the full state
    double buf[S::n_state_max] = {};
    std::copy_n(y, n, buf);
    std::copy(special.begin(), special.end(), buf + n);
    double out[S::n_state_max] = {};
    S::rhs(t, buf, shared, internal, out);
    std::copy_n(out, n, dy);
  }

  static constexpr double C2 = 0.2, C3 = 0.3, C4 = 0.8, C5 = 8.0 / 9.0;
  static constexpr double A21 = 0.2, A31 = 3.0 / 40.0, A32 = 9.0 / 40.0;
  static constexpr double A41 = 44.0 / 45.0, A42 = -56.0 / 15.0,
    A43 = 32.0 / 9.0;
  static constexpr double A51 = 19372.0 / 6561.0, A52 = -25360.0 / 2187.0,
    A53 = 64448.0 / 6561.0, A54 = -212.0 / 729.0;
  static constexpr double A61 = 9017.0 / 3168.0, A62 = -355.0 / 33.0,
    A63 = 46732.0 / 5247.0, A64 = 49.0 / 176.0, A65 = -5103.0 / 18656.0;
  static constexpr double A71 = 35.0 / 384.0, A73 = 500.0 / 1113.0,
    A74 = 125.0 / 192.0, A75 = -2187.0 / 6784.0, A76 = 11.0 / 84.0;
  static constexpr double E1 = 71.0 / 57600.0, E3 = -71.0 / 16695.0,
    E4 = 71.0 / 1920.0, E5 = -17253.0 / 339200.0, E6 = 22.0 / 525.0,
    E7 = -1.0 / 40.0;
  static constexpr double D1 = -12715105075.0 / 11282082432.0,
    D3 = 87487479700.0 / 32700410799.0, D4 = -10690763975.0 / 1880347072.0,
    D5 = 701980252875.0 / 199316789632.0, D6 = -1453857185.0 / 822651844.0,
    D7 = 69997945.0 / 29380423.0;

  // solver.hpp:96-149
  double try_step(double t, double h, const double* y, const double* k1,
                  double* c5) {
    const double t_next = t + h;
    for (size_t i = 0; i < n; ++i) y_next[i] = y[i] + h * A21 * k1[i];
    rhs(t + C2 * h, y_next.data(), k2.data());
    for (size_t i = 0; i < n; ++i)
      y_next[i] = y[i] + h * (A31 * k1[i] + A32 * k2[i]);
    rhs(t + C3 * h, y_next.data(), k3.data());
    for (size_t i = 0; i < n; ++i)
      y_next[i] = y[i] + h * (A41 * k1[i] + A42 * k2[i] + A43 * k3[i]);
    rhs(t + C4 * h, y_next.data(), k4.data());
    for (size_t i = 0; i < n; ++i)
      y_next[i] = y[i] + h * (A51 * k1[i] + A52 * k2[i] + A53 * k3[i] +
                              A54 * k4[i]);
    rhs(t + C5 * h, y_next.data(), k5.data());
    for (size_t i = 0; i < n; ++i)
      y_stiff[i] = y[i] + h * (A61 * k1[i] + A62 * k2[i] + A63 * k3[i] +
                               A64 * k4[i] + A65 * k5[i]);
    rhs(t_next, y_stiff.data(), k6.data());
    for (size_t i = 0; i < n; ++i)
      y_next[i] = y[i] + h * (A71 * k1[i] + A73 * k3[i] + A74 * k4[i] +
                              A75 * k5[i] + A76 * k6[i]);
    rhs(t_next, y_next.data(), k2.data());
    for (size_t i = 0; i < n; ++i)
      c5[i] = h * (D1 * k1[i] + D3 * k3[i] + D4 * k4[i] + D5 * k5[i] +
                   D6 * k6[i] + D7 * k2[i]);
    for (size_t i = 0; i < n; ++i)
      k4[i] = h * (E1 * k1[i] + E3 * k3[i] + E4 * k4[i] + E5 * k5[i] +
                   E6 * k6[i] + E7 * k2[i]);
    double err = 0.0;
    for (size_t i = 0; i < n; ++i) {
      const double sk = k4[i] / (ctl.atol + ctl.rtol *
                                 std::max(std::abs(y[i]), std::abs(y_next[i])));
      err += sk * sk;
    }
    return std::sqrt(err / n);
  }

  // solver.hpp:153-229
  double step(double t, double t_end, double* y, ode_internals& in) {
    bool success = false, reject = false, truncated = false;
    double h = in.step_size;
    while (!success) {
      if (in.n_steps > ctl.max_steps) {
        throw std::runtime_error("too many steps");
      }
      if (h < ctl.step_size_min) {
        throw std::runtime_error("step too small");
      }
      if (h <= std::abs(t) * std::numeric_limits<double>::epsilon()) {
        throw std::runtime_error("step size vanished");
      }
      truncated = t + h > t_end;
      if (truncated) {
        h = t_end - t;
      }
      const double err = try_step(t, h, y, in.dydt.data(), in.c5.data());
      in.n_steps++;
      const double fac11 = std::pow(err, ctl.constant);
      if (err <= 1) {
        success = true;
        in.t0 = t;
        in.t1 = t + h;
        in.h = h;
        for (size_t i = 0; i < n; ++i) {
          const double ydiff = y_next[i] - y[i];
          const double bspl = h * in.dydt[i] - ydiff;
          in.c1[i] = y[i];
          in.c2[i] = ydiff;
          in.c3[i] = bspl;
          in.c4[i] = -h * k2[i] + ydiff - bspl;
        }
        std::copy_n(k2.begin(), n, in.dydt.begin());
        std::copy_n(y_next.begin(), n, y);
        in.n_steps_accepted++;
        if (!truncated) {
          const double fac_old = std::max(in.error, 1e-4);
          double fac = fac11 / std::pow(fac_old, ctl.beta);
          fac = std::max(std::min(fac / ctl.factor_safe, facc1), facc2);
          const double h_new = h / fac;
          const double h_max = reject ? h : ctl.step_size_max;
          in.step_size = std::min(h_new, h_max);
          in.error = err;
        }
      } else {
        reject = true;
        if (in.n_steps_accepted >= 1) {
          in.n_steps_rejected++;
        }
        h /= std::min(facc1, fac11 / ctl.factor_safe);
      }
    }
    return truncated ? t_end : t + h;
  }

  // history_step::interpolate into c4 (solver.hpp:456-461)
  void interpolate_into_c4(double t_reset, const std::vector<int>& index,
                           double* y, ode_internals& in) {
    const double u = (t_reset - in.t0) / in.h;
    const double v = 1 - u;
    size_t r = 0;
    for (auto i : index) {
      in.c4[r++] = in.c1[i] + u * (in.c2[i] + v * (in.c3[i] + u *
                                   (in.c4[i] + v * in.c5[i])));
    }
    for (size_t q = 0; q < index.size(); ++q) {
      y[index[q]] -= in.c4[q];
    }
  }

  // solver.hpp:437-465
  void apply_zero_every(double t, double* y, const zero_list& z,
                        ode_internals& in) {
    if (z.empty() || in.h == 0) {
      return;
    }
    for (const auto& el : z) {
      const double period = el.first;
      const int nn = std::floor(t / period);
      const int m = std::floor(in.t0 / period);
      if (nn > m) {
        const double t_reset = nn * period;
        if (t_reset == t) {
          for (auto j : el.second) {
            y[j] = 0;
          }
        } else {
          interpolate_into_c4(t_reset, el.second, y, in);
        }
      }
    }
  }

  // solver.hpp:468-492
  void apply_zero_every_final(double t, double* y, const zero_list& z,
                              ode_internals& in) {
    if (z.empty() || in.h == 0) {
      return;
    }
    for (const auto& el : z) {
      const double period = el.first;
      if (in.h > period) {
        const int nn = std::ceil(t / period);
        const int m = std::ceil(in.t0 / period);
        if (nn > m) {
          interpolate_into_c4((nn - 1) * period, el.second, y, in);
        }
      }
    }
  }

  // solver.hpp:232-262
  void run(double t, double t_end, double* y, const zero_list& z,
           ode_internals& in) {
    set_special(y);
    const auto& ct = ctl.critical_times;
    if (ct.empty()) {
      while (t < t_end) {
        apply_zero_every(t, y, z, in);
        t = step(t, t_end, y, in);
      }
    } else {
      auto tc = std::upper_bound(ct.begin(), ct.end(), t);
      double t_end_i = (tc == ct.end() || *tc >= t_end) ? t_end : *tc;
      while (t < t_end) {
        apply_zero_every(t, y, z, in);
        t = step(t, t_end_i, y, in);
        if (t >= t_end_i && t < t_end) {
          ++tc;
          t_end_i = (tc == ct.end() || *tc >= t_end) ? t_end : *tc;
        }
      }
    }
    apply_zero_every_final(t, y, z, in);
  }

  // solver.hpp:265-324
  void initialise(double t, const double* y, ode_internals& in) {
    set_special(y);
    in.step_size = 0;
    in.error = 0;
    in.n_steps = 0;
    in.n_steps_accepted = 0;
    in.n_steps_rejected = 0;
    double* f0 = in.dydt.data();
    double* f1 = k3.data();
    double* y1 = y_next.data();
    rhs(t, y, f0);
    double norm_f = 0.0, norm_y = 0.0;
    for (size_t i = 0; i < n; ++i) {
      const double sk = ctl.atol + ctl.rtol * std::abs(y[i]);
      norm_f += (f0[i] / sk) * (f0[i] / sk);
      norm_y += (y[i] / sk) * (y[i] / sk);
    }
    double h = (norm_f <= 1e-10 || norm_y <= 1e-10) ?
      1e-6 : std::sqrt(norm_y / norm_f) * 0.01;
    h = std::min(h, ctl.step_size_max);
    for (size_t i = 0; i < n; ++i) {
      y1[i] = y[i] + h * f0[i];
    }
    rhs(t + h, y1, f1);
    double der2 = 0.0;
    for (size_t i = 0; i < n; ++i) {
      const double sk = ctl.atol + ctl.rtol * std::abs(y[i]);
      der2 += ((f1[i] - f0[i]) / sk) * ((f1[i] - f0[i]) / sk);
    }
    der2 = std::sqrt(der2) / h;
    const double order = 5;
    const double der12 = std::max(std::abs(der2), std::sqrt(norm_f));
    const double h1 = (der12 <= 1e-15) ?
      std::max(1e-6, std::abs(h) * 1e-3) : std::pow(0.01 / der12, 1.0 / order);
    h = std::min(100 * std::abs(h), h1);
    if (!std::isfinite(h)) {
      throw std::runtime_error("Initial step size was not finite");
    }
    h = std::max(h, ctl.step_size_min * 100);
    h = std::min(h, ctl.step_size_max);
    in.step_size = h;
  }
};

template <typename S>
void ode_simulate(const double* pars, int n_groups, int n_particles,
                  double time, const ode_ctl& ctl, const double* times,
                  int n_times, double* out, int64_t* stats, int n_threads) {
  auto shared = shared_of<S>(pars, n_groups);
  const int n_state = S::n_state(shared[0]);
  const int n_var = n_state - S::n_output;
  const size_t n_total = static_cast<size_t>(n_particles) * n_groups;
  errors err(n_total);
#pragma omp parallel for schedule(static) num_threads(n_threads)
  for (long k = 0; k < static_cast<long>(n_total); ++k) {
    const int g = k / n_particles;
    typename S::internal_state internal{};
    rng_t rng{};
    rng.deterministic = true;
    std::vector<double> y(n_state, 0.0);
    S::initial(time, shared[g], internal, rng, y.data());
    ode_internals in(n_var);
    dopri5_port<S> sol(ctl, shared[g], n_var);
    const auto z = zero_every_of<S>(shared[g]);
    try {
      sol.initialise(time, y.data(), in);
      double t = time;
      for (int i = 0; i < n_times; ++i) {
        sol.run(t, times[i], y.data(), z, in);
        t = times[i];
        if constexpr (dust2gpu::has_output<S>::value) {
          S::output(t, y.data(), shared[g], internal);
        }
        std::copy(y.begin(), y.end(),
                  out + (static_cast<size_t>(i) * n_total + k) * n_state);
      }
    } catch (const std::exception& e) {
      err.e[k].code = std::string(e.what()) == "too many steps" ?
        dust2gpu::ERR_ODE_TOO_MANY_STEPS : dust2gpu::ERR_ODE_STEP_TOO_SMALL;
    }
    stats[3 * k] = in.n_steps;
    stats[3 * k + 1] = in.n_steps_accepted;
    stats[3 * k + 2] = in.n_steps_rejected;
  }
  err.report();
}

// A mixed-time system (continuous/system.hpp:80-106, 544-585) from its
// initial conditions through `times`.  Between output times: with dt = 0
// the ODE alone; otherwise n = (t_end - t) / dt truncated steps, step s
// integrating to t + s dt (the last to t_end; the first is empty), each
// followed by the update at t_end with a copy of the particle's generator
// (never advanced) applied to a copy of the state, and a re-initialisation
// of the solver at t when the state changed.
template <typename S>
void mixed_simulate(const double* pars, int n_groups, int n_particles,
                    double time, double dt, const ode_ctl& ctl,
                    const uint64_t* rng_words, const double* times,
                    int n_times, double* out, int64_t* stats) {
  auto shared = shared_of<S>(pars, n_groups);
  const int n_state = S::n_state(shared[0]);
  const int n_special = dust2gpu::n_special<S>();
  const int n_variables = n_state - S::n_output;
  const int n_var = n_variables - n_special;
  const size_t n_total = static_cast<size_t>(n_particles) * n_groups;
  auto rngs = make_rng(rng_words, n_total, false);
  errors err(n_total);
  for (size_t k = 0; k < n_total; ++k) {
    const int g = k / n_particles;
    typename S::internal_state internal{};
    std::vector<double> y(n_state, 0.0), y_other(n_state, 0.0);
    S::initial(time, shared[g], internal, rngs[k], y.data());
    ode_internals in(n_var);
    dopri5_port<S> sol(ctl, shared[g], n_var);
    sol.special.resize(n_special);
    const auto z = zero_every_of<S>(shared[g]);
    try {
      sol.initialise(time, y.data(), in);
      double t = time;
      for (int i = 0; i < n_times; ++i) {
        const double t_end = times[i];
        if (dt == 0) {
          sol.run(t, t_end, y.data(), z, in);
        } else if (t_end > t) {
          const long n_steps = static_cast<long>((t_end - t) / dt);
          double t1 = t;
          for (long step = 0; step < n_steps; ++step) {
            const double t0 = t1;
            t1 = (step == n_steps - 1) ? t_end : t + step * dt;
            sol.run(t0, t1, y.data(), z, in);
            std::copy_n(y.begin(), n_variables, y_other.begin());
            rng_t r = rngs[k];
            S::update(t_end, dt, y.data(), shared[g], internal, r,
                      y_other.data());
            const bool same = std::equal(y_other.begin(),
                                         y_other.begin() + n_variables,
                                         y.begin());
            std::copy_n(y_other.begin(), n_variables, y.begin());
            if (!same) {
              sol.initialise(t, y.data(), in);
            }
          }
        }
        t = t_end;
        std::copy(y.begin(), y.end(),
                  out + (static_cast<size_t>(i) * n_total + k) * n_state);
      }
    } catch (const std::exception& e) {
      err.e[k].code = std::string(e.what()) == "too many steps" ?
        dust2gpu::ERR_ODE_TOO_MANY_STEPS : dust2gpu::ERR_ODE_STEP_TOO_SMALL;
    }
    stats[3 * k] = in.n_steps;
    stats[3 * k + 1] = in.n_steps_accepted;
    stats[3 * k + 2] = in.n_steps_rejected;
  }
  err.report();
}

void set_err(char* err, int err_len, const std::string& msg) {
  if (err != nullptr && err_len > 0) {
    std::strncpy(err, msg.c_str(), err_len - 1);
    err[err_len - 1] = '\0';
  }
}

std::vector<char> active_of(int n_groups, const int* index_group,
                            int n_index_group) {
  std::vector<char> a(n_groups, index_group == nullptr ? 1 : 0);
  if (index_group != nullptr) {
    for (int i = 0; i < n_index_group; ++i) {
      a[index_group[i]] = 1;
    }
  }
  return a;
}

}  // namespace

extern "C" {

int oracle_max_threads(void) {
  return omp_get_max_threads();
}

int oracle_discrete_simulate(const char* name, const double* pars,
                             int n_groups, int n_particles, double time,
                             double dt, const uint64_t* rng,
                             int deterministic, const double* initial,
                             const double* times, int n_times, double* out,
                             uint64_t* rng_out, int n_threads, char* err,
                             int err_len) {
  try {
    bool ok = dispatch_discrete(name, [&](auto t) {
      using S = typename decltype(t)::type;
      discrete_sys<S> sys(shared_of<S>(pars, n_groups),
                          std::vector<int>(n_groups, n_particles), time, dt,
                          rng, deterministic != 0, n_threads);
      if (initial == nullptr) {
        sys.set_state_initial();
      } else {
        std::copy_n(initial, sys.state.size(), sys.state.begin());
      }
      const std::vector<char> all(n_groups, 1);
      for (int i = 0; i < n_times; ++i) {
        sys.run_to_time(times[i], all);
        std::copy(sys.state.begin(), sys.state.end(),
                  out + i * sys.state.size());
      }
      for (size_t k = 0; k < sys.n_total; ++k) {
        for (int w = 0; w < 4; ++w) {
          rng_out[4 * k + w] = sys.rng[k].state[w];
        }
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

int oracle_compare(const char* name, const double* pars, int n_groups,
                   int n_particles, double time, const double* state,
                   const double* data, int n_groups_data, const uint64_t* rng,
                   double* out, uint64_t* rng_out, char* err, int err_len) {
  try {
    bool ok = dispatch_discrete(name, [&](auto t) {
      using S = typename decltype(t)::type;
      if constexpr (dust2gpu::has_compare_data<S>::value) {
        discrete_sys<S> sys(shared_of<S>(pars, n_groups),
                            std::vector<int>(n_groups, n_particles), time,
                            1.0, rng, false, 1);
        std::copy_n(state, sys.state.size(), sys.state.begin());
        std::vector<typename S::data_type> d;
        const int nd = sizeof(typename S::data_type) / sizeof(double);
        for (int g = 0; g < n_groups_data; ++g) {
          d.push_back(dust2gpu::build_data_of<S>(
            data + g * nd, sys.shared[n_groups_data == 1 ? 0 : g]));
        }
        const std::vector<char> all(n_groups, 1);
        sys.compare_data(d.data(), n_groups_data, all, out);
        for (size_t k = 0; k < sys.n_total; ++k) {
          for (int w = 0; w < 4; ++w) {
            rng_out[4 * k + w] = sys.rng[k].state[w];
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

// Filter over groups of n_particles[g] particles; rng holds, per group,
// 2 filter streams then n_particles[g] particle streams.  Runs n_runs
// times; ll_out: [n_runs][n_groups] (entries of groups not in
// index_group are left untouched).  state_out: final state (group-major
// AoS), rng_out: final streams in the input layout.
int oracle_filter_run(const char* name, const double* pars, int n_groups,
                      const int* n_particles, double time_start,
                      const double* times, int n_times, const double* data,
                      int n_groups_data, double dt, const uint64_t* rng,
                      int n_runs, const double* initial,
                      const int* index_group, int n_index_group,
                      double* ll_out, double* state_out, uint64_t* rng_out,
                      int n_threads, char* err, int err_len) {
  try {
    bool ok = dispatch_discrete(name, [&](auto t) {
      using S = typename decltype(t)::type;
      if constexpr (dust2gpu::has_compare_data<S>::value) {
        std::vector<int> np(n_particles, n_particles + n_groups);
        filter_port<S> f(shared_of<S>(pars, n_groups), np, time_start, times,
                         n_times, data, n_groups_data, dt, rng, n_threads);
        const auto active = active_of(n_groups, index_group, n_index_group);
        for (int r = 0; r < n_runs; ++r) {
          f.run(initial, active);
          for (int g = 0; g < n_groups; ++g) {
            if (active[g]) {
              ll_out[r * n_groups + g] = f.ll[g];
            }
          }
        }
        if (state_out != nullptr) {
          std::copy(f.sys.state.begin(), f.sys.state.end(), state_out);
        }
        if (rng_out != nullptr) {
          size_t pos = 0;
          for (int g = 0; g < n_groups; ++g) {
            for (int s = 0; s < 2; ++s) {
              for (int w = 0; w < 4; ++w) {
                rng_out[pos++] = f.frng[2 * g + s].state[w];
              }
            }
            for (int j = 0; j < np[g]; ++j) {
              for (int w = 0; w < 4; ++w) {
                rng_out[pos++] = f.sys.rng[f.sys.offset[g] + j].state[w];
              }
            }
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

// The adjoint run of a deterministic likelihood (unfilter.hpp:77-110 and
// compute_gradient_, :188-229, with discrete/system.hpp:95-117, 425-481)
// for the sir system, any number of particles per group: a forward pass
// over all steps keeping the state after every step (before zero_every
// resets, which act on the running copy), the compares at each data
// time's saved state with the final system time, then the reverse
// pass.  ll_out: [group][particle]; gradient_out:
// [group][particle][n_gradient]; state_out: the state after the run.
int oracle_unfilter_adjoint(const char* name, const double* pars,
                            int n_groups, int n_particles, double time_start,
                            const double* times, int n_times,
                            const double* data, int n_groups_data, double dt,
                            double* ll_out, double* gradient_out,
                            double* state_out, char* err, int err_len) {
  try {
    const std::string nm(name);
    if (nm != "sir") {
      throw std::runtime_error("no adjoint for system " + nm);
    }
    using S = dust2gpu::systems::sir;
    auto shared = shared_of<S>(pars, n_groups);
    const int ns = S::n_state(shared[0]);
    const int na = ns + 3;
    std::vector<int> step_of(n_times);
    for (int i = 0; i < n_times; ++i) {
      step_of[i] = static_cast<int>(
        std::round(std::max(0.0, times[i] - time_start) / dt));
    }
    const int n_steps = static_cast<int>(
      std::round(std::max(0.0, times[n_times - 1] - time_start) / dt));
    const double time_end = time_start + n_steps * dt;
    std::vector<typename S::data_type> d;
    for (int i = 0; i < n_times * n_groups_data; ++i) {
      d.push_back(dust2gpu::build_data_of<S>(data + i,
                                             shared[i % n_groups_data]));
    }
    for (int g = 0; g < n_groups; ++g) {
      const auto z = zero_every_of<S>(shared[g]);
      for (int j = 0; j < n_particles; ++j) {
        const size_t k = static_cast<size_t>(g) * n_particles + j;
        typename S::internal_state internal{};
        rng_t rng{};
        rng.deterministic = true;
        std::vector<double> hist(static_cast<size_t>(n_steps + 1) * ns);
        S::initial(time_start, shared[g], internal, rng, hist.data());
        std::vector<double> x(hist.begin(), hist.begin() + ns);
        for (int i = 0; i < n_steps; ++i) {
          const double t = time_start + i * dt;
          for (const auto& el : z) {
            if (std::fmod(t, el.first) == 0) {
              for (int s : el.second) {
                x[s] = 0;
              }
            }
          }
          double* y = hist.data() + static_cast<size_t>(i + 1) * ns;
          S::update(t, dt, x.data(), shared[g], internal, rng, y);
          std::copy(y, y + ns, x.begin());
        }
        const auto& data_of = [&](int i) -> const typename S::data_type& {
          return d[i * n_groups_data + (n_groups_data == 1 ? 0 : g)];
        };
        double acc = 0;
        for (int i = 0; i < n_times; ++i) {
          acc += S::compare_data(time_end, hist.data() + step_of[i] * ns,
                                 data_of(i), shared[g], internal, rng);
        }
        std::vector<double> adj(na, 0.0), next(na, 0.0);
        double time = time_end;
        for (int i = n_times - 1; i >= 0; --i) {
          const double time_i = i == 0 ? time_start : times[i - 1];
          const double* st = hist.data() + static_cast<size_t>(step_of[i]) *
            ns;
          S::adjoint_compare_data(time, st, adj.data(), data_of(i),
                                  shared[g], internal, next.data());
          std::swap(adj, next);
          const int n_back = static_cast<int>(
            std::round(std::max(0.0, time - time_i) / dt));
          for (int b = 1; b <= n_back; ++b) {
            const double tb = time - b * dt;
            S::adjoint_update(tb, dt, st - static_cast<size_t>(b) * ns,
                              adj.data(), shared[g], internal, next.data());
            std::swap(adj, next);
            for (const auto& el : z) {
              if (std::fmod(tb, el.first) == 0) {
                for (int s : el.second) {
                  adj[s] = 0;
                }
              }
            }
          }
          time = time_i;
        }
        S::adjoint_initial(time, hist.data(), adj.data(), shared[g],
                           internal, next.data());
        ll_out[k] = acc;
        std::copy(next.begin() + ns, next.end(), gradient_out + k * 3);
        std::copy(x.begin(), x.end(), state_out + k * ns);
      }
    }
    return 0;
  } catch (const std::exception& e) {
    set_err(err, err_len, e.what());
    return 1;
  }
}

// dust2::unfilter (unfilter.hpp:42-73, reset :162-186) on a deterministic
// system: initial conditions, then for each data time run_to_time and
// compare_data, summing per particle.  ll_out: [n_runs][group][particle];
// state_out (optional): the state after the last run.
// states_out (oracle_unfilter_states; may be null): the full state of the
// last run at every data time, [time][group][particle][state], as
// trajectories and snapshots record it (unfilter.hpp:60-62).
static int unfilter_run_impl(const char* name, const double* pars,
                             int n_groups, int n_particles,
                             double time_start, const double* times,
                             int n_times, const double* data,
                             int n_groups_data, double dt, int max_steps,
                             double atol, double rtol, double step_size_min,
                             double step_size_max, int n_runs,
                             double* ll_out, double* state_out,
                             double* states_out, int n_threads, char* err,
                             int err_len) {
  try {
    const size_t n_total = static_cast<size_t>(n_groups) * n_particles;
    const std::string nm(name);
    if (nm == "sirode") {
      using S = dust2gpu::systems::sirode;
      auto shared = shared_of<S>(pars, n_groups);
      const int n_state = S::n_state(shared[0]);
      const int n_var = n_state - S::n_output;
      ode_ctl ctl;
      ctl.max_steps = max_steps;
      ctl.atol = atol;
      ctl.rtol = rtol;
      ctl.step_size_min = step_size_min;
      ctl.step_size_max = step_size_max;
      std::vector<typename S::data_type> d;
      for (int i = 0; i < n_times * n_groups_data; ++i) {
        d.push_back(dust2gpu::build_data_of<S>(data + i,
                                             shared[i % n_groups_data]));
      }
      for (int r = 0; r < n_runs; ++r) {
        errors err_k(n_total);
#pragma omp parallel for schedule(static) num_threads(n_threads)
        for (long k = 0; k < static_cast<long>(n_total); ++k) {
          const int g = k / n_particles;
          typename S::internal_state internal{};
          rng_t rng{};
          rng.deterministic = true;
          std::vector<double> y(n_state, 0.0);
          S::initial(time_start, shared[g], internal, rng, y.data());
          ode_internals in(n_var);
          dopri5_port<S> sol(ctl, shared[g], n_var);
          const auto z = zero_every_of<S>(shared[g]);
          double acc = 0;
          try {
            sol.initialise(time_start, y.data(), in);
            double t = time_start;
            for (int i = 0; i < n_times; ++i) {
              sol.run(t, times[i], y.data(), z, in);
              t = times[i];
              acc += S::compare_data(
                t, y.data(), d[i * n_groups_data + (n_groups_data == 1 ? 0 :
                                                    g)],
                shared[g], internal, rng);
              if (states_out != nullptr && r == n_runs - 1) {
                std::copy(y.begin(), y.end(), states_out +
                          (static_cast<size_t>(i) * n_total + k) * n_state);
              }
            }
          } catch (const std::exception& e) {
            err_k.e[k].code = std::string(e.what()) == "too many steps" ?
              dust2gpu::ERR_ODE_TOO_MANY_STEPS :
              dust2gpu::ERR_ODE_STEP_TOO_SMALL;
          }
          ll_out[r * n_total + k] = acc;
          if (state_out != nullptr && r == n_runs - 1) {
            std::copy(y.begin(), y.end(), state_out + k * n_state);
          }
        }
        err_k.report();
      }
      return 0;
    }
    bool ok = dispatch_discrete(name, [&](auto t) {
      using S = typename decltype(t)::type;
      if constexpr (dust2gpu::has_compare_data<S>::value) {
        std::vector<int> np(n_groups, n_particles);
        std::vector<uint64_t> words(4 * n_total, 0);
        discrete_sys<S> sys(shared_of<S>(pars, n_groups), np, time_start, dt,
                            words.data(), true, n_threads);
        std::vector<typename S::data_type> d;
        const int nd = sizeof(typename S::data_type) / sizeof(double);
        for (int i = 0; i < n_times * n_groups_data; ++i) {
          d.push_back(dust2gpu::build_data_of<S>(
            data + static_cast<size_t>(i) * nd,
            sys.shared[i % n_groups_data]));
        }
        const std::vector<char> active(n_groups, 1);
        std::vector<double> step(n_total);
        for (int r = 0; r < n_runs; ++r) {
          sys.time = time_start;
          sys.set_state_initial();
          double* ll = ll_out + static_cast<size_t>(r) * n_total;
          std::fill(ll, ll + n_total, 0.0);
          for (int i = 0; i < n_times; ++i) {
            sys.run_to_time(times[i], active);
            sys.compare_data(d.data() + static_cast<size_t>(i) *
                             n_groups_data, n_groups_data, active,
                             step.data());
            for (size_t k = 0; k < n_total; ++k) {
              ll[k] += step[k];
            }
            if (states_out != nullptr && r == n_runs - 1) {
              std::copy(sys.state.begin(), sys.state.end(), states_out +
                        static_cast<size_t>(i) * sys.state.size());
            }
          }
        }
        if (state_out != nullptr) {
          std::copy(sys.state.begin(), sys.state.end(), state_out);
        }
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

int oracle_unfilter_run(const char* name, const double* pars, int n_groups,
                        int n_particles, double time_start,
                        const double* times, int n_times, const double* data,
                        int n_groups_data, double dt, int max_steps,
                        double atol, double rtol, double step_size_min,
                        double step_size_max, int n_runs, double* ll_out,
                        double* state_out, int n_threads, char* err,
                        int err_len) {
  return unfilter_run_impl(name, pars, n_groups, n_particles, time_start,
                           times, n_times, data, n_groups_data, dt,
                           max_steps, atol, rtol, step_size_min,
                           step_size_max, n_runs, ll_out, state_out, nullptr,
                           n_threads, err, err_len);
}

int oracle_unfilter_states(const char* name, const double* pars,
                           int n_groups, int n_particles, double time_start,
                           const double* times, int n_times,
                           const double* data, int n_groups_data, double dt,
                           int max_steps, double atol, double rtol,
                           double step_size_min, double step_size_max,
                           double* ll_out, double* states_out, char* err,
                           int err_len) {
  return unfilter_run_impl(name, pars, n_groups, n_particles, time_start,
                           times, n_times, data, n_groups_data, dt,
                           max_steps, atol, rtol, step_size_min,
                           step_size_max, 1, ll_out, nullptr, states_out, 1,
                           err, err_len);
}

// One filter run saving trajectories of state entries index_state (all
// when n_index_state is 0), then their export with reordering (select:
// -1 for every particle, else the particle kept in each group).
// out: [time][group][particle][state]
int oracle_filter_trajectories(const char* name, const double* pars,
                               int n_groups, int n_particles,
                               double time_start, const double* times,
                               int n_times, const double* data,
                               int n_groups_data, double dt,
                               const uint64_t* rng, const int* index_state,
                               int n_index_state, const int* snap_obs,
                               int n_snap, const int* select,
                               double* ll_out, double* out, double* snap_out,
                               int n_threads, char* err, int err_len) {
  try {
    bool ok = dispatch_discrete(name, [&](auto t) {
      using S = typename decltype(t)::type;
      if constexpr (dust2gpu::has_compare_data<S>::value) {
        std::vector<int> np(n_groups, n_particles);
        filter_port<S> f(shared_of<S>(pars, n_groups), np, time_start, times,
                         n_times, data, n_groups_data, dt, rng, n_threads);
        f.save = true;
        if (n_index_state > 0) {
          f.index_state.assign(index_state, index_state + n_index_state);
        } else {
          for (int j = 0; j < f.sys.n_state; ++j) {
            f.index_state.push_back(j);
          }
        }
        f.snap_obs.assign(snap_obs, snap_obs + n_snap);
        f.run(nullptr, std::vector<char>(n_groups, 1));
        std::copy(f.ll.begin(), f.ll.end(), ll_out);
        f.export_trajectories(select, out);
        if (n_snap > 0) {
          f.export_snapshots(select, snap_out);
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

int oracle_ode_simulate(const char* name, const double* pars, int n_groups,
                        int n_particles, double time, int max_steps,
                        double atol, double rtol, double step_size_min,
                        double step_size_max, const double* critical,
                        int n_critical, const double* times, int n_times,
                        double* out, int64_t* stats_out, int n_threads,
                        char* err, int err_len) {
  try {
    ode_ctl ctl;
    ctl.max_steps = max_steps;
    ctl.atol = atol;
    ctl.rtol = rtol;
    ctl.step_size_min = step_size_min;
    ctl.step_size_max = step_size_max;
    ctl.critical_times.assign(critical, critical + n_critical);
    const std::string nm(name);
    if (nm == "sirode") {
      ode_simulate<dust2gpu::systems::sirode>(pars, n_groups, n_particles,
                                              time, ctl, times, n_times, out,
                                              stats_out, n_threads);
    } else if (nm == "logistic") {
      ode_simulate<dust2gpu::systems::logistic>(pars, n_groups, n_particles,
                                                time, ctl, times, n_times,
                                                out, stats_out, n_threads);
    } else {
      throw std::runtime_error("unknown system " + nm);
    }
    return 0;
  } catch (const std::exception& e) {
    set_err(err, err_len, e.what());
    return 1;
  }
}

// mixed_simulate for the named mixed-time system; rng: 4 words per
// particle.
int oracle_mixed_simulate(const char* name, const double* pars, int n_groups,
                          int n_particles, double time, double dt,
                          int max_steps, double atol, double rtol,
                          double step_size_min, double step_size_max,
                          const uint64_t* rng, const double* times,
                          int n_times, double* out, int64_t* stats_out,
                          char* err, int err_len) {
  try {
    ode_ctl ctl;
    ctl.max_steps = max_steps;
    ctl.atol = atol;
    ctl.rtol = rtol;
    ctl.step_size_min = step_size_min;
    ctl.step_size_max = step_size_max;
    const std::string nm(name);
    if (nm != "malaria") {
      throw std::runtime_error("unknown system " + nm);
    }
    mixed_simulate<dust2gpu::systems::malaria>(
      pars, n_groups, n_particles, time, dt, ctl, rng, times, n_times, out,
      stats_out);
    return 0;
  } catch (const std::exception& e) {
    set_err(err, err_len, e.what());
    return 1;
  }
}

// The project's elementary functions evaluated on the host (fn: 0 exp,
// 1 log, 2 lgamma, 3 cos(2 pi x), 4 sin(2 pi x), 5 rcp).
void oracle_math(int fn, const double* x, int n, double* out) {
  for (int i = 0; i < n; ++i) {
    double s, c;
    switch (fn) {
    case 0: out[i] = dust2gpu::math::exp(x[i]); break;
    case 1: out[i] = dust2gpu::math::log(x[i]); break;
    case 2: out[i] = dust2gpu::math::lgamma(x[i]); break;
    case 3: dust2gpu::math::sincos_2pi(x[i], &s, &c); out[i] = c; break;
    case 5: out[i] = dust2gpu::math::rcp(x[i]); break;
    default: dust2gpu::math::sincos_2pi(x[i], &s, &c); out[i] = s; break;
    }
  }
}

// n draws from one stream (dist: 0 binomial(a, b), 1 poisson(a),
// 2 normal(a, b), 3 exponential_rate(a), 4 uniform(a, b),
// 5 random_real); returns the error code of the generator.
int oracle_draws(int dist, double a, double b, int n, const uint64_t* rng,
                 double* out) {
  auto r = make_rng(rng, 1, false)[0];
  for (int i = 0; i < n; ++i) {
    switch (dist) {
    case 0: out[i] = dust2gpu::random::binomial(r, a, b); break;
    case 1: out[i] = dust2gpu::random::poisson(r, a); break;
    case 2: out[i] = dust2gpu::random::normal(r, a, b); break;
    case 3: out[i] = dust2gpu::random::exponential_rate(r, a); break;
    case 4: out[i] = dust2gpu::random::uniform(r, a, b); break;
    default: out[i] = dust2gpu::random::random_real(r); break;
    }
  }
  return r.err;
}

// log densities (dist: 0 poisson(x | a), 1 negative_binomial_mu(x | a, b),
// 2 normal(x | a, b))
void oracle_density(int dist, const double* x, int n, double a, double b,
                    double* out) {
  for (int i = 0; i < n; ++i) {
    switch (dist) {
    case 0: out[i] = dust2gpu::density::poisson(x[i], a, true); break;
    case 1:
      out[i] = dust2gpu::density::negative_binomial_mu(x[i], a, b, true);
      break;
    default: out[i] = dust2gpu::density::normal(x[i], a, b, true); break;
    }
  }
}

double oracle_scale_log_weights(int n, double* w) {
  return scale_log_weights(n, w);
}

void oracle_resample_weight(int n, const double* w, double u, int64_t* idx) {
  std::vector<size_t> i(n);
  resample_weight(n, w, u, i.data());
  for (int k = 0; k < n; ++k) {
    idx[k] = static_cast<int64_t>(i[k]);
  }
}

// The parameter table of a discrete-time system as text, one
// "name length" pair per line (so that callers can pack parameter rows
// without the CUDA library).  Returns the text length, or -1 for an
// unknown system or a buffer that is too small.
int oracle_parameters(const char* name, char* out, int len) {
  std::string text;
  const bool ok = dispatch_discrete(name, [&](auto t) {
    using S = typename decltype(t)::type;
    for (const auto& p : S::parameters) {
      text += std::string(p.name) + " " + std::to_string(p.length) + "\n";
    }
  });
  if (!ok || static_cast<int>(text.size()) >= len) {
    return -1;
  }
  std::memcpy(out, text.c_str(), text.size() + 1);
  return static_cast<int>(text.size());
}

// The first n streams of an integer seed: SplitMix64 expansion of the
// seed into the first stream, then one 2^128 jump per further stream
// (the stream contract of dust2's filters, r/discrete/filter.hpp:63-75).
void oracle_rng_streams(uint64_t seed, int n, uint64_t* out) {
  uint64_t s[4];
  dust2gpu::random::seed_state(seed, s);
  for (int k = 0; k < n; ++k) {
    if (k > 0) {
      dust2gpu::random::jump(s);
    }
    for (int w = 0; w < 4; ++w) {
      out[4 * static_cast<size_t>(k) + w] = s[w];
    }
  }
}

}  // extern "C"
