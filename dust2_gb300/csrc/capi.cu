// The extern "C" entry points declared in include/dust2_gb300.h.  Each
// one validates its arguments the way dust2's R adaptors do
// (inst/include/dust2/r/*.hpp), forwards to the type-erased engine, and
// turns exceptions into a status code plus a thread-local message.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <limits>
#include <map>
#include <memory>
#include <mutex>
#include <stdexcept>
#include <string>
#include <vector>

#include "../../include/dust2_gb300.h"
#include "dust2gpu/random.hpp"
#include "engine/api.hpp"
#include "engine/registry.hpp"
#include "engine/seeding.hpp"

struct dust2_gb300_system {
  std::unique_ptr<dust2gpu::engine::system_api> impl;
};

struct dust2_gb300_filter {
  std::unique_ptr<dust2gpu::engine::filter_api> impl;
  std::vector<int> last_index_group;
};

struct dust2_gb300_server {
  std::unique_ptr<dust2gpu::engine::server_api> impl;
};

struct dust2_gb300_unfilter {
  std::unique_ptr<dust2gpu::engine::unfilter_api> impl;
};

namespace dust2gpu {
namespace engine {

namespace {

std::map<std::string, const system_factory*>& registry() {
  static std::map<std::string, const system_factory*> r;
  return r;
}

std::mutex& registry_mutex() {
  static std::mutex m;
  return m;
}

}  // namespace

void register_system(const system_factory* f) {
  std::lock_guard<std::mutex> lock(registry_mutex());
  registry()[f->name] = f;
}

const system_factory* find_system(const char* name) {
  std::lock_guard<std::mutex> lock(registry_mutex());
  auto it = registry().find(name == nullptr ? "" : name);
  if (it == registry().end()) {
    throw std::runtime_error(std::string("Unknown system '") +
                             (name == nullptr ? "" : name) + "'");
  }
  return it->second;
}

std::vector<const system_factory*> all_systems() {
  std::lock_guard<std::mutex> lock(registry_mutex());
  std::vector<const system_factory*> ret;
  for (auto& el : registry()) {
    ret.push_back(el.second);
  }
  return ret;
}

}  // namespace engine
}  // namespace dust2gpu

namespace {

using dust2gpu::engine::filter_api;
using dust2gpu::engine::system_api;

thread_local std::string last_error;

}  // namespace

void dust2gpu::engine::set_last_error(const std::string& msg) {
  last_error = msg;
}

namespace {

template <typename F>
int guard(F f) {
  try {
    f();
    return DUST2_GB300_OK;
  } catch (const std::exception& e) {
    last_error = e.what();
  } catch (...) {
    last_error = "unknown error";
  }
  return DUST2_GB300_ERROR;
}

void need(bool ok, const char* msg) {
  if (!ok) {
    throw std::runtime_error(msg);
  }
}

// r/system.hpp:66-73
void check_errors(system_api& sys, const char* action) {
  if (sys.errors_pending()) {
    throw std::runtime_error(std::string("Can't currently ") + action +
                             " this system: errors are pending");
  }
}

// Stream block from a seed (see the header for the accepted forms).
std::vector<std::uint64_t> seed_streams(const std::uint64_t* seed,
                                        std::size_t seed_len,
                                        std::size_t n_streams) {
  need(seed != nullptr && seed_len > 0, "A seed is required");
  if (seed_len == 1) {
    return dust2gpu::engine::make_streams_from_seed(seed[0], n_streams);
  }
  if (seed_len % 4 != 0) {
    throw std::runtime_error(
      "Expected a seed of 1 word or a multiple of 4 words (32 bytes per "
      "stream)");
  }
  const std::size_t given = seed_len / 4;
  if (given >= n_streams) {
    return std::vector<std::uint64_t>(seed, seed + 4 * n_streams);
  }
  auto tail = dust2gpu::engine::make_streams(seed + 4 * (given - 1),
                                             n_streams - given + 1);
  std::vector<std::uint64_t> ret(seed, seed + 4 * given);
  ret.insert(ret.end(), tail.begin() + 4, tail.end());
  return ret;
}

dust2gpu::engine::ode_control to_control(const dust2_gb300_ode_control* c) {
  dust2gpu::engine::ode_control ctl;
  if (c != nullptr) {
    ctl.max_steps = c->max_steps;
    ctl.atol = c->atol;
    ctl.rtol = c->rtol;
    ctl.step_size_min = c->step_size_min;
    ctl.step_size_max = c->step_size_max;
    if (c->critical_times != nullptr) {
      ctl.critical_times.assign(c->critical_times,
                                c->critical_times + c->n_critical_times);
    }
    ctl.debug_record_step_times = c->debug_record_step_times != 0;
  }
  // r/continuous/control.hpp:15-17
  ctl.step_size_min = std::max(ctl.step_size_min,
                               std::numeric_limits<double>::epsilon());
  return ctl;
}

std::vector<int> to_int_index(const std::size_t* index, std::size_t n,
                              std::size_t max, const char* name) {
  std::vector<int> ret;
  if (index == nullptr) {
    return ret;
  }
  for (std::size_t i = 0; i < n; ++i) {
    if (index[i] >= max) {
      char buf[256];
      std::snprintf(buf, sizeof(buf),
                    "All values of '%s' must be in [1, %zu], but '%s[%zu]' "
                    "was %zu", name, max, name, i + 1, index[i] + 1);
      throw std::runtime_error(buf);
    }
    ret.push_back(static_cast<int>(index[i]));
  }
  return ret;
}

system_api& sysref(dust2_gb300_system* sys) {
  need(sys != nullptr && sys->impl != nullptr, "Invalid system handle");
  return *sys->impl;
}

filter_api& filref(dust2_gb300_filter* f) {
  need(f != nullptr && f->impl != nullptr, "Invalid filter handle");
  return *f->impl;
}

dust2gpu::engine::unfilter_api& unfref(dust2_gb300_unfilter* u) {
  need(u != nullptr && u->impl != nullptr, "Invalid unfilter handle");
  return *u->impl;
}

dust2gpu::engine::server_api& servref(dust2_gb300_server* s) {
  need(s != nullptr && s->impl != nullptr, "Invalid server handle");
  return *s->impl;
}

// r/helpers.hpp check_time_sequence(require_later = true), as for filters
void check_data_times(double time_start, const double* time, size_t n_time) {
  need(time != nullptr && n_time >= 1,
       "Expected 'data' to have at least one row");
  if (time[0] < time_start) {
    char buf[200];
    std::snprintf(buf, sizeof(buf),
                  "'time_start' (%g) is later than the first time in "
                  "'data' (%g)", time_start, time[0]);
    throw std::runtime_error(buf);
  }
  for (std::size_t i = 1; i < n_time; ++i) {
    need(time[i] > time[i - 1], "Values in 'time' must be increasing");
  }
}

}  // namespace

extern "C" {

int dust2_gb300_abi_version(void) {
  return 1;
}

size_t dust2_gb300_last_error(char* buf, size_t len) {
  if (buf != nullptr && len > 0) {
    const std::size_t n = std::min(len - 1, last_error.size());
    std::memcpy(buf, last_error.data(), n);
    buf[n] = '\0';
  }
  return last_error.size();
}

int dust2_gb300_device_count(int32_t* n) {
  return guard([&] {
    int c = 0;
    const cudaError_t err = cudaGetDeviceCount(&c);
    if (err != cudaSuccess) {
      cudaGetLastError();
      c = 0;
    }
    *n = c;
  });
}

int dust2_gb300_systems(char* buf, size_t len) {
  return guard([&] {
    std::string s;
    for (auto* f : dust2gpu::engine::all_systems()) {
      s += (s.empty() ? "" : ",") + std::string(f->name);
    }
    need(buf != nullptr && len > s.size(), "buffer too small");
    std::memcpy(buf, s.c_str(), s.size() + 1);
  });
}

int dust2_gb300_system_info(const char* name, char* json, size_t len) {
  return guard([&] {
    const auto* f = dust2gpu::engine::find_system(name);
    const std::string s = f->info_json();
    need(json != nullptr && len > s.size(), "buffer too small");
    std::memcpy(json, s.c_str(), s.size() + 1);
  });
}

int dust2_gb300_rng_streams(const uint64_t* seed, size_t seed_len,
                            size_t n_streams, uint64_t* out) {
  return guard([&] {
    const auto words = seed_streams(seed, seed_len, n_streams);
    std::copy(words.begin(), words.end(), out);
  });
}

int dust2_gb300_system_alloc(const char* name, const double* pars,
                             size_t n_groups, size_t n_particles,
                             double time, double dt,
                             const dust2_gb300_ode_control* control,
                             const uint64_t* seed, size_t seed_len,
                             int32_t deterministic,
                             dust2_gb300_system** out) {
  return guard([&] {
    need(out != nullptr, "out is NULL");
    need(n_particles >= 1, "'n_particles' must be at least 1");
    need(n_groups >= 1, "'n_groups' must be at least 1");
    const auto* f = dust2gpu::engine::find_system(name);
    if (!f->continuous) {
      need(dt > 0, "Expected 'dt' to be greater than 0");
    }
    const std::size_t n_total = n_particles * n_groups;
    auto words = seed_streams(seed, seed_len, n_total);
    std::vector<int> np(n_groups, static_cast<int>(n_particles));
    auto ctl = to_control(control);
    auto* impl = f->create_system(pars, static_cast<int>(n_groups), np, time,
                                  dt, ctl, words, deterministic != 0, 0);
    *out = new dust2_gb300_system{std::unique_ptr<system_api>(impl)};
  });
}

int dust2_gb300_system_free(dust2_gb300_system* sys) {
  return guard([&] { delete sys; });
}

int dust2_gb300_system_dim(const dust2_gb300_system* sys, size_t* n_state,
                           size_t* n_particles, size_t* n_groups) {
  return guard([&] {
    need(sys != nullptr && sys->impl != nullptr, "Invalid system handle");
    *n_state = sys->impl->n_state();
    *n_particles = sys->impl->n_particles()[0];
    *n_groups = sys->impl->n_groups();
  });
}

// The state packing as JSON, [{"name": ..., "dims": [...]}, ...], into
// buf (NUL-terminated, truncated to len); *needed gets the full length.
static void write_packing(const dust2gpu::engine::system_api& s, char* buf,
                          size_t len, size_t* needed) {
  std::string out = "[";
  bool first = true;
  for (const auto& e : s.packing_state()) {
    out += first ? "" : ", ";
    first = false;
    out += "{\"name\": \"" + e.name + "\", \"dims\": [";
    for (std::size_t i = 0; i < e.dims.size(); ++i) {
      out += (i ? ", " : "") + std::to_string(e.dims[i]);
    }
    out += "]}";
  }
  out += "]";
  if (needed != nullptr) {
    *needed = out.size();
  }
  if (buf != nullptr && len > 0) {
    const std::size_t n = std::min(len - 1, out.size());
    std::memcpy(buf, out.data(), n);
    buf[n] = '\0';
  }
}

int dust2_gb300_system_packing_state(dust2_gb300_system* sys, char* buf,
                                     size_t len, size_t* needed) {
  return guard([&] { write_packing(sysref(sys), buf, len, needed); });
}

int dust2_gb300_filter_packing_state(dust2_gb300_filter* filter, char* buf,
                                     size_t len, size_t* needed) {
  return guard([&] {
    write_packing(filref(filter).sys(), buf, len, needed);
  });
}

int dust2_gb300_unfilter_packing_state(dust2_gb300_unfilter* unfilter,
                                       char* buf, size_t len,
                                       size_t* needed) {
  return guard([&] {
    write_packing(unfref(unfilter).sys(), buf, len, needed);
  });
}

int dust2_gb300_system_state(dust2_gb300_system* sys, double* out) {
  return guard([&] {
    auto& s = sysref(sys);
    check_errors(s, "get state from");
    s.get_state(out);
  });
}

int dust2_gb300_system_set_state(dust2_gb300_system* sys, const double* value,
                                 const size_t* index_state, size_t n_index_state,
                                 const size_t* index_particle,
                                 size_t n_index_particle,
                                 const size_t* index_group, size_t n_index_group,
                                 int32_t recycle_particle,
                                 int32_t recycle_group) {
  return guard([&] {
    auto& s = sysref(sys);
    const std::size_t n_state = s.n_state();
    const std::size_t n_particles = s.n_particles()[0];
    const std::size_t n_groups = s.n_groups();
    auto is = to_int_index(index_state, n_index_state, n_state, "index_state");
    auto ip = to_int_index(index_particle, n_index_particle, n_particles,
                           "index_particle");
    auto ig = to_int_index(index_group, n_index_group, n_groups,
                           "index_group");
    std::vector<double> state(n_state * n_particles * n_groups);
    const bool simple = is.empty() && ip.empty() && ig.empty() &&
      !recycle_particle && !recycle_group;
    if (simple) {
      std::copy_n(value, state.size(), state.begin());
    } else {
      // internals.hpp:110-163
      s.get_state(state.data());
      const std::size_t n_state_in = is.empty() ? n_state : is.size();
      const std::size_t n_particles_in = ip.empty() ? n_particles : ip.size();
      const std::size_t n_groups_in = ig.empty() ? n_groups : ig.size();
      const std::size_t off_particle = recycle_particle ? 0 : n_state_in;
      const std::size_t off_group = recycle_group ? 0 :
        (n_state_in * (recycle_particle ? 1 : n_particles_in));
      for (std::size_t i = 0; i < n_groups_in; ++i) {
        for (std::size_t j = 0; j < n_particles_in; ++j) {
          const std::size_t src = i * off_group + j * off_particle;
          const std::size_t gi = ig.empty() ? i : ig[i];
          const std::size_t pj = ip.empty() ? j : ip[j];
          const std::size_t dst = (n_particles * gi + pj) * n_state;
          if (!is.empty()) {
            for (std::size_t k = 0; k < n_state_in; ++k) {
              state[dst + is[k]] = value[src + k];
            }
          } else {
            std::copy_n(value + src, n_state, state.begin() + dst);
          }
        }
      }
    }
    s.put_state(state.data());
  });
}

int dust2_gb300_system_set_state_initial(dust2_gb300_system* sys) {
  return guard([&] { sysref(sys).set_state_initial(); });
}

int dust2_gb300_system_time(dust2_gb300_system* sys, double* time) {
  return guard([&] {
    auto& s = sysref(sys);
    check_errors(s, "get time from");
    *time = s.time();
  });
}

int dust2_gb300_system_set_time(dust2_gb300_system* sys, double time) {
  return guard([&] {
    auto& s = sysref(sys);
    check_errors(s, "set time for");
    s.set_time(time);
  });
}

int dust2_gb300_system_rng_state(dust2_gb300_system* sys, uint64_t* out) {
  return guard([&] { sysref(sys).get_rng_state(out); });
}

int dust2_gb300_system_set_rng_state(dust2_gb300_system* sys,
                                     const uint64_t* state, size_t len) {
  return guard([&] {
    auto& s = sysref(sys);
    const std::size_t expected = 4 * static_cast<std::size_t>(
      s.n_particles_total());
    if (len != expected) {
      char buf[200];
      std::snprintf(buf, sizeof(buf),
                    "Incorrect length for 'rng_state'; expected %zu but "
                    "given %zu", expected * 8, len * 8);
      throw std::runtime_error(buf);
    }
    s.put_rng_state(state);
  });
}

int dust2_gb300_system_update_pars(dust2_gb300_system* sys,
                                   const double* pars,
                                   const size_t* index_group,
                                   size_t n_index_group) {
  return guard([&] {
    auto& s = sysref(sys);
    auto ig = to_int_index(index_group, n_index_group, s.n_groups(),
                           "index_group");
    if (ig.empty()) {
      s.update_pars(pars, nullptr, 0);
    } else {
      s.update_pars(pars, ig.data(), static_cast<int>(ig.size()));
    }
  });
}

int dust2_gb300_system_run_to_time(dust2_gb300_system* sys, double time) {
  return guard([&] {
    auto& s = sysref(sys);
    check_errors(s, "run");
    const double curr = s.time();
    if (time < curr) {
      char buf[200];
      std::snprintf(buf, sizeof(buf),
                    "Can't run to time %f, system already at time %f", time,
                    curr);
      throw std::runtime_error(buf);
    }
    s.run_to_time(time);
  });
}

// r/system.hpp:286-327 (check_time_sequence of the output times)
static void check_simulate_times(system_api& s, const double* times,
                                 size_t n_times) {
  check_errors(s, "simulate");
  need(times != nullptr && n_times >= 1,
       "Expected at least one value in 'times'");
  if (times[0] < s.time()) {
    char buf[200];
    std::snprintf(buf, sizeof(buf),
                  "Expected 'time[1]' (%d) to be larger than the previous "
                  "value (%d)", static_cast<int>(times[0]),
                  static_cast<int>(s.time()));
    throw std::runtime_error(buf);
  }
  for (std::size_t i = 1; i < n_times; ++i) {
    need(times[i] > times[i - 1], "Values in 'times' must be increasing");
  }
}

int dust2_gb300_system_simulate(dust2_gb300_system* sys, const double* times,
                                size_t n_times, const size_t* index_state,
                                size_t n_index_state, double* out) {
  return guard([&] {
    auto& s = sysref(sys);
    check_simulate_times(s, times, n_times);
    auto is = to_int_index(index_state, n_index_state, s.n_state(),
                           "index_state");
    s.simulate(times, static_cast<int>(n_times), is.empty() ? nullptr : is.data(),
               static_cast<int>(is.size()), out);
  });
}

int dust2_gb300_system_simulate_device(dust2_gb300_system* sys,
                                       const double* times, size_t n_times,
                                       double* out_device) {
  return guard([&] {
    auto& s = sysref(sys);
    check_simulate_times(s, times, n_times);
    need(out_device != nullptr, "out_device is NULL");
    s.simulate_device(times, static_cast<int>(n_times), out_device);
  });
}

int dust2_gb300_system_stream(dust2_gb300_system* sys, void** stream) {
  return guard([&] {
    need(stream != nullptr, "stream is NULL");
    *stream = sysref(sys).stream_handle();
  });
}

int dust2_gb300_system_reorder(dust2_gb300_system* sys, const size_t* index,
                               size_t len) {
  return guard([&] {
    auto& s = sysref(sys);
    check_errors(s, "reorder");
    const std::size_t n_particles = s.n_particles()[0];
    const std::size_t n_total = s.n_particles_total();
    if (len != n_total) {
      throw std::runtime_error("Expected an index of length " +
                               std::to_string(n_total));
    }
    std::vector<int> idx(len);
    for (std::size_t i = 0; i < len; ++i) {
      if (index[i] >= n_particles) {
        throw std::runtime_error("Expected 'index' values to lie in [1, " +
                                 std::to_string(n_particles) + "]");
      }
      idx[i] = static_cast<int>(index[i]);
    }
    s.reorder(idx.data());
  });
}

int dust2_gb300_system_compare_data(dust2_gb300_system* sys,
                                    const double* data, size_t n_groups_data,
                                    double* out) {
  return guard([&] {
    auto& s = sysref(sys);
    check_errors(s, "compare data for");
    if (!s.has_compare()) {
      throw std::runtime_error(
        std::string("Can't compare against data; the '") + s.name() +
        "' system does not have 'compare_data'");
    }
    if (n_groups_data != 1 &&
        n_groups_data != static_cast<std::size_t>(s.n_groups())) {
      throw std::runtime_error(
        "Expected 'data' to have length " + std::to_string(s.n_groups()) +
        ", but it had length " + std::to_string(n_groups_data));
    }
    s.compare_data(data, static_cast<int>(n_groups_data), out);
  });
}

int dust2_gb300_system_internals(dust2_gb300_system* sys, double* step_size,
                                 double* error, int64_t* n_steps,
                                 int64_t* n_steps_accepted,
                                 int64_t* n_steps_rejected) {
  return guard([&] {
    auto& s = sysref(sys);
    need(s.is_continuous(), "discrete-time systems have no internals");
    const auto rows = s.ode_internals();
    for (std::size_t k = 0; k < rows.size(); ++k) {
      step_size[k] = rows[k].step_size;
      error[k] = rows[k].error;
      n_steps[k] = rows[k].n_steps;
      n_steps_accepted[k] = rows[k].n_steps_accepted;
      n_steps_rejected[k] = rows[k].n_steps_rejected;
    }
  });
}

int dust2_gb300_system_step_times(dust2_gb300_system* sys, size_t particle,
                                  double* out, size_t cap, size_t* n) {
  return guard([&] {
    auto& s = sysref(sys);
    need(s.is_continuous(), "discrete-time systems have no step times");
    const auto times = s.ode_step_times();
    need(particle < times.size(), "particle out of range");
    const auto& t = times[particle];
    *n = t.size();
    for (std::size_t i = 0; i < std::min(cap, t.size()); ++i) {
      out[i] = t[i];
    }
  });
}

static int filter_alloc_impl(const char* name, const double* pars,
                             size_t n_groups, const std::vector<int>& np,
                             double time_start, const double* time,
                             size_t n_time, const double* data,
                             size_t n_groups_data, double dt,
                             const dust2_gb300_ode_control* control,
                             const uint64_t* seed, size_t seed_len,
                             dust2_gb300_filter** out) {
  return guard([&] {
    need(out != nullptr, "out is NULL");
    need(n_groups >= 1, "'n_groups' must be at least 1");
    need(n_time >= 1, "Expected 'data' to have at least one row");
    // discrete systems need dt > 0; a mixed-time system may run without
    // updates (dt = 0, check_dt(allow_null = TRUE), R/filter-support.R)
    const auto* f0 = dust2gpu::engine::find_system(name);
    if (control == nullptr || !f0->continuous) {
      need(dt > 0, "Expected 'dt' to be greater than 0");
    } else {
      need(dt >= 0, "Expected 'dt' to be greater than 0");
    }
    need(n_groups_data == 1 || n_groups_data == n_groups,
         "Expected 'data' to have 1 or n_groups groups");
    // r/helpers.hpp check_time_sequence(require_later = true)
    if (time[0] <= time_start) {
      char buf[200];
      std::snprintf(buf, sizeof(buf),
                    "'time_start' (%g) is later than the first time in "
                    "'data' (%g)", time_start, time[0]);
      if (time[0] < time_start) {
        throw std::runtime_error(buf);
      }
    }
    for (std::size_t i = 1; i < n_time; ++i) {
      need(time[i] > time[i - 1], "Values in 'time' must be increasing");
    }
    const auto* f = dust2gpu::engine::find_system(name);
    std::size_t n_streams = 0;
    for (auto n : np) {
      need(n >= 1, "'n_particles' must be at least 1");
      n_streams += static_cast<std::size_t>(n) + 2;
    }
    auto words = seed_streams(seed, seed_len, n_streams);
    const auto ctl = to_control(control);
    auto* impl = f->create_filter(pars, static_cast<int>(n_groups), np,
                                  time_start, time, static_cast<int>(n_time),
                                  data, static_cast<int>(n_groups_data), dt,
                                  ctl, words, 0);
    *out = new dust2_gb300_filter{std::unique_ptr<filter_api>(impl), {}};
  });
}

int dust2_gb300_filter_alloc(const char* name, const double* pars,
                             size_t n_groups, size_t n_particles,
                             double time_start, const double* time,
                             size_t n_time, const double* data,
                             size_t n_groups_data, double dt,
                             const uint64_t* seed, size_t seed_len,
                             dust2_gb300_filter** out) {
  std::vector<int> np(n_groups, static_cast<int>(n_particles));
  return filter_alloc_impl(name, pars, n_groups, np, time_start, time, n_time,
                           data, n_groups_data, dt, nullptr, seed, seed_len,
                           out);
}

int dust2_gb300_filter_alloc_uneven(const char* name, const double* pars,
                                    size_t n_groups,
                                    const size_t* n_particles,
                                    double time_start, const double* time,
                                    size_t n_time, const double* data,
                                    size_t n_groups_data, double dt,
                                    const uint64_t* seed, size_t seed_len,
                                    dust2_gb300_filter** out) {
  std::vector<int> np;
  for (std::size_t g = 0; g < n_groups; ++g) {
    np.push_back(static_cast<int>(n_particles[g]));
  }
  return filter_alloc_impl(name, pars, n_groups, np, time_start, time, n_time,
                           data, n_groups_data, dt, nullptr, seed, seed_len,
                           out);
}

int dust2_gb300_filter_alloc_continuous(
    const char* name, const double* pars, size_t n_groups,
    size_t n_particles, double time_start, const double* time, size_t n_time,
    const double* data, size_t n_groups_data, double dt,
    const dust2_gb300_ode_control* control, const uint64_t* seed,
    size_t seed_len, dust2_gb300_filter** out) {
  std::vector<int> np(n_groups, static_cast<int>(n_particles));
  static const dust2_gb300_ode_control defaults{
    10000, 1e-6, 1e-6, 0, std::numeric_limits<double>::infinity(), nullptr,
    0, 0};
  return filter_alloc_impl(name, pars, n_groups, np, time_start, time, n_time,
                           data, n_groups_data, dt,
                           control == nullptr ? &defaults : control, seed,
                           seed_len, out);
}

int dust2_gb300_filter_free(dust2_gb300_filter* filter) {
  return guard([&] { delete filter; });
}

int dust2_gb300_filter_dim(const dust2_gb300_filter* filter, size_t* n_state,
                           size_t* n_particles_total, size_t* n_groups,
                           size_t* n_time) {
  return guard([&] {
    need(filter != nullptr && filter->impl != nullptr,
         "Invalid filter handle");
    auto& s = filter->impl->sys();
    *n_state = s.n_state();
    *n_particles_total = s.n_particles_total();
    *n_groups = s.n_groups();
    *n_time = filter->impl->n_times();
  });
}

int dust2_gb300_filter_run(dust2_gb300_filter* filter, const double* initial,
                           const size_t* index_group, size_t n_index_group,
                           double* ll) {
  return guard([&] {
    auto& f = filref(filter);
    auto ig = to_int_index(index_group, n_index_group, f.sys().n_groups(),
                           "index_group");
    f.run(initial, ig.empty() ? nullptr : ig.data(),
          static_cast<int>(ig.size()), ll);
    filter->last_index_group = ig;
  });
}

int dust2_gb300_filter_update_pars(dust2_gb300_filter* filter,
                                   const double* pars,
                                   const size_t* index_group,
                                   size_t n_index_group) {
  return guard([&] {
    auto& f = filref(filter);
    auto ig = to_int_index(index_group, n_index_group, f.sys().n_groups(),
                           "index_group");
    f.update_pars(pars, ig.empty() ? nullptr : ig.data(),
                  static_cast<int>(ig.size()));
  });
}

int dust2_gb300_filter_rng_state(dust2_gb300_filter* filter, uint64_t* out,
                                 size_t len) {
  return guard([&] {
    auto& f = filref(filter);
    need(len == 4 * f.n_rng_streams(), "rng buffer has the wrong length");
    f.get_rng_state(out);
  });
}

int dust2_gb300_filter_set_rng_state(dust2_gb300_filter* filter,
                                     const uint64_t* state, size_t len) {
  return guard([&] {
    auto& f = filref(filter);
    const std::size_t expected = 4 * f.n_rng_streams();
    if (len != expected) {
      char buf[200];
      std::snprintf(buf, sizeof(buf),
                    "Incorrect length for 'rng_state'; expected %zu but "
                    "given %zu", expected * 8, len * 8);
      throw std::runtime_error(buf);
    }
    f.put_rng_state(state);
  });
}

static std::vector<int> last_groups(dust2_gb300_filter* filter) {
  std::vector<int> groups = filter->last_index_group;
  if (groups.empty()) {
    for (int g = 0; g < filter->impl->sys().n_groups(); ++g) {
      groups.push_back(g);
    }
  }
  return groups;
}

int dust2_gb300_filter_set_save_trajectories(dust2_gb300_filter* filter,
                                             int32_t save,
                                             const size_t* index_state,
                                             size_t n_index_state) {
  return guard([&] {
    auto& f = filref(filter);
    auto is = to_int_index(index_state, n_index_state, f.sys().n_state(),
                           "index_state");
    f.set_save_trajectories(save != 0, is.empty() ? nullptr : is.data(),
                            static_cast<int>(is.size()));
  });
}

int dust2_gb300_filter_trajectory_dim(dust2_gb300_filter* filter,
                                      int32_t select_random_particle,
                                      size_t* n_state, size_t* n_particles,
                                      size_t* n_groups, size_t* n_time) {
  return guard([&] {
    auto& f = filref(filter);
    need(f.trajectories_current(), "Trajectories are not current");
    const auto groups = last_groups(filter);
    *n_state = f.n_trajectory_state();
    *n_particles = select_random_particle ? 1 :
      f.sys().n_particles()[groups[0]];
    *n_groups = groups.size();
    *n_time = f.n_times();
  });
}

int dust2_gb300_filter_last_trajectories(dust2_gb300_filter* filter,
                                         int32_t select_random_particle,
                                         double* out) {
  return guard([&] {
    auto& f = filref(filter);
    need(f.trajectories_current(), "Trajectories are not current");
    need(out != nullptr, "out is NULL");
    const auto groups = last_groups(filter);
    const auto& np = f.sys().n_particles();
    for (int g : groups) {
      need(np[g] == np[groups[0]],
           "Trajectories need equal particle counts in every group");
    }
    std::vector<int> select;
    if (select_random_particle) {
      const auto pick = f.select_random_particle();
      for (int g : groups) {
        select.push_back(pick[g]);
      }
    }
    f.last_trajectories(groups.data(), static_cast<int>(groups.size()),
                        select.empty() ? nullptr : select.data(), out);
  });
}

int dust2_gb300_filter_set_save_snapshots(dust2_gb300_filter* filter,
                                          const size_t* time_index,
                                          size_t n) {
  return guard([&] {
    auto& f = filref(filter);
    auto idx = to_int_index(time_index, n, f.n_times(), "save_snapshots");
    for (std::size_t i = 1; i < idx.size(); ++i) {
      need(idx[i] > idx[i - 1], "'save_snapshots' must be increasing");
    }
    f.set_save_snapshots(idx.data(), static_cast<int>(idx.size()));
  });
}

int dust2_gb300_filter_snapshot_dim(dust2_gb300_filter* filter,
                                    int32_t select_random_particle,
                                    size_t* n_state, size_t* n_particles,
                                    size_t* n_groups, size_t* n_snapshots) {
  return guard([&] {
    auto& f = filref(filter);
    need(f.snapshots_current(), "Snapshots are not current");
    const auto groups = last_groups(filter);
    *n_state = f.sys().n_state();
    *n_particles = select_random_particle ? 1 :
      f.sys().n_particles()[groups[0]];
    *n_groups = groups.size();
    *n_snapshots = f.n_snapshots();
  });
}

int dust2_gb300_filter_last_snapshots(dust2_gb300_filter* filter,
                                      int32_t select_random_particle,
                                      double* out) {
  return guard([&] {
    auto& f = filref(filter);
    need(f.snapshots_current(), "Snapshots are not current");
    need(out != nullptr, "out is NULL");
    const auto groups = last_groups(filter);
    const auto& np = f.sys().n_particles();
    for (int g : groups) {
      need(np[g] == np[groups[0]],
           "Snapshots need equal particle counts in every group");
    }
    std::vector<int> select;
    if (select_random_particle) {
      const auto pick = f.select_random_particle();
      for (int g : groups) {
        select.push_back(pick[g]);
      }
    }
    f.last_snapshots(groups.data(), static_cast<int>(groups.size()),
                     select.empty() ? nullptr : select.data(), out);
  });
}

int dust2_gb300_filter_last_state(dust2_gb300_filter* filter,
                                  int32_t select_random_particle,
                                  double* out) {
  return guard([&] {
    auto& f = filref(filter);
    need(f.has_run(), "State is not current");
    auto& s = f.sys();
    const std::size_t n_state = s.n_state();
    std::vector<double> state(n_state * s.n_particles_total());
    s.get_state(state.data());
    std::vector<int> groups = filter->last_index_group;
    if (groups.empty()) {
      for (int g = 0; g < s.n_groups(); ++g) {
        groups.push_back(g);
      }
    }
    std::vector<int> offset(s.n_groups(), 0);
    for (int g = 1; g < s.n_groups(); ++g) {
      offset[g] = offset[g - 1] + s.n_particles()[g - 1];
    }
    if (select_random_particle) {
      const auto pick = f.select_random_particle();
      std::size_t pos = 0;
      for (int g : groups) {
        const std::size_t from = (offset[g] + pick[g]) * n_state;
        std::copy_n(state.begin() + from, n_state, out + pos);
        pos += n_state;
      }
    } else {
      std::size_t pos = 0;
      for (int g : groups) {
        const std::size_t from = offset[g] * n_state;
        const std::size_t n = n_state * s.n_particles()[g];
        std::copy_n(state.begin() + from, n, out + pos);
        pos += n;
      }
    }
  });
}

int dust2_gb300_filter_serial_fallbacks(dust2_gb300_filter* filter,
                                        int64_t* n) {
  return guard([&] { *n = filref(filter).n_serial_fallbacks(); });
}

int dust2_gb300_filter_set_serial_resample(dust2_gb300_filter* filter,
                                           int32_t serial) {
  return guard([&] { filref(filter).set_serial_resample(serial != 0); });
}

int dust2_gb300_filter_set_fused_tail(dust2_gb300_filter* filter,
                                      int32_t fused) {
  return guard([&] { filref(filter).set_fused_tail(fused != 0); });
}

int dust2_gb300_filter_run_async(dust2_gb300_filter* filter,
                                 const size_t* index_group,
                                 size_t n_index_group) {
  return guard([&] {
    auto& f = filref(filter);
    auto ig = to_int_index(index_group, n_index_group, f.sys().n_groups(),
                           "index_group");
    f.run_async(ig.empty() ? nullptr : ig.data(),
                static_cast<int>(ig.size()));
    filter->last_index_group = ig;
  });
}

int dust2_gb300_filter_last_log_likelihood(dust2_gb300_filter* filter,
                                           double* ll) {
  return guard([&] { filref(filter).last_log_likelihood(ll); });
}

int dust2_gb300_filter_stream(dust2_gb300_filter* filter, void** stream) {
  return guard([&] { *stream = filref(filter).stream_handle(); });
}

int dust2_gb300_filter_set_timing(dust2_gb300_filter* filter,
                                  int32_t enable) {
  return guard([&] { filref(filter).set_timing(enable != 0); });
}

int dust2_gb300_filter_kernel_times(dust2_gb300_filter* filter,
                                    double* step_ms, int64_t* n_step_launches,
                                    double* run_ms, int64_t* n_runs) {
  return guard([&] {
    long a = 0, b = 0;
    filref(filter).kernel_times(step_ms, &a, run_ms, &b);
    *n_step_launches = a;
    *n_runs = b;
  });
}

int dust2_gb300_filter_reorder_times(dust2_gb300_filter* filter,
                                     double* ms, int64_t* n_launches) {
  return guard([&] {
    long n = 0;
    filref(filter).reorder_times(ms, &n);
    *n_launches = n;
  });
}

int dust2_gb300_filter_set_autotune(dust2_gb300_filter* filter,
                                    int32_t enable) {
  return guard([&] { filref(filter).set_autotune(enable != 0); });
}

int dust2_gb300_filter_set_step_shape(dust2_gb300_filter* filter,
                                      int32_t block, int32_t per_tile,
                                      int32_t persistent) {
  return guard([&] {
    filref(filter).set_step_shape(block, per_tile, persistent != 0);
  });
}

int dust2_gb300_filter_step_shape(dust2_gb300_filter* filter, int32_t* block,
                                  int32_t* per_tile, int32_t* persistent,
                                  int32_t* n_candidates, double* best_ms) {
  return guard([&] {
    int b = 0, p = 0, q = 0, n = 0;
    filref(filter).step_shape_info(&b, &p, &q, &n, best_ms);
    *block = b;
    *per_tile = p;
    *persistent = q;
    *n_candidates = n;
  });
}

int dust2_gb300_unfilter_alloc(const char* name, const double* pars,
                               size_t n_groups, size_t n_particles,
                               double time_start, const double* time,
                               size_t n_time, const double* data,
                               size_t n_groups_data, double dt,
                               const dust2_gb300_ode_control* control,
                               dust2_gb300_unfilter** out) {
  return guard([&] {
    need(out != nullptr && pars != nullptr && data != nullptr,
         "NULL argument");
    need(n_groups >= 1, "'n_groups' must be at least 1");
    need(n_particles >= 1, "'n_particles' must be at least 1");
    need(n_groups_data == 1 || n_groups_data == n_groups,
         "Expected 'data' to have 1 or n_groups groups");
    check_data_times(time_start, time, n_time);
    const auto* f = dust2gpu::engine::find_system(name);
    need(f->continuous || dt > 0, "Expected 'dt' to be greater than 0");
    std::vector<int> np(n_groups, static_cast<int>(n_particles));
    auto* impl = f->create_unfilter(pars, static_cast<int>(n_groups), np,
                                    time_start, time,
                                    static_cast<int>(n_time), data,
                                    static_cast<int>(n_groups_data), dt,
                                    to_control(control));
    *out = new dust2_gb300_unfilter{
      std::unique_ptr<dust2gpu::engine::unfilter_api>(impl)};
  });
}

int dust2_gb300_unfilter_free(dust2_gb300_unfilter* unfilter) {
  return guard([&] { delete unfilter; });
}

int dust2_gb300_unfilter_run(dust2_gb300_unfilter* unfilter,
                             const double* initial,
                             const size_t* index_group,
                             size_t n_index_group, double* ll) {
  return guard([&] {
    auto& u = unfref(unfilter);
    need(ll != nullptr, "ll is NULL");
    auto ig = to_int_index(index_group, n_index_group, u.sys().n_groups(),
                           "index_group");
    u.run(initial, ig.empty() ? nullptr : ig.data(),
          static_cast<int>(ig.size()), ll);
  });
}

int dust2_gb300_unfilter_run_adjoint(dust2_gb300_unfilter* unfilter,
                                     const double* initial,
                                     const size_t* index_group,
                                     size_t n_index_group, double* ll) {
  return guard([&] {
    auto& u = unfref(unfilter);
    need(ll != nullptr, "ll is NULL");
    auto ig = to_int_index(index_group, n_index_group, u.sys().n_groups(),
                           "index_group");
    u.run_adjoint(initial, ig.empty() ? nullptr : ig.data(),
                  static_cast<int>(ig.size()), ll);
  });
}

int dust2_gb300_unfilter_gradient_dim(const dust2_gb300_unfilter* unfilter,
                                      size_t* n_gradient,
                                      size_t* n_groups_last) {
  return guard([&] {
    need(unfilter != nullptr && unfilter->impl != nullptr,
         "Invalid unfilter handle");
    need(n_gradient != nullptr && n_groups_last != nullptr,
         "output is NULL");
    *n_gradient = unfilter->impl->n_gradient();
    *n_groups_last = unfilter->impl->n_last_gradient_groups();
  });
}

int dust2_gb300_unfilter_last_gradient(dust2_gb300_unfilter* unfilter,
                                       double* out) {
  return guard([&] {
    auto& u = unfref(unfilter);
    need(out != nullptr, "out is NULL");
    need(u.n_gradient() > 0, "This system does not support adjoint methods");
    u.last_gradient(out);
  });
}

int dust2_gb300_unfilter_set_save_trajectories(dust2_gb300_unfilter* unfilter,
                                               int32_t save,
                                               const size_t* index_state,
                                               size_t n_index_state) {
  return guard([&] {
    auto& u = unfref(unfilter);
    auto is = to_int_index(index_state, n_index_state, u.sys().n_state(),
                           "index_state");
    u.set_save_trajectories(save != 0, is.empty() ? nullptr : is.data(),
                            static_cast<int>(is.size()));
  });
}

int dust2_gb300_unfilter_set_save_snapshots(dust2_gb300_unfilter* unfilter,
                                            const size_t* time_index,
                                            size_t n) {
  return guard([&] {
    auto& u = unfref(unfilter);
    auto idx = to_int_index(time_index, n, u.n_times(), "save_snapshots");
    for (std::size_t i = 1; i < idx.size(); ++i) {
      need(idx[i] > idx[i - 1], "'save_snapshots' must be increasing");
    }
    u.set_save_snapshots(idx.data(), static_cast<int>(idx.size()));
  });
}

int dust2_gb300_unfilter_trajectory_dim(dust2_gb300_unfilter* unfilter,
                                        size_t* n_state, size_t* n_particles,
                                        size_t* n_groups, size_t* n_time) {
  return guard([&] {
    auto& u = unfref(unfilter);
    need(u.trajectories_current(), "Trajectories are not current");
    const auto& groups = u.saved_groups();
    *n_state = u.n_trajectory_state();
    *n_particles = u.sys().n_particles()[groups[0]];
    *n_groups = groups.size();
    *n_time = u.n_times();
  });
}

int dust2_gb300_unfilter_last_trajectories(dust2_gb300_unfilter* unfilter,
                                           double* out) {
  return guard([&] {
    auto& u = unfref(unfilter);
    need(out != nullptr, "out is NULL");
    u.last_trajectories(out);
  });
}

int dust2_gb300_unfilter_snapshot_dim(dust2_gb300_unfilter* unfilter,
                                      size_t* n_state, size_t* n_particles,
                                      size_t* n_groups,
                                      size_t* n_snapshots) {
  return guard([&] {
    auto& u = unfref(unfilter);
    need(u.snapshots_current(), "Snapshots are not current");
    const auto& groups = u.saved_groups();
    *n_state = u.sys().n_state();
    *n_particles = u.sys().n_particles()[groups[0]];
    *n_groups = groups.size();
    *n_snapshots = u.n_snapshots();
  });
}

int dust2_gb300_unfilter_last_snapshots(dust2_gb300_unfilter* unfilter,
                                        double* out) {
  return guard([&] {
    auto& u = unfref(unfilter);
    need(out != nullptr, "out is NULL");
    u.last_snapshots(out);
  });
}

int dust2_gb300_unfilter_update_pars(dust2_gb300_unfilter* unfilter,
                                     const double* pars,
                                     const size_t* index_group,
                                     size_t n_index_group) {
  return guard([&] {
    auto& u = unfref(unfilter);
    need(pars != nullptr, "pars is NULL");
    auto ig = to_int_index(index_group, n_index_group, u.sys().n_groups(),
                           "index_group");
    u.update_pars(pars, ig.empty() ? nullptr : ig.data(),
                  static_cast<int>(ig.size()));
  });
}

int dust2_gb300_unfilter_dim(const dust2_gb300_unfilter* unfilter,
                             size_t* n_state, size_t* n_particles_total,
                             size_t* n_groups, size_t* n_time) {
  return guard([&] {
    need(unfilter != nullptr && unfilter->impl != nullptr,
         "Invalid unfilter handle");
    auto& u = *unfilter->impl;
    *n_state = u.sys().n_state();
    *n_particles_total = u.sys().n_particles_total();
    *n_groups = u.sys().n_groups();
    *n_time = u.n_times();
  });
}

int dust2_gb300_unfilter_state(dust2_gb300_unfilter* unfilter, double* out) {
  return guard([&] {
    need(out != nullptr, "out is NULL");
    unfref(unfilter).sys().get_state(out);
  });
}

int dust2_gb300_server_create(const char* name, double hbm_budget_bytes,
                              size_t max_sessions,
                              dust2_gb300_server** out) {
  return guard([&] {
    need(out != nullptr, "out is NULL");
    need(max_sessions >= 1 && max_sessions <= (1u << 20),
         "'max_sessions' must be between 1 and 2^20");
    const auto* f = dust2gpu::engine::find_system(name);
    auto* impl = f->create_server(hbm_budget_bytes,
                                  static_cast<int>(max_sessions));
    *out = new dust2_gb300_server{
      std::unique_ptr<dust2gpu::engine::server_api>(impl)};
  });
}

int dust2_gb300_server_free(dust2_gb300_server* server) {
  return guard([&] { delete server; });
}

int dust2_gb300_server_capacity(dust2_gb300_server* server,
                                size_t* n_particles, size_t* n_sessions,
                                size_t* n_observations) {
  return guard([&] {
    servref(server).capacity(n_particles, n_sessions, n_observations);
  });
}

int dust2_gb300_server_open(dust2_gb300_server* server, const double* pars,
                            size_t n_particles, double time_start,
                            const double* time, size_t n_time,
                            const double* data, double dt,
                            const uint64_t* seed, size_t seed_len,
                            int64_t* session) {
  return guard([&] {
    auto& srv = servref(server);
    need(session != nullptr && pars != nullptr && data != nullptr,
         "NULL argument");
    need(n_particles >= 1 && n_particles < (1u << 29),
         "'n_particles' must be at least 1");
    need(dt > 0, "Expected 'dt' to be greater than 0");
    check_data_times(time_start, time, n_time);
    std::size_t cap_particles, cap_sessions, cap_obs;
    srv.capacity(&cap_particles, &cap_sessions, &cap_obs);
    need(n_particles <= cap_particles && n_time <= cap_obs,
         "This session needs more device memory than the server's budget");
    auto words = seed_streams(seed, seed_len, n_particles + 2);
    *session = srv.open_session(pars, static_cast<int>(n_particles),
                                time_start, time, static_cast<int>(n_time),
                                data, dt, std::move(words));
  });
}

int dust2_gb300_server_submit(dust2_gb300_server* server, int64_t session,
                              const double* pars, int64_t* ticket) {
  return guard([&] {
    need(ticket != nullptr, "ticket is NULL");
    *ticket = servref(server).submit(session, pars);
  });
}

int dust2_gb300_server_wait(dust2_gb300_server* server, int64_t ticket,
                            double timeout, double* log_likelihood,
                            double* latency) {
  int status = DUST2_GB300_OK;
  const int ret = guard([&] {
    need(log_likelihood != nullptr && latency != nullptr, "NULL argument");
    std::string error;
    status = servref(server).wait(ticket, timeout, log_likelihood, latency,
                                  &error);
    if (status == 1) {
      throw std::runtime_error(error);
    }
  });
  return ret != DUST2_GB300_OK ? ret :
    (status == 2 ? DUST2_GB300_PENDING : DUST2_GB300_OK);
}

int dust2_gb300_server_close(dust2_gb300_server* server, int64_t session) {
  return guard([&] { servref(server).close_session(session); });
}

int dust2_gb300_server_rng_state(dust2_gb300_server* server, int64_t session,
                                 uint64_t* out) {
  return guard([&] {
    need(out != nullptr, "out is NULL");
    servref(server).session_rng_state(session, out);
  });
}

int dust2_gb300_server_set_timing(dust2_gb300_server* server,
                                  int32_t enable) {
  return guard([&] { servref(server).set_timing(enable != 0); });
}

int dust2_gb300_server_stats(dust2_gb300_server* server, double* out,
                             size_t n) {
  return guard([&] {
    need(out != nullptr, "out is NULL");
    servref(server).stats(out, static_cast<int>(std::min<size_t>(n, 64)));
  });
}

}  // extern "C"
