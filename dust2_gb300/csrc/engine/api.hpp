// Type-erased interfaces between the C ABI and the templated engines.
// One object of each kind exists per allocated system / filter handle;
// the C ABI (capi.cu) owns them and turns C++ exceptions into status
// codes.
#pragma once

#include <cstdint>
#include <string>
#include <vector>

#include "../dust2gpu/common.hpp"
#include "../dust2gpu/system.hpp"

namespace dust2gpu {
namespace engine {

// Summary of per-particle errors in the format of
// inst/include/dust2/errors.hpp:29-54.
std::string format_errors(const std::vector<particle_error>& errors,
                          const char* title = "particles",
                          std::size_t n_max = 4);
std::string describe_error(const particle_error& e);

// Set the calling thread's error message returned by
// dust2_gb300_last_error (for entry points outside capi.cu).
void set_last_error(const std::string& msg);

struct ode_control {
  // inst/include/dust2/continuous/control.hpp:11-27; step_size_min is
  // clamped below by machine epsilon as in
  // inst/include/dust2/r/continuous/control.hpp:15-17.
  int max_steps = 10000;
  double atol = 1e-6;
  double rtol = 1e-6;
  double step_size_min = 1e-8;
  double step_size_max = 1.0 / 0.0;
  double factor_safe = 0.9;
  double factor_min = 0.2;
  double factor_max = 10.0;
  double beta = 0.04;
  double constant = 0.2 - 0.04 * 0.75;
  std::vector<double> critical_times;
  bool debug_record_step_times = false;
};

// Per-particle solver statistics (dust_system_internals, R/interface.R).
struct ode_internals_row {
  double step_size;
  double error;
  long n_steps;
  long n_steps_accepted;
  long n_steps_rejected;
};

class system_api {
public:
  virtual ~system_api() = default;

  virtual const char* name() const = 0;
  virtual bool is_continuous() const = 0;
  virtual bool has_compare() const = 0;
  virtual int n_state() const = 0;
  virtual int n_groups() const = 0;
  virtual int n_particles_total() const = 0;
  virtual const std::vector<int>& n_particles() const = 0;
  virtual std::vector<packing_entry> packing_state() const = 0;

  virtual double time() const = 0;
  virtual double dt() const = 0;
  virtual void set_time(double time) = 0;

  virtual void run_to_time(double time) = 0;
  virtual void set_state_initial() = 0;
  // Full state in dust2's dimension order: state fastest, then particle,
  // then group.
  virtual void get_state(double* out) = 0;
  virtual void put_state(const double* in) = 0;
  // Raw generator state: 4 words per stream, streams in particle order.
  virtual void get_rng_state(std::uint64_t* out) = 0;
  virtual void put_rng_state(const std::uint64_t* in) = 0;
  virtual int n_pars() const = 0;
  virtual void update_pars(const double* pars, const int* index_group,
                           int n_index_group) = 0;
  // out: [time][group][particle][index_state or all state]
  virtual void simulate(const double* times, int n_times,
                        const int* index_state, int n_index_state,
                        double* out) = 0;
  // simulate with all state, output left in device memory (out_dev, the
  // same order); returns when the work is done
  virtual void simulate_device(const double* times, int n_times,
                               double* out_dev) = 0;
  // the CUDA stream the system's work is issued on
  virtual void* stream_handle() = 0;
  // index: group-local particle index per particle, group-major
  virtual void reorder(const int* index) = 0;
  // data: [group][n_data] doubles; out: [group][particle]
  virtual int n_data() const = 0;
  virtual void compare_data(const double* data, int n_groups_data,
                            double* out) = 0;
  virtual bool errors_pending() const = 0;
  virtual std::vector<ode_internals_row> ode_internals() = 0;
  virtual std::vector<std::vector<double>> ode_step_times() = 0;
};

class filter_api {
public:
  virtual ~filter_api() = default;
  virtual system_api& sys() = 0;
  virtual int n_times() const = 0;
  // initial: optional full state (dust2 order) applied instead of the
  // system's initial conditions; index_group: groups to run (nullptr =
  // all).  ll_out receives one value per requested group.
  virtual void run(const double* initial, const int* index_group,
                   int n_index_group, double* ll_out) = 0;
  virtual void update_pars(const double* pars, const int* index_group,
                           int n_index_group) = 0;
  // Raw generator state in the layout of
  // inst/include/dust2/r/filter.hpp:273-298: per group, the 2 filter
  // streams followed by that group's particle streams.
  virtual void get_rng_state(std::uint64_t* out) = 0;
  virtual void put_rng_state(const std::uint64_t* in) = 0;
  virtual std::size_t n_rng_streams() const = 0;
  // For each group, draw (once per run) a random particle from the
  // group's second filter stream (filter.hpp:130-138).
  virtual std::vector<int> select_random_particle() = 0;
  virtual bool has_run() const = 0;
  // Fallback statistics of the resampler: groups recomputed serially.
  virtual long n_serial_fallbacks() const = 0;
  // Run options.
  virtual void set_use_graph(bool use) = 0;
  // Resample every group with the serial algorithm (verification mode).
  virtual void set_serial_resample(bool serial) = 0;
  // Run the per-observation tail of filters whose groups all have at most
  // 1024 particles as one launch (default) or as separate kernels; both
  // give the same results.
  virtual void set_fused_tail(bool fused) = 0;
  // Enqueue a run on the filter's stream without waiting; the
  // log-likelihood stays on the device until last_log_likelihood().
  virtual void run_async(const int* index_group, int n_index_group) = 0;
  virtual void last_log_likelihood(double* ll_out) = 0;
  virtual void* stream_handle() = 0;
  // Record CUDA events around every step kernel (inside the graph) and
  // accumulate their device time.
  virtual void set_timing(bool enable) = 0;
  virtual void kernel_times(double* step_ms, long* n_step_launches,
                            double* run_ms, long* n_runs) = 0;
  // Device time of the reorder (state gather) launches timed the same
  // way, when the tail runs as separate kernels (else none are timed).
  virtual void reorder_times(double* ms, long* n_launches) = 0;
  // The step kernel's launch shape (filter.cuh step_shape): tuned by
  // timing candidates before the first run (enable), forced, or read.
  virtual void set_autotune(bool enable) = 0;
  virtual void set_step_shape(int block, int per_tile, bool persistent) = 0;
  virtual void step_shape_info(int* block, int* per_tile, int* persistent,
                               int* n_candidates, double* best_ms) = 0;
  // Save trajectories in the following runs (index_state: state entries,
  // nullptr = all); export those of the last run for `groups`, all
  // particles or select[i] of each, as [time][group][particle][state].
  virtual void set_save_trajectories(bool save, const int* index_state,
                                     int n_index_state) = 0;
  virtual bool trajectories_current() const = 0;
  virtual int n_trajectory_state() const = 0;
  virtual void last_trajectories(const int* groups, int n_groups,
                                 const int* select, double* out) = 0;
  // Snapshots of the full state at the data times with these indices.
  virtual void set_save_snapshots(const int* obs, int n_obs) = 0;
  virtual bool snapshots_current() const = 0;
  virtual int n_snapshots() const = 0;
  virtual void last_snapshots(const int* groups, int n_groups,
                              const int* select, double* out) = 0;
};

// The deterministic likelihood (dust2::unfilter, unfilter.hpp:10-73).
class unfilter_api {
public:
  virtual ~unfilter_api() = default;
  virtual system_api& sys() = 0;
  virtual int n_times() const = 0;
  // initial: optional full state used instead of the initial conditions;
  // index_group: groups to run (nullptr = all); ll_out: n_particles
  // values per requested group, in index_group order.
  virtual void run(const double* initial, const int* index_group,
                   int n_index_group, double* ll_out) = 0;
  virtual void update_pars(const double* pars, const int* index_group,
                           int n_index_group) = 0;
  // Gradient entries of the system (packing_gradient; 0 without adjoint
  // support), and the adjoint run returning them with the likelihood.
  virtual int n_gradient() const = 0;
  virtual void run_adjoint(const double* initial, const int* index_group,
                           int n_index_group, double* ll_out) = 0;
  virtual void last_gradient(double* out) = 0;
  virtual int n_last_gradient_groups() const = 0;
  // Trajectories (state entries index_state, nullptr = all, at every data
  // time) and snapshots (full state at the data times `obs`) of the
  // following runs (unfilter.hpp:42-73 trajectories_.add); exports are
  // [time][group][particle][entry] over the groups of the run that saved
  // them, no reordering (r/unfilter.hpp:64-136).
  virtual void set_save_trajectories(bool save, const int* index_state,
                                     int n_index_state) = 0;
  virtual void set_save_snapshots(const int* obs, int n_obs) = 0;
  virtual bool trajectories_current() const = 0;
  virtual bool snapshots_current() const = 0;
  virtual int n_trajectory_state() const = 0;
  virtual int n_snapshots() const = 0;
  virtual const std::vector<int>& saved_groups() const = 0;
  virtual void last_trajectories(double* out) = 0;
  virtual void last_snapshots(double* out) = 0;
};

}  // namespace engine
}  // namespace dust2gpu
