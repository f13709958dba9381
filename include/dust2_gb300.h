/*
 * dust2_gb300: C ABI of the GPU engine for dust2's data-parallel hot path
 * (batched stepping of discrete-time stochastic systems, the bootstrap
 * particle filter, and the dopri5 integrator of continuous-time systems).
 *
 * dust2 reaches its engines through generated `.Call` entry points, one
 * family per system: `_<pkg>_dust2_system_<name>_<verb>` and
 * `_<pkg>_dust2_filter_<name>_<verb>` (src/cpp11.cpp:302-405, templates
 * inst/template/*.cpp), implemented by the adaptors in
 * inst/include/dust2/r/{system,filter,helpers}.hpp and
 * r/{discrete,continuous}/{system,filter}.hpp.  Each function below
 * replaces one of those verbs; the reference function it replaces is
 * named beside it (paths relative to the dust2 source tree).
 *
 * Conventions
 *   - Plain C types only.  Handles are opaque.
 *   - Every function returns DUST2_GB300_OK (0) or DUST2_GB300_ERROR (1);
 *     on error, dust2_gb300_last_error() returns the message (thread
 *     local), in the wording of the reference's R errors where one exists.
 *   - Indices are 0-based (the R layer subtracts 1, as
 *     r/helpers.hpp:279-306 does).
 *   - Parameters are a flat double array of n_groups rows laid out by the
 *     system's parameter table (dust2_gb300_system_info); NaN marks a
 *     value that was not given (the default applies, or, on update, the
 *     current value is kept).
 *   - State arrays use dust2's dimension order: state fastest, then
 *     particle, then group (then time for simulate).
 *   - Random number generator state is 4 uint64 words (32 bytes) per
 *     stream, in stream order; raw bytes are the little-endian words, as
 *     dust2's raw vectors.
 *   - Calls are synchronous: inputs are read and outputs written before
 *     the function returns.
 */
#ifndef DUST2_GB300_H
#define DUST2_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define DUST2_GB300_OK 0
#define DUST2_GB300_ERROR 1

typedef struct dust2_gb300_system dust2_gb300_system;
typedef struct dust2_gb300_filter dust2_gb300_filter;

/* Adaptive-stepper controls (R/interface-continuous.R dust_ode_control,
 * inst/include/dust2/continuous/control.hpp:11-27). */
typedef struct dust2_gb300_ode_control {
  int32_t max_steps;
  double atol;
  double rtol;
  double step_size_min;
  double step_size_max;
  const double* critical_times;
  size_t n_critical_times;
  int32_t debug_record_step_times;
} dust2_gb300_ode_control;

/* ---- library ---------------------------------------------------------- */

/* ABI version of this header. */
int dust2_gb300_abi_version(void);

/* Copy the calling thread's last error message into buf (NUL-terminated,
 * truncated to len); returns the full message length. */
size_t dust2_gb300_last_error(char* buf, size_t len);

/* Number of CUDA devices visible (0 without a GPU). */
int dust2_gb300_device_count(int32_t* n);

/* Measured FP64 FMA throughput of the current device in TFLOP/s
 * (independent DFMA chains on every SM); the denominator of the
 * FP64-pipe roofline.  No counterpart in dust2. */
int dust2_gb300_fp64_peak(double* tflops);

/* Names of the compiled-in systems, comma separated. */
int dust2_gb300_systems(char* buf, size_t len);

/* JSON description of a system: time type, parameter table (name, length,
 * default, required, constant), data columns.  Replaces the generator
 * metadata R reads from `[[dust2::...]]` annotations (R/metadata.R). */
int dust2_gb300_system_info(const char* name, char* json, size_t len);

/* The first n_streams generator streams of a seed (same seed forms as
 * dust2_gb300_system_alloc), 4 words per stream.  Replaces the monty
 * calls of R/interface-filter.R:120-124 (filter_rng_state:
 * monty_rng_create + monty_rng_state). */
int dust2_gb300_rng_streams(const uint64_t* seed, size_t seed_len,
                            size_t n_streams, uint64_t* out);

/* ---- systems (r/system.hpp, r/discrete/system.hpp,
 *      r/continuous/system.hpp) ------------------------------------------ */

/* dust2_discrete_alloc / dust2_continuous_alloc
 * (r/discrete/system.hpp:13-55, r/continuous/system.hpp:13-50).
 * seed: either 1 word (an integer seed, expanded with SplitMix64) or
 * 4 * k words (raw state of the first k streams; further streams are
 * successive jumps).  dt is ignored for continuous-time systems, control
 * for discrete-time ones (may be NULL: defaults). */
int dust2_gb300_system_alloc(const char* name, const double* pars,
                             size_t n_groups, size_t n_particles,
                             double time, double dt,
                             const dust2_gb300_ode_control* control,
                             const uint64_t* seed, size_t seed_len,
                             int32_t deterministic,
                             dust2_gb300_system** out);

/* Finalizer of the external pointer (r/discrete/system.hpp:46). */
int dust2_gb300_system_free(dust2_gb300_system* sys);

/* Dimensions: n_state, n_particles (per group), n_groups. */
int dust2_gb300_system_dim(const dust2_gb300_system* sys, size_t* n_state,
                           size_t* n_particles, size_t* n_groups);

/* dust2_system_state (r/system.hpp:89-161), full state:
 * out has n_state * n_particles * n_groups doubles. */
int dust2_gb300_system_state(dust2_gb300_system* sys, double* out);

/* dust2_system_set_state (r/system.hpp:189-195 via
 * internals.hpp:10-62): value holds len(index_state or n_state) *
 * len(index_particle or n_particles, or 1 when recycling particles) *
 * len(index_group or n_groups, or 1 when recycling groups) doubles; any
 * index may be NULL (all). */
int dust2_gb300_system_set_state(dust2_gb300_system* sys, const double* value,
                                 const size_t* index_state, size_t n_index_state,
                                 const size_t* index_particle,
                                 size_t n_index_particle,
                                 const size_t* index_group, size_t n_index_group,
                                 int32_t recycle_particle,
                                 int32_t recycle_group);

/* dust2_system_set_state_initial (r/system.hpp:182-187). */
int dust2_gb300_system_set_state_initial(dust2_gb300_system* sys);

/* dust2_system_time / dust2_system_set_time (r/system.hpp:163-168,
 * 240-247). */
int dust2_gb300_system_time(dust2_gb300_system* sys, double* time);
int dust2_gb300_system_set_time(dust2_gb300_system* sys, double time);

/* dust2_system_rng_state / dust2_system_set_rng_state
 * (r/system.hpp:223-238): 4 * n_particles * n_groups words. */
int dust2_gb300_system_rng_state(dust2_gb300_system* sys, uint64_t* out);
int dust2_gb300_system_set_rng_state(dust2_gb300_system* sys,
                                     const uint64_t* state, size_t len);

/* dust2_system_update_pars (r/system.hpp:249-254, r/helpers.hpp
 * update_pars): pars has one row per group (or per entry of index_group
 * when given). */
int dust2_gb300_system_update_pars(dust2_gb300_system* sys,
                                   const double* pars,
                                   const size_t* index_group,
                                   size_t n_index_group);

/* dust2_system_run_to_time (r/system.hpp:75-87). */
int dust2_gb300_system_run_to_time(dust2_gb300_system* sys, double time);

/* dust2_system_simulate (r/system.hpp:286-327): out has
 * len(index_state or n_state) * n_particles * n_groups * n_times doubles. */
int dust2_gb300_system_simulate(dust2_gb300_system* sys, const double* times,
                                size_t n_times, const size_t* index_state,
                                size_t n_index_state, double* out);

/* As dust2_gb300_system_simulate with all state, writing into device
 * memory at out_device (n_times * n_particles * n_groups * n_state
 * doubles, the same order); returns when done.  No counterpart in dust2,
 * whose verb returns host arrays: for callers that keep results on the
 * GPU. */
int dust2_gb300_system_simulate_device(dust2_gb300_system* sys,
                                       const double* times, size_t n_times,
                                       double* out_device);

/* The CUDA stream (cudaStream_t) the system's work is issued on. */
int dust2_gb300_system_stream(dust2_gb300_system* sys, void** stream);

/* dust2_system_reorder (r/system.hpp:199-221): index has
 * n_particles * n_groups entries, each a particle index within its group. */
int dust2_gb300_system_reorder(dust2_gb300_system* sys, const size_t* index,
                               size_t len);

/* dust2_system_compare_data (r/system.hpp:258-284): data holds
 * n_groups_data (1 or n_groups) rows of the system's data columns (NaN =
 * missing); out has n_particles * n_groups doubles. */
int dust2_gb300_system_compare_data(dust2_gb300_system* sys,
                                    const double* data, size_t n_groups_data,
                                    double* out);

/* dust2_system_internals (r/continuous/system.hpp:60-159), per particle:
 * step_size, error, n_steps, n_steps_accepted, n_steps_rejected.
 * Discrete-time systems have none (returns an error). */
int dust2_gb300_system_internals(dust2_gb300_system* sys, double* step_size,
                                 double* error, int64_t* n_steps,
                                 int64_t* n_steps_accepted,
                                 int64_t* n_steps_rejected);

/* Recorded step times of one particle (control.debug_record_step_times);
 * writes at most cap values and the total count to *n. */
int dust2_gb300_system_step_times(dust2_gb300_system* sys, size_t particle,
                                  double* out, size_t cap, size_t* n);

/* ---- filters (r/filter.hpp, r/discrete/filter.hpp) -------------------- */

/* dust2_discrete_filter_alloc (r/discrete/filter.hpp:13-88).
 * time: n_time data times; data: n_time * n_groups_data rows of the
 * system's data columns, time-major (r/helpers.hpp:404-427).  seed as for
 * systems; the n_groups * (n_particles + 2) streams are split per group
 * into 2 filter streams and n_particles particle streams. */
int dust2_gb300_filter_alloc(const char* name, const double* pars,
                             size_t n_groups, size_t n_particles,
                             double time_start, const double* time,
                             size_t n_time, const double* data,
                             size_t n_groups_data, double dt,
                             const uint64_t* seed, size_t seed_len,
                             dust2_gb300_filter** out);

/* dust2_continuous_filter_alloc (r/continuous/filter.hpp:13-90) for
 * mixed-time systems (an ODE with a discrete-time update every dt; dt = 0
 * runs the ODE alone).  Pure continuous-time systems are refused, as
 * R/interface-filter.R:59-65 refuses them.  control NULL = the defaults
 * of dust_ode_control.  Otherwise as dust2_gb300_filter_alloc. */
int dust2_gb300_filter_alloc_continuous(
    const char* name, const double* pars, size_t n_groups,
    size_t n_particles, double time_start, const double* time, size_t n_time,
    const double* data, size_t n_groups_data, double dt,
    const dust2_gb300_ode_control* control, const uint64_t* seed,
    size_t seed_len, dust2_gb300_filter** out);

/* As dust2_gb300_filter_alloc with a particle count per group (groups of
 * uneven size share one launch; dust2 itself requires equal counts). */
int dust2_gb300_filter_alloc_uneven(const char* name, const double* pars,
                                    size_t n_groups,
                                    const size_t* n_particles,
                                    double time_start, const double* time,
                                    size_t n_time, const double* data,
                                    size_t n_groups_data, double dt,
                                    const uint64_t* seed, size_t seed_len,
                                    dust2_gb300_filter** out);

int dust2_gb300_filter_free(dust2_gb300_filter* filter);

/* n_state, total particles, n_groups and number of data times. */
int dust2_gb300_filter_dim(const dust2_gb300_filter* filter, size_t* n_state,
                           size_t* n_particles_total, size_t* n_groups,
                           size_t* n_time);

/* dust2_filter_run (r/filter.hpp:112-143): initial may be NULL (system
 * initial conditions) or a full state; index_group may be NULL (all
 * groups).  ll receives one log-likelihood per group run. */
int dust2_gb300_filter_run(dust2_gb300_filter* filter, const double* initial,
                           const size_t* index_group, size_t n_index_group,
                           double* ll);

/* dust2_filter_update_pars (r/filter.hpp:101-110). */
int dust2_gb300_filter_update_pars(dust2_gb300_filter* filter,
                                   const double* pars,
                                   const size_t* index_group,
                                   size_t n_index_group);

/* dust2_filter_rng_state / dust2_filter_set_rng_state
 * (r/filter.hpp:273-329): per group, 2 filter streams then the group's
 * particle streams, 4 words each. */
int dust2_gb300_filter_rng_state(dust2_gb300_filter* filter, uint64_t* out,
                                 size_t len);
int dust2_gb300_filter_set_rng_state(dust2_gb300_filter* filter,
                                     const uint64_t* state, size_t len);

/* dust2_filter_last_state (r/filter.hpp:233-271): full final state, or
 * with select_random_particle one particle per group chosen from the
 * group's second filter stream (filter.hpp:130-138). */
int dust2_gb300_filter_last_state(dust2_gb300_filter* filter,
                                  int32_t select_random_particle,
                                  double* out);

/* Save trajectories in the following runs (filter.hpp:89-100, the
 * save_trajectories / index_state arguments of dust2_filter_<sys>_run,
 * r/filter.hpp:22-52): save = 1 or 0; index_state (NULL = all) selects
 * the state entries kept. */
int dust2_gb300_filter_set_save_trajectories(dust2_gb300_filter* filter,
                                             int32_t save,
                                             const size_t* index_state,
                                             size_t n_index_state);

/* Shape of dust2_gb300_filter_last_trajectories: saved state entries,
 * particles per group (1 with select_random_particle), groups of the last
 * run's index_group, data times. */
int dust2_gb300_filter_trajectory_dim(dust2_gb300_filter* filter,
                                      int32_t select_random_particle,
                                      size_t* n_state, size_t* n_particles,
                                      size_t* n_groups, size_t* n_time);

/* dust2_filter_<sys>_last_trajectories (r/filter.hpp:55-96): the last
 * run's trajectories with each particle's ancestry followed back through
 * the resampling (trajectories.hpp:135-190), state fastest, then
 * particle, group, time; with select_random_particle one particle per
 * group (as dust2_gb300_filter_last_state).  Fails with "Trajectories are
 * not current" unless the last run saved them.  Groups must have equal
 * particle counts. */
int dust2_gb300_filter_last_trajectories(dust2_gb300_filter* filter,
                                         int32_t select_random_particle,
                                         double* out);

/* Save snapshots of the full state in the following runs
 * (save_snapshots of dust2_filter_<sys>_run; trajectories.hpp:84-97) at
 * the data times with these 0-based indices (increasing; n = 0 stops
 * saving).  The R layer maps snapshot times to indices and rejects times
 * not in the data (R/interface-likelihood.R:83-92). */
int dust2_gb300_filter_set_save_snapshots(dust2_gb300_filter* filter,
                                          const size_t* time_index,
                                          size_t n);

/* Shape of dust2_gb300_filter_last_snapshots: state entries, particles
 * per group (1 with select_random_particle), groups, snapshots. */
int dust2_gb300_filter_snapshot_dim(dust2_gb300_filter* filter,
                                    int32_t select_random_particle,
                                    size_t* n_state, size_t* n_particles,
                                    size_t* n_groups, size_t* n_snapshots);

/* dust2_filter_<sys>_last_snapshots (r/filter.hpp:98-137): the saved
 * states with ancestry followed back through the resampling
 * (trajectories.hpp:199-268); layout and random particle as
 * dust2_gb300_filter_last_trajectories.  Fails with "Snapshots are not
 * current" unless the last run saved them. */
int dust2_gb300_filter_last_snapshots(dust2_gb300_filter* filter,
                                      int32_t select_random_particle,
                                      double* out);

/* Groups whose resampling was recomputed serially so far (diagnostic of
 * the exact-resampling check). */
int dust2_gb300_filter_serial_fallbacks(dust2_gb300_filter* filter,
                                        int64_t* n);

/* ---- filter helpers (src/test.cpp:10-23) ------------------------------- */

/* test_resample_weight (filter_details.hpp:45-74): systematic resampling
 * of n non-negative weights w with uniform u; idx receives the 0-based
 * source particle of each of the n new particles.  Runs the filter's GPU
 * resampling kernels (exact: ties within rounding distance fall back to
 * the serial algorithm). */
int dust2_gb300_resample_weight(const double* w, size_t n, double u,
                                size_t* idx);

/* test_scale_log_weights (filter_details.hpp:11-39): replaces the n log
 * weights in w by exp(w - max) (NaN -> weight 0), and writes
 * log(mean(exp(w - max))) + max to result; a single weight is returned
 * unchanged; all -Inf gives -Inf with the weights left as log weights. */
int dust2_gb300_scale_log_weights(double* w, size_t n, double* result);

/* dust2_gb300_resample_weight without any device allocation: the
 * working arrays live in a fixed scratch area compiled into the library
 * (2 MiB reserved on every device that loads it; a call uses at most
 * about 1.9 MB).  For callers that cannot allocate device memory at call
 * time, e.g. when another allocator owns the GPU's memory or when
 * cudaFree's device-wide synchronisation is unacceptable.  At most 65536
 * weights (an error otherwise).  Runs on the calling thread's per-thread
 * default stream (cudaStreamPerThread).  The first call on a device looks
 * up the scratch area's address with that device current and later calls
 * reuse it: make the first call before any stream capture, and do not
 * call it on a device after cudaDeviceReset in the same process.  All
 * calls share the area, so calls that overlap on the GPU race: serialise
 * them.  No counterpart in dust2. */
int dust2_gb300_resample_weight_noalloc(const double* w, size_t n, double u,
                                        size_t* idx);

/* 1: resample every group with the serial algorithm of
 * filter_details.hpp:45-74 (verification of the parallel resampler);
 * 0 (default): parallel search with the serial algorithm only for groups
 * whose decision is within rounding distance of a boundary. */
int dust2_gb300_filter_set_serial_resample(dust2_gb300_filter* filter,
                                           int32_t serial);

/* 1 (default): when every group has at most 1024 particles, the weights,
 * log-likelihood, resampling and reorder of an observation run as one
 * launch with one block per group; 0: as separate kernels over the whole
 * particle range.  The results are identical; this is a tuning switch
 * with no counterpart in dust2. */
int dust2_gb300_filter_set_fused_tail(dust2_gb300_filter* filter,
                                      int32_t fused);

/* Asynchronous form of dust2_gb300_filter_run (system initial conditions,
 * current parameters): enqueues the run on the filter's CUDA stream and
 * returns; results stay on the device.  No counterpart in dust2, whose
 * verbs are synchronous; it lets a caller keep several filters busy. */
int dust2_gb300_filter_run_async(dust2_gb300_filter* filter,
                                 const size_t* index_group,
                                 size_t n_index_group);

/* Wait for the last run and copy one log-likelihood per group (all
 * groups) into ll; reports errors of an asynchronous run. */
int dust2_gb300_filter_last_log_likelihood(dust2_gb300_filter* filter,
                                           double* ll);

/* The CUDA stream (cudaStream_t) the filter's work is issued on. */
int dust2_gb300_filter_stream(dust2_gb300_filter* filter, void** stream);

/* Enable (1) or disable (0) device timing of the filter's step kernels:
 * CUDA events recorded around every step launch inside the captured
 * graph.  Resets the accumulated times. */
int dust2_gb300_filter_set_timing(dust2_gb300_filter* filter, int32_t enable);

/* Accumulated device time of the step kernels (ms, number of launches)
 * and of whole runs (ms, number of runs) since timing was enabled. */
int dust2_gb300_filter_kernel_times(dust2_gb300_filter* filter,
                                    double* step_ms, int64_t* n_step_launches,
                                    double* run_ms, int64_t* n_runs);

/* Accumulated device time (ms) and number of the reorder launches (the
 * state gather of discrete/system.hpp:170-181) timed the same way; none
 * are timed when the filter's tail runs as one cluster launch (groups of
 * at most 1024 particles).  No counterpart in the reference: it serves
 * the benchmark's HBM roofline of the gather. */
int dust2_gb300_filter_reorder_times(dust2_gb300_filter* filter, double* ms,
                                     int64_t* n_launches);

/* The step kernel's launch shape: group tiles of `block` threads
 * (per_tile 0), or one-warp tiles of per_tile (1..32) particles (block
 * 32); one block per tile (persistent 0), or (persistent 1) a grid that
 * fills the device once and takes tiles from a device work queue.  By default (autotune 1) the filter times every candidate
 * shape once, before its first run, on scratch copies of its particles,
 * and keeps the fastest; set_step_shape forces one and turns that off.
 * Results do not depend on the shape.  No counterpart in the reference,
 * whose CPU loop has no launch shape. */
int dust2_gb300_filter_set_autotune(dust2_gb300_filter* filter,
                                    int32_t enable);
int dust2_gb300_filter_set_step_shape(dust2_gb300_filter* filter,
                                      int32_t block, int32_t per_tile,
                                      int32_t persistent);
/* The shape in use, how many candidates were timed (0 before tuning or
 * when it was skipped) and the chosen candidate's time (ms) for one
 * observation's steps. */
int dust2_gb300_filter_step_shape(dust2_gb300_filter* filter, int32_t* block,
                                  int32_t* per_tile, int32_t* persistent,
                                  int32_t* n_candidates, double* best_ms);

/* ---- deterministic likelihood (r/unfilter.hpp, unfilter.hpp) ---------- */

typedef struct dust2_gb300_unfilter dust2_gb300_unfilter;

/* dust2_unfilter_<sys>_alloc (r/discrete/unfilter.hpp:14-56,
 * r/continuous/unfilter.hpp:14-56): a deterministic system of n_groups x
 * n_particles with data as for dust2_gb300_filter_alloc; control (may be
 * NULL for the defaults) applies to continuous-time systems, dt to
 * discrete-time ones. */
int dust2_gb300_unfilter_alloc(const char* name, const double* pars,
                               size_t n_groups, size_t n_particles,
                               double time_start, const double* time,
                               size_t n_time, const double* data,
                               size_t n_groups_data, double dt,
                               const dust2_gb300_ode_control* control,
                               dust2_gb300_unfilter** out);

int dust2_gb300_unfilter_free(dust2_gb300_unfilter* unfilter);

/* dust2_unfilter_<sys>_run (r/unfilter.hpp:20-62, unfilter.hpp:42-73):
 * initial (NULL = initial conditions) is a full state in dust2's order;
 * ll receives n_particles values per group of index_group (NULL = all),
 * the log-likelihood of each particle summed over the data. */
int dust2_gb300_unfilter_run(dust2_gb300_unfilter* unfilter,
                             const double* initial,
                             const size_t* index_group,
                             size_t n_index_group, double* ll);

/* dust2_unfilter_<sys>_run with adjoint = TRUE (r/unfilter.hpp:42-44,
 * unfilter.hpp:77-110): the same log-likelihood as
 * dust2_gb300_unfilter_run, through the saved state history, and the
 * gradient of each particle's log-likelihood with respect to the
 * system's packing_gradient parameters.  A system without adjoint support
 * runs as dust2_gb300_unfilter_run and has no current gradient. */
int dust2_gb300_unfilter_run_adjoint(dust2_gb300_unfilter* unfilter,
                                     const double* initial,
                                     const size_t* index_group,
                                     size_t n_index_group, double* ll);

/* Gradient length (packing_gradient; 0 without adjoint support) and the
 * groups covered by the current gradient (0 when the last run was not an
 * adjoint run). */
int dust2_gb300_unfilter_gradient_dim(const dust2_gb300_unfilter* unfilter,
                                      size_t* n_gradient,
                                      size_t* n_groups_last);

/* dust2_discrete_unfilter_last_gradient (r/unfilter.hpp:153-180,
 * unfilter.hpp:135-142): n_gradient x n_particles x n_groups_last
 * doubles, gradient entries fastest.  Fails with "System was not run with
 * 'adjoint = TRUE'" after a plain run.  Unlike the reference, more than
 * one particle per group is supported (each particle's own gradient). */
int dust2_gb300_unfilter_last_gradient(dust2_gb300_unfilter* unfilter,
                                       double* out);

/* Save trajectories (state entries index_state, NULL = all) at every
 * data time in the following runs (save_trajectories / index_state of
 * dust2_unfilter_<sys>_run, r/unfilter.hpp:20-47, unfilter.hpp:60-62,
 * 100-102). */
int dust2_gb300_unfilter_set_save_trajectories(dust2_gb300_unfilter* unfilter,
                                               int32_t save,
                                               const size_t* index_state,
                                               size_t n_index_state);

/* Save the full state at the data times time_index (increasing; 0-based
 * data-time positions) in the following runs (save_snapshots of
 * dust2_unfilter_<sys>_run; trajectories.hpp:84-97).  Unlike the
 * reference's plain run, snapshots are kept whether or not trajectories
 * are. */
int dust2_gb300_unfilter_set_save_snapshots(dust2_gb300_unfilter* unfilter,
                                            const size_t* time_index,
                                            size_t n);

/* Shape of dust2_gb300_unfilter_last_trajectories: saved entries,
 * particles per group, groups of the run that saved them, data times. */
int dust2_gb300_unfilter_trajectory_dim(dust2_gb300_unfilter* unfilter,
                                        size_t* n_state, size_t* n_particles,
                                        size_t* n_groups, size_t* n_time);

/* dust2_unfilter_<sys>_last_trajectories (r/unfilter.hpp:64-93): entries
 * fastest, then particle, group, data time.  Fails with "Trajectories are
 * not current" unless the last run saved them. */
int dust2_gb300_unfilter_last_trajectories(dust2_gb300_unfilter* unfilter,
                                           double* out);

/* Shape of dust2_gb300_unfilter_last_snapshots: state entries, particles
 * per group, groups, snapshots. */
int dust2_gb300_unfilter_snapshot_dim(dust2_gb300_unfilter* unfilter,
                                      size_t* n_state, size_t* n_particles,
                                      size_t* n_groups,
                                      size_t* n_snapshots);

/* dust2_unfilter_<sys>_last_snapshots (r/unfilter.hpp:95-125); layout as
 * dust2_gb300_unfilter_last_trajectories.  Fails with "Snapshots are not
 * current" unless the last run saved them. */
int dust2_gb300_unfilter_last_snapshots(dust2_gb300_unfilter* unfilter,
                                        double* out);

/* The state packing (packing_state of the system class; the
 * `packing_state` element that dust2_discrete_alloc,
 * dust2_discrete_filter_alloc and the unfilter allocators return,
 * r/discrete/system.hpp:46-53) as JSON, [{"name": "S", "dims": []}, ...],
 * into buf (NUL-terminated, truncated to len; *needed = full length, may
 * be NULL).  Used by dust_unpack_state / dust_unpack_index. */
int dust2_gb300_system_packing_state(dust2_gb300_system* sys, char* buf,
                                     size_t len, size_t* needed);
int dust2_gb300_filter_packing_state(dust2_gb300_filter* filter, char* buf,
                                     size_t len, size_t* needed);
int dust2_gb300_unfilter_packing_state(dust2_gb300_unfilter* unfilter,
                                       char* buf, size_t len,
                                       size_t* needed);

/* dust2_unfilter_<sys>_update_pars (r/unfilter.hpp:10-18). */
int dust2_gb300_unfilter_update_pars(dust2_gb300_unfilter* unfilter,
                                     const double* pars,
                                     const size_t* index_group,
                                     size_t n_index_group);

/* Dimensions: state length, particles over all groups, groups, data
 * times. */
int dust2_gb300_unfilter_dim(const dust2_gb300_unfilter* unfilter,
                             size_t* n_state, size_t* n_particles_total,
                             size_t* n_groups, size_t* n_time);

/* State after the last run (dust_likelihood_last_state for an unfilter):
 * n_state x n_particles x n_groups doubles. */
int dust2_gb300_unfilter_state(dust2_gb300_unfilter* unfilter, double* out);

/* ---- likelihood server ---------------------------------------------------
 *
 * Continuous batching of filter likelihoods for many concurrent callers
 * (MCMC chains).  dust2 has no counterpart: each chain calls
 * dust_likelihood_run (R/interface-likelihood.R, filter.hpp:42-104) on
 * its own object, one run at a time, from dust_likelihood_monty
 * (R/monty.R:90-317).  Here each chain opens a session (its likelihood
 * object: one parameter group, particle count, data and generator
 * streams, kept on the device) and submits requests (a run at new
 * parameters); the server runs all pending requests together, one
 * observation per step of the device loop, admitting sessions as slots
 * and memory under the HBM budget free up.  A request's result equals
 * that of dust2_gb300_filter_run on a one-group filter created with the
 * same parameters, data and seed, after the same earlier runs.
 *
 * Calls are thread safe; submit returns at once, wait blocks. */

typedef struct dust2_gb300_server dust2_gb300_server;

#define DUST2_GB300_PENDING 2

/* A server for system `name` (a discrete-time system with compare_data)
 * using at most hbm_budget_bytes of device memory for particles, data
 * and per-session state, with at most max_sessions resident sessions. */
int dust2_gb300_server_create(const char* name, double hbm_budget_bytes,
                              size_t max_sessions,
                              dust2_gb300_server** out);

/* Stop the server: requests not yet started fail, running ones finish. */
int dust2_gb300_server_free(dust2_gb300_server* server);

/* Particles, sessions and observations the budget holds. */
int dust2_gb300_server_capacity(dust2_gb300_server* server,
                                size_t* n_particles, size_t* n_sessions,
                                size_t* n_observations);

/* Open a session: as dust2_gb300_filter_alloc with n_groups = 1 (pars one
 * row of the parameter table; data n_time rows, time-major; seed as
 * there).  The session becomes resident as soon as memory allows. */
int dust2_gb300_server_open(dust2_gb300_server* server, const double* pars,
                            size_t n_particles, double time_start,
                            const double* time, size_t n_time,
                            const double* data, double dt,
                            const uint64_t* seed, size_t seed_len,
                            int64_t* session);

/* Queue one likelihood evaluation of `session`.  pars (one row; NaN keeps
 * a value) updates the session's parameters first, as
 * dust2_gb300_filter_update_pars does; NULL keeps them. */
int dust2_gb300_server_submit(dust2_gb300_server* server, int64_t session,
                              const double* pars, int64_t* ticket);

/* Wait at most `timeout` seconds (negative: no limit) for a request:
 * DUST2_GB300_OK with its log-likelihood and latency (seconds from submit
 * to result), DUST2_GB300_ERROR if it failed (message as for particle
 * errors of a filter run), DUST2_GB300_PENDING if not finished in time.
 * A finished ticket is consumed. */
int dust2_gb300_server_wait(dust2_gb300_server* server, int64_t ticket,
                            double timeout, double* log_likelihood,
                            double* latency);

/* Close a session once its queued requests have run. */
int dust2_gb300_server_close(dust2_gb300_server* server, int64_t session);

/* Generator state of a session (waits until it is idle), in the layout of
 * dust2_gb300_filter_rng_state for one group: 2 + n_particles streams. */
int dust2_gb300_server_rng_state(dust2_gb300_server* server, int64_t session,
                                 uint64_t* out);

/* Enable (1) or disable (0) device timing of the step+compare kernel of
 * every device step (CUDA events); resets the accumulated time. */
int dust2_gb300_server_set_timing(dust2_gb300_server* server,
                                  int32_t enable);

/* Counters: [0] device steps (observations advanced), [1] particle-steps
 * of started requests, [2] finished requests, [3] resident sessions,
 * [4] sessions waiting for memory, [5] queued requests, [6] particle
 * capacity, [7] particles in use, [8] most requests running at once,
 * [9] step-kernel device time (ms, while timing), [10] timed device
 * steps, [11] kernel launches.  Writes min(n, 12) values. */
int dust2_gb300_server_stats(dust2_gb300_server* server, double* out,
                             size_t n);

#ifdef __cplusplus
}
#endif

#endif
