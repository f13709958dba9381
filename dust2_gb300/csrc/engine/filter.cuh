// Bootstrap particle filter on the GPU: the counterpart of dust2::filter
// (inst/include/dust2/filter.hpp:11-176) and its helpers
// scale_log_weights / resample_weight (filter_details.hpp:11-74).
//
// Per data time, for the groups being run:
//   1. k_step_compare  one thread per particle: advance the particle to
//                      the data time (filter.hpp:59), evaluate
//                      compare_data (:60), and reduce per group the
//                      "any weight non-zero" flag (:71-72) and the maximum
//                      log weight (filter_details.hpp:19-25; NaN counts as
//                      -Inf).
//   2. k_weights       w = exp(logw - max); one warp per 32-particle
//                      chunk of a group: inclusive prefix sums and the
//                      chunk total (FP64).
//   3. k_group         one block per group: scan of the chunk totals
//                      (one warp per window of 32 chunks), the
//                      log-likelihood increment log(sum/n) + max (:32-38),
//                      and the uniform u from the group's filter stream 2g
//                      (filter.hpp:75).
//   4. k_resample      one thread per particle: systematic resampling
//                      target uu_i = sum*u/n + i*sum/n and a search of the
//                      prefix sums (filter_details.hpp:45-74).
//   5. k_fallback      one block per flagged group: the serial algorithm
//                      (its running sum reproduced exactly in parallel).
//   6. k_reorder       gather of the resampled state (discrete/system.hpp
//                      :170-181).
//
// The sums of steps 2-3 have a fixed structure (chunks of 32 particles,
// then windows of 32 chunks with a carry) that does not depend on the
// tile size, so neither the log-likelihood nor the indices do.
//
// Exactness of the resampling indices.  dust2 accumulates the weights
// serially; a parallel scan rounds differently, so a search target that
// falls within a few ulps of a cumulative boundary could pick a
// neighbouring particle.  Step 4 therefore checks every decision against
// a rigorous, position-dependent bound on the difference between the
// serial and the parallel prefix sums (see k_resample); a decision is
// accepted only when both neighbouring prefix sums are farther than that
// from the target, otherwise the whole group is recomputed with the
// reference algorithm (step 5), whose left-to-right running sum the block
// reproduces bit for bit (exact_running_sums in filter_kernels.cu).  The
// log-likelihood uses the parallel total; it matches the serial one to
// better than n u relative (u = 2^-53).
//
// When every group has at most 1024 particles, steps 2-6 run as one
// launch, k_tail_cluster (a cluster of blocks per group), with the same
// results.
//
// The whole sequence for all data times is captured once into a CUDA
// graph and replayed on every run.
#pragma once

#include <cuda_runtime.h>

#include <cfloat>
#include <cmath>
#include <memory>
#include <vector>

#include "../dust2gpu/math.hpp"
#include "../dust2gpu/random.hpp"
#include "api.hpp"
#include "continuous.cuh"
#include "device.cuh"
#include "discrete.cuh"
#include "kernels_common.cuh"

namespace dust2gpu {
namespace engine {

enum group_mode : int {
  MODE_KEEP = 0,      // no data: particles stay where they are
  MODE_RESAMPLE = 1,  // systematic resampling by weight
  MODE_FIRST = 2      // every particle takes particle 0 (n == 1 or all -Inf)
};

// Per-group scratch of the filter, all device pointers.
struct filter_view {
  const tile* tiles;
  const int* active;          // [n_groups] 1 = run this group
  const int* n_particles;     // [n_groups]
  const int* offset;          // [n_groups]
  const int* chunk_first;     // [n_groups] first 32-particle chunk
  const int* chunk_count;     // [n_groups]
  double* w;                  // [n_total] raw log weights
  double* ew;                 // [n_total] exp(w - max)
  double* pre;                // [n_total] tile-local inclusive prefix
  double* chunk_sum;          // [n_chunks] chunk totals of ew (ends after k_group)
  double* chunk_off;          // [n_chunks] exclusive offsets within group
  unsigned long long* gkey;   // [n_groups] ordered key of max log weight
  int* gnz;                   // [n_groups] any weight != 0
  int* gflag;                 // [n_groups] ambiguous decision seen
  int* mode;                  // [n_groups] group_mode
  double* ll;                 // [n_groups]
  double* gu;                 // [n_groups] uniform draw
  double* guu0;               // [n_groups]
  double* gdu;                // [n_groups]
  double* gtot;               // [n_groups]
  int* idx;                   // [n_total] group-local source particle
  std::uint64_t* frng;        // [2 n_groups][4] filter streams
  int* set_initial;           // scalar flag read by the initial kernel
  const int* force_serial;    // scalar flag: resample every group serially
};

__global__ void k_filter_reset(filter_view f, int n_groups);

// Launch shape of the filter's step kernel: group tiles of `block`
// particles (per_tile == 0), or one-warp tiles of per_tile particles
// (block 32); one block per tile, or (persistent) a grid that fills the
// device once and takes tiles from a device work queue.  Every shape
// gives the same results: the step kernel is per particle, and its group
// reductions (any non-zero weight, maximum log weight) are atomics that
// do not depend on order.
struct step_shape {
  int block;
  int per_tile;
  bool persistent;
};

template <typename T>
DUST2_PARTICLE_KERNEL(T) k_initial_flagged(system_view<T> v, const int* flag,
                                  double time) {
  __shared__ shared_smem<T> sm;
  if (*flag == 0) {
    return;
  }
  const tile tl = v.tiles[blockIdx.x];
  sm.load(v, tl.group);
  __syncthreads();
  if (static_cast<int>(threadIdx.x) >= tl.count) {
    return;
  }
  const int k = tl.start + threadIdx.x;
  auto rng = load_rng(v.rng, v.stride, k, v.deterministic);
  typename T::internal_state internal{};
  double x[T::n_state_max];
  load_state<T>(v, k, x);
  T::initial(time, sm.shared(), internal, rng, x);
  store_state<T>(v, k, x);
  store_rng(v.rng, v.stride, k, rng);
  capture_error(v.errors, v.any_error, k, rng);
}

// The per-tile work of k_step_compare, shared with the likelihood
// server: advance each particle of tile `tl` n_steps from `time`, compare
// it with `d` (this tile's data row), store its log weight, and reduce the
// group's "any weight non-zero" flag and maximum log weight.
template <typename T>
__device__ __forceinline__ void step_compare_tile(
    const system_view<T>& v, const filter_view& f, const tile& tl,
    shared_smem<T>& sm, double* red, double time, double dt, int n_steps,
    double time_compare, const typename T::data_type* d) {
  sm.load(v, tl.group);
  sm.load_zero_steps(v, tl.group, time, dt, n_steps);
  __syncthreads();
  const bool valid = static_cast<int>(threadIdx.x) < tl.count;
  double logw = 0;
  if (valid) {
    const int k = tl.start + threadIdx.x;
    auto rng = load_rng(v.rng, v.stride, k, v.deterministic);
    typename T::internal_state internal{};
    double x[T::n_state_max];
    double y[update_in_place_of<T>::value ? 1 : T::n_state_max];
    load_state<T>(v, k, x);
    run_particle<T>(time, dt, n_steps, sm.shared(), internal, sm.zero,
                    sm.zero_steps, rng, x, y);
    logw = T::compare_data(time_compare, x, *d, sm.shared(), internal, rng);
    store_state<T>(v, k, x);
    store_rng(v.rng, v.stride, k, rng);
    capture_error(v.errors, v.any_error, k, rng);
    f.w[k] = logw;
  }
  // NaN != 0 counts as data (filter.hpp:71-72); NaN is -Inf for the max.
  const int nz = __syncthreads_or(valid && logw != 0);
  const double mx = block_max(valid && !(logw != logw) ? logw : -INFINITY,
                              red);
  if (threadIdx.x == 0) {
    if (nz) {
      atomicOr(f.gnz + tl.group, 1);
    }
    atomicMax(f.gkey + tl.group, ordered_key(mx));
  }
}

// k_step_compare for mixed-time systems (filter.hpp:59-60 over
// dust_continuous): each particle integrates from time0 to the data time
// with its solver record (initialised first when `initialise` is set, at
// the first data time of a run), applying updates every dt (see
// advance()), and compares its state as it stands, outputs not refreshed
// (continuous/system.hpp:279-305).  The group reductions are
// k_step_compare's.
template <typename T>
DUST2_PARTICLE_KERNEL(T) k_step_compare_mixed(
    system_view<T> v, ode_view o, dopri5::control_dev ctl, filter_view f,
    double time0, double time, double dt, int initialise,
    const typename T::data_type* data, int n_groups_data) {
  constexpr int NV = n_var_max<T>();
  __shared__ shared_smem<T> sm;
  __shared__ double red[33];
  const tile tl = v.tiles[blockIdx.x];
  if (!f.active[tl.group]) {
    return;
  }
  sm.load(v, tl.group);
  __syncthreads();
  const bool valid = static_cast<int>(threadIdx.x) < tl.count;
  double logw = 0;
  if (valid) {
    const int k = tl.start + threadIdx.x;
    const auto& shared = sm.shared();
    auto rng = load_rng(v.rng, v.stride, k, v.deterministic);
    typename T::internal_state internal{};
    const int n_var = v.n_state - T::n_output - n_special<T>();
    double y[T::n_state_max];
    load_state<T>(v, k, y);
    dopri5::state<NV> st;
    dopri5::scratch<NV> s;
    load_ode<NV>(o, k, n_var, st);
    dopri5::solver<T, NV> sol{ctl, shared, internal, n_var, k};
    sol.n_special = n_special<T>();
    if (initialise) {
      sol.initialise(time0, y, st, s);
    }
    int update_err = 0;
    if (st.err == 0) {
      update_err = advance<T, NV>(sol, time0, time, dt, y, sm.zero, st, s,
                                  rng, shared, internal);
    }
    const auto& d = data[n_groups_data == 1 ? 0 : tl.group];
    logw = T::compare_data(time, y, d, shared, internal, rng);
    store_state<T>(v, k, y);
    store_ode<NV>(o, k, n_var, st);
    if (st.err != 0 || update_err != 0) {
      rng.err = st.err != 0 ? st.err : update_err;
    }
    capture_error(v.errors, v.any_error, k, rng);
    f.w[k] = logw;
  }
  const int nz = __syncthreads_or(valid && logw != 0);
  const double mx = block_max(valid && !(logw != logw) ? logw : -INFINITY,
                              red);
  if (threadIdx.x == 0) {
    if (nz) {
      atomicOr(f.gnz + tl.group, 1);
    }
    atomicMax(f.gkey + tl.group, ordered_key(mx));
  }
}

template <typename T>
DUST2_PARTICLE_KERNEL(T) k_step_compare(system_view<T> v, filter_view f,
                                        double time,
                               double dt, int n_steps, double time_compare,
                               const typename T::data_type* data,
                               int n_groups_data) {
  __shared__ shared_smem<T> sm;
  __shared__ double red[33];
  const tile tl = v.tiles[blockIdx.x];
  if (!f.active[tl.group]) {
    return;
  }
  step_compare_tile<T>(v, f, tl, sm, red, time, dt, n_steps, time_compare,
                       data + (n_groups_data == 1 ? 0 : tl.group));
}

// k_step_compare as a persistent kernel: a grid sized to fill the device
// once, whose blocks take tiles in order from a device work queue (an
// atomic counter, zero before the launch) until none are left.  Tiles of
// groups of very different sizes then share one launch without a block
// per tile, and a block that finishes early takes the next tile at once.
template <typename T>
DUST2_PARTICLE_KERNEL(T) k_step_compare_queue(
    system_view<T> v, filter_view f, double time, double dt, int n_steps,
    double time_compare, const typename T::data_type* data,
    int n_groups_data, int n_tiles, int* next_tile) {
  __shared__ shared_smem<T> sm;
  __shared__ double red[33];
  __shared__ int taken;
  for (;;) {
    if (threadIdx.x == 0) {
      taken = atomicAdd(next_tile, 1);
    }
    __syncthreads();
    const int t = taken;
    __syncthreads();  // every thread has read `taken` before it changes
    if (t >= n_tiles) {
      return;
    }
    const tile tl = v.tiles[t];
    if (!f.active[tl.group]) {
      continue;
    }
    step_compare_tile<T>(v, f, tl, sm, red, time, dt, n_steps,
                         time_compare,
                         data + (n_groups_data == 1 ? 0 : tl.group));
  }
}

// Exclusive offsets of a group's chunks (warp scans of 32 chunk totals
// and a running carry; the exclusive value comes from the neighbour
// lane, so every offset is a plain sum); returns the group total.
// Afterwards chunk_sum holds each chunk's end, offset + total (the value
// the resampling search compares with, computed once here).
__device__ __forceinline__ double group_chunk_offsets(const filter_view& f,
                                                      int g, int lane) {
  const int c0 = f.chunk_first[g];
  const int nc = f.chunk_count[g];
  double carry = 0;
  for (int base = 0; base < nc; base += 32) {
    const int c = base + lane;
    const double v = c < nc ? f.chunk_sum[c0 + c] : 0.0;
    const double incl = warp_inclusive_scan(v);
    double excl = __shfl_up_sync(0xffffffffu, incl, 1);
    if (lane == 0) {
      excl = 0;
    }
    if (c < nc) {
      const double off = carry + excl;
      f.chunk_off[c0 + c] = off;
      f.chunk_sum[c0 + c] = off + v;
    }
    carry = carry + __shfl_sync(0xffffffffu, incl, 31);
  }
  return carry;
}

__global__ void k_weights(filter_view f);
__global__ void k_group(filter_view f, int n_groups);
__global__ void k_resample(filter_view f);
// Block size of k_fallback_count (any multiple of 32 up to 1024 works).
constexpr int FALLBACK_THREADS = 1024;
// The one-launch tail: a cluster of TAIL_CLUSTER blocks of TAIL_BLOCK
// threads per group, for groups of at most TAIL_MAX_PARTICLES.
constexpr int TAIL_CLUSTER = 8;
constexpr int TAIL_BLOCK = 128;
constexpr int TAIL_MAX_PARTICLES = TAIL_CLUSTER * TAIL_BLOCK;
__global__ void k_tail_cluster(filter_view f, int* count, const double* src,
                               double* dst, int stride, int n_state);
__global__ void k_save_history(const double* state, int stride,
                               const int* index_state, int n_save,
                               const tile* tiles, const int* active,
                               const int* mode, const int* idx,
                               double* hist_state, int* hist_order);
__global__ void k_export_snapshots(const double* snap_state,
                                   const int* hist_order, int n_times,
                                   const int* snap_obs, int n_snap,
                                   int n_state, int stride,
                                   const int* group_offset, const int* groups,
                                   int n_groups_out, const int* select,
                                   int n_particles_out, double* out);
__global__ void k_export_history(const double* hist_state,
                                 const int* hist_order, int n_times,
                                 int n_save, int stride,
                                 const int* group_offset, const int* groups,
                                 int n_groups_out, const int* select,
                                 int n_particles_out, double* out);

// Host-side description of the observation schedule.
struct obs_step {
  double t0;            // system time before the step
  int n_steps;
  double t_compare;     // system time after the step
};

template <typename T>
class filter_engine : public filter_api {
public:
  using data_type = typename T::data_type;
  // Discrete-time systems, or mixed-time ones (an ODE with updates; the
  // filter of r/continuous/filter.hpp over dust_continuous).
  using system_type = std::conditional_t<is_continuous<T>(),
                                         continuous_system<T>,
                                         discrete_system<T>>;

  // data: [n_times][n_groups_data] data_type; rng_words: the full stream
  // block of the filter, per group [2 filter | n_g particle] streams.
  filter_engine(std::unique_ptr<system_type> sys, double time_start,
                std::vector<double> times, std::vector<data_type> data,
                int n_groups_data, const std::vector<std::uint64_t>& rng_words) :
    owner_(std::move(sys)), sys_(&base_of(*owner_)), time_start_(time_start),
    times_(std::move(times)), n_groups_data_(n_groups_data) {
    const auto& L = sys_->layout();
    const int G = L.n_groups;
    const int N = L.n_total;
    const int NT = L.n_tiles();
    // schedule: discrete systems step to the data times
    // (discrete/system.hpp:62); continuous ones run to them exactly
    double t = time_start_;
    for (double ti : times_) {
      if constexpr (is_continuous<T>()) {
        schedule_.push_back(obs_step{t, 0, ti});
        t = ti;
      } else {
        const int n = static_cast<int>(
          std::round(std::max(0.0, ti - t) / sys_->dt()));
        schedule_.push_back(obs_step{t, n, t + n * sys_->dt()});
        t = t + n * sys_->dt();
      }
    }
    active_.resize(G);
    n_part_.resize(G);
    offset_.resize(G);
    chunk_first_.resize(G);
    chunk_count_.resize(G);
    w_.resize(N);
    ew_.resize(N);
    pre_.resize(N);
    chunk_sum_.resize(L.n_chunks);
    chunk_off_.resize(L.n_chunks);
    gkey_.resize(G);
    gnz_.resize(G);
    gflag_.resize(G);
    mode_.resize(G);
    ll_.resize(G);
    gu_.resize(G);
    guu0_.resize(G);
    gdu_.resize(G);
    gtot_.resize(G);
    idx_.resize(N);
    frng_.resize(8 * static_cast<std::size_t>(G));
    set_initial_.resize(1);
    fallback_count_.resize(G);
    force_serial_.resize(1);
    DUST2_CUDA(cudaMemsetAsync(force_serial_.data(), 0, sizeof(int),
                               sys_->stream()));
    data_.resize(data.size());
    auto s = sys_->stream();
    DUST2_CUDA(cudaMemcpyAsync(n_part_.data(), L.n_particles.data(),
                               G * sizeof(int), cudaMemcpyHostToDevice, s));
    DUST2_CUDA(cudaMemcpyAsync(offset_.data(), L.offset.data(),
                               G * sizeof(int), cudaMemcpyHostToDevice, s));
    DUST2_CUDA(cudaMemcpyAsync(chunk_first_.data(), L.chunk_first.data(),
                               G * sizeof(int), cudaMemcpyHostToDevice, s));
    DUST2_CUDA(cudaMemcpyAsync(chunk_count_.data(), L.chunk_count.data(),
                               G * sizeof(int), cudaMemcpyHostToDevice, s));
    DUST2_CUDA(cudaMemcpyAsync(data_.data(), data.data(),
                               data.size() * sizeof(data_type),
                               cudaMemcpyHostToDevice, s));
    put_rng_state(rng_words.data());
    sys_->sync();
    set_fused_tail(true);
    if constexpr (!is_continuous<T>()) {
      queue_.resize(std::max<std::size_t>(1, schedule_.size()));
      set_shape(default_shape());
    }
    // k_group: one warp per window of 32 chunks of the largest group
    int n_win = 1;
    for (int c : L.chunk_count) {
      n_win = std::max(n_win, (c + 31) / 32);
    }
    group_threads_ = 32 * std::min(n_win, 32);
  }

  system_api& sys() override {
    return *owner_;
  }
  discrete_system<T>& system() {
    return *sys_;
  }
  int n_times() const override {
    return static_cast<int>(times_.size());
  }
  bool has_run() const override {
    return has_run_;
  }
  long n_serial_fallbacks() const override {
    return n_fallbacks_;
  }
  void set_use_graph(bool use) override {
    use_graph_ = use;
  }

  void set_fused_tail(bool fused) override {
    if (pending_) {
      finish(nullptr);
    }
    int n_max = 0;
    for (int n : sys_->layout().n_particles) {
      n_max = std::max(n_max, n);
    }
    fused_tail_ = fused && n_max <= TAIL_MAX_PARTICLES;
    graph_state_ptr_ = nullptr;  // force a re-capture
  }

  void set_serial_resample(bool serial) override {
    if (pending_) {
      finish(nullptr);
    }
    const int v = serial ? 1 : 0;
    DUST2_CUDA(cudaMemcpy(force_serial_.data(), &v, sizeof(int),
                          cudaMemcpyHostToDevice));
  }

  filter_view view() {
    const auto& L = sys_->layout();
    (void)L;
    return filter_view{sys_->tiles_dev(), active_.data(), n_part_.data(),
                       offset_.data(), chunk_first_.data(),
                       chunk_count_.data(), w_.data(), ew_.data(), pre_.data(),
                       chunk_sum_.data(), chunk_off_.data(), gkey_.data(),
                       gnz_.data(), gflag_.data(), mode_.data(), ll_.data(),
                       gu_.data(), guu0_.data(), gdu_.data(), gtot_.data(),
                       idx_.data(), frng_.data(), set_initial_.data(),
                       force_serial_.data()};
  }

  void run(const double* initial, const int* index_group, int n_index_group,
           double* ll_out) override {
    launch(initial, index_group, n_index_group);
    std::vector<double> ll(sys_->layout().n_groups);
    finish(ll.data());
    if (index_group == nullptr) {
      std::copy(ll.begin(), ll.end(), ll_out);
    } else {
      for (int i = 0; i < n_index_group; ++i) {
        ll_out[i] = ll[index_group[i]];
      }
    }
  }

  void run_async(const int* index_group, int n_index_group) override {
    if (pending_) {
      finish(nullptr);
    }
    launch(nullptr, index_group, n_index_group);
  }

  void last_log_likelihood(double* ll_out) override {
    if (pending_) {
      finish(ll_out);
    } else {
      DUST2_CUDA(cudaMemcpy(ll_out, ll_.data(),
                            sys_->layout().n_groups * sizeof(double),
                            cudaMemcpyDeviceToHost));
    }
  }

  void* stream_handle() override {
    return static_cast<void*>(sys_->stream());
  }

  // Trajectory saving (filter.hpp:89-100, trajectories.hpp): after each
  // data time the post-reorder state (index_state entries, or all) and the
  // resampling indices go to device history buffers.
  void set_save_trajectories(bool save, const int* index_state,
                             int n_index_state) override {
    if (pending_) {
      finish(nullptr);
    }
    std::vector<int> is;
    if (save) {
      const int n_state = sys_->n_state();
      if (index_state == nullptr) {
        for (int i = 0; i < n_state; ++i) {
          is.push_back(i);
        }
      } else {
        is.assign(index_state, index_state + n_index_state);
      }
    }
    if (save != save_traj_ || is != traj_index_) {
      save_traj_ = save;
      traj_index_ = is;
      graph_state_ptr_ = nullptr;  // force a re-capture
      if (save) {
        const std::size_t stride = sys_->layout().stride;
        const std::size_t n_t = times_.size();
        hist_state_.resize(n_t * is.size() * stride);
        hist_order_.resize(n_t * stride);
        traj_index_dev_.resize(is.size());
        DUST2_CUDA(cudaMemcpy(traj_index_dev_.data(), is.data(),
                              is.size() * sizeof(int),
                              cudaMemcpyHostToDevice));
      }
    }
  }

  // Snapshots (filter.hpp:89-100, trajectories.hpp:84-97): the full
  // state after the reorder of the data times with these indices
  // (increasing).
  void set_save_snapshots(const int* obs, int n_obs) override {
    if (pending_) {
      finish(nullptr);
    }
    std::vector<int> v(obs, obs + n_obs);
    if (v != snap_obs_) {
      snap_obs_ = v;
      graph_state_ptr_ = nullptr;  // force a re-capture
      if (!v.empty()) {
        const std::size_t stride = sys_->layout().stride;
        const int n_state = sys_->n_state();
        snap_state_.resize(v.size() * n_state * stride);
        snap_obs_dev_.resize(v.size());
        DUST2_CUDA(cudaMemcpy(snap_obs_dev_.data(), v.data(),
                              v.size() * sizeof(int),
                              cudaMemcpyHostToDevice));
        std::vector<int> all(n_state);
        for (int i = 0; i < n_state; ++i) {
          all[i] = i;
        }
        all_state_dev_.resize(n_state);
        DUST2_CUDA(cudaMemcpy(all_state_dev_.data(), all.data(),
                              n_state * sizeof(int), cudaMemcpyHostToDevice));
      }
    }
    if (!v.empty()) {
      const std::size_t stride = sys_->layout().stride;
      if (hist_order_.size() < times_.size() * stride) {
        hist_order_.resize(times_.size() * stride);
      }
    }
  }

  bool snapshots_current() const override {
    return snap_current_;
  }

  int n_snapshots() const override {
    return static_cast<int>(snap_obs_.size());
  }

  // trajectories.hpp:199-268 (export_snapshots with reorder).
  // out: [snapshot][group][particle][state]
  void last_snapshots(const int* groups, int n_groups, const int* select,
                      double* out) override {
    if (pending_) {
      finish(nullptr);
    }
    if (!snap_current_) {
      throw std::runtime_error("Snapshots are not current");
    }
    const auto& L = sys_->layout();
    const int n_particles = L.n_particles[groups[0]];
    const int n_out = select != nullptr ? 1 : n_particles;
    const int n_state = sys_->n_state();
    const int n_snap = n_snapshots();
    const std::size_t len =
      static_cast<std::size_t>(n_snap) * n_groups * n_out * n_state;
    device_array<double> buf(len);
    device_array<int> g_dev(n_groups);
    device_array<int> sel_dev(select != nullptr ? n_groups : 1);
    auto s = sys_->stream();
    DUST2_CUDA(cudaMemcpyAsync(g_dev.data(), groups, n_groups * sizeof(int),
                               cudaMemcpyHostToDevice, s));
    if (select != nullptr) {
      DUST2_CUDA(cudaMemcpyAsync(sel_dev.data(), select,
                                 n_groups * sizeof(int),
                                 cudaMemcpyHostToDevice, s));
    }
    const long n_threads = static_cast<long>(n_groups) * n_out;
    k_export_snapshots<<<n_blocks(n_threads, 128), 128, 0, s>>>(
      snap_state_.data(), hist_order_.data(), n_times(), snap_obs_dev_.data(),
      n_snap, n_state, L.stride, offset_.data(), g_dev.data(), n_groups,
      select != nullptr ? sel_dev.data() : nullptr, n_out, buf.data());
    DUST2_CUDA(cudaGetLastError());
    DUST2_CUDA(cudaMemcpyAsync(out, buf.data(), len * sizeof(double),
                               cudaMemcpyDeviceToHost, s));
    DUST2_CUDA(cudaStreamSynchronize(s));
  }

  bool trajectories_current() const override {
    return traj_current_;
  }

  int n_trajectory_state() const override {
    return static_cast<int>(traj_index_.size());
  }

  // trajectories.hpp export_state with reorder = true: for each output
  // particle (all, or select[i] of group groups[i]) walk its ancestry
  // back from the last data time.  out: [time][group][particle][state].
  void last_trajectories(const int* groups, int n_groups,
                         const int* select, double* out) override {
    if (pending_) {
      finish(nullptr);
    }
    if (!traj_current_) {
      throw std::runtime_error("Trajectories are not current");
    }
    const auto& L = sys_->layout();
    const int n_particles = L.n_particles[groups[0]];
    const int n_out = select != nullptr ? 1 : n_particles;
    const int n_save = n_trajectory_state();
    const int n_t = n_times();
    const std::size_t len =
      static_cast<std::size_t>(n_t) * n_groups * n_out * n_save;
    device_array<double> buf(len);
    device_array<int> g_dev(n_groups);
    device_array<int> sel_dev(select != nullptr ? n_groups : 1);
    auto s = sys_->stream();
    DUST2_CUDA(cudaMemcpyAsync(g_dev.data(), groups, n_groups * sizeof(int),
                               cudaMemcpyHostToDevice, s));
    if (select != nullptr) {
      DUST2_CUDA(cudaMemcpyAsync(sel_dev.data(), select,
                                 n_groups * sizeof(int),
                                 cudaMemcpyHostToDevice, s));
    }
    const long n_threads = static_cast<long>(n_groups) * n_out;
    k_export_history<<<n_blocks(n_threads, 128), 128, 0, s>>>(
      hist_state_.data(), hist_order_.data(), n_t, n_save, L.stride,
      offset_.data(), g_dev.data(), n_groups,
      select != nullptr ? sel_dev.data() : nullptr, n_out, buf.data());
    DUST2_CUDA(cudaGetLastError());
    DUST2_CUDA(cudaMemcpyAsync(out, buf.data(), len * sizeof(double),
                               cudaMemcpyDeviceToHost, s));
    DUST2_CUDA(cudaStreamSynchronize(s));
  }

  void set_timing(bool enable) override {
    if (enable != timing_) {
      if (pending_) {
        finish(nullptr);
      }
      timing_ = enable;
      graph_state_ptr_ = nullptr;  // force a re-capture
      if (timing_) {
        ensure_events();  // no allocation may happen during capture
      }
    }
    step_ms_ = 0;
    run_ms_ = 0;
    reorder_ms_ = 0;
    n_step_launches_ = 0;
    n_reorder_launches_ = 0;
    n_timed_runs_ = 0;
  }

  void reorder_times(double* ms, long* n_launches) override {
    if (pending_) {
      finish(nullptr);
    }
    *ms = reorder_ms_;
    *n_launches = n_reorder_launches_;
  }

  void kernel_times(double* step_ms, long* n_step_launches, double* run_ms,
                    long* n_runs) override {
    if (pending_) {
      finish(nullptr);
    }
    *step_ms = step_ms_;
    *n_step_launches = n_step_launches_;
    *run_ms = run_ms_;
    *n_runs = n_timed_runs_;
  }

  // Enqueue one run: reset (filter.hpp:156-175) then the observation loop.
  void launch(const double* initial, const int* index_group,
              int n_index_group) {
    auto& S = *sys_;
    const auto& L = S.layout();
    const int G = L.n_groups;
    auto s = S.stream();
    if (pending_) {
      finish(nullptr);
    }
    if constexpr (!is_continuous<T>()) {
      if (autotune_ && !tuned_) {
        autotune();
      }
    }
    traj_current_ = false;
    snap_current_ = false;
    active_host_.assign(G, index_group == nullptr ? 1 : 0);
    if (index_group != nullptr) {
      for (int i = 0; i < n_index_group; ++i) {
        active_host_[index_group[i]] = 1;
      }
    }
    S.reset_errors();
    S.set_time(time_start_);
    if (initial != nullptr) {
      S.put_state(initial);
    }
    set_initial_host_ = initial == nullptr ? 1 : 0;
    DUST2_CUDA(cudaMemcpyAsync(active_.data(), active_host_.data(),
                               G * sizeof(int), cudaMemcpyHostToDevice, s));
    DUST2_CUDA(cudaMemcpyAsync(set_initial_.data(), &set_initial_host_,
                               sizeof(int), cudaMemcpyHostToDevice, s));
    if (use_graph_) {
      if (graph_exec_ == nullptr || graph_state_ptr_ != S.state_ptr()) {
        capture();
      }
      DUST2_CUDA(cudaGraphLaunch(graph_exec_, s));
    } else {
      enqueue();
    }
    pending_ = true;
  }

  // Wait for the last launched run; copy its log-likelihoods (all
  // groups) to ll_out when given; raise any particle errors.
  void finish(double* ll_out) {
    auto& S = *sys_;
    const int G = S.layout().n_groups;
    auto s = S.stream();
    pending_ = false;
    fallback_host_.resize(G);
    if (ll_out != nullptr) {
      DUST2_CUDA(cudaMemcpyAsync(ll_out, ll_.data(), G * sizeof(double),
                                 cudaMemcpyDeviceToHost, s));
    }
    DUST2_CUDA(cudaMemcpyAsync(fallback_host_.data(), fallback_count_.data(),
                               G * sizeof(int), cudaMemcpyDeviceToHost, s));
    S.check_errors_after();
    for (int g = 0; g < G; ++g) {
      n_fallbacks_ += fallback_host_[g];
    }
    if (timing_) {
      accumulate_timing();
    }
    S.set_time(schedule_.empty() ? time_start_ : schedule_.back().t_compare);
    random_particle_.assign(G, -1);
    has_run_ = true;
    traj_current_ = save_traj_;
    snap_current_ = !snap_obs_.empty();
  }

  void update_pars(const double* pars, const int* index_group,
                   int n_index_group) override {
    owner_->update_pars(pars, index_group, n_index_group);
  }

  std::size_t n_rng_streams() const override {
    const auto& L = sys_->layout();
    return static_cast<std::size_t>(L.n_total) + 2 * L.n_groups;
  }

  void get_rng_state(std::uint64_t* out) override {
    const auto& L = sys_->layout();
    const int G = L.n_groups;
    std::vector<std::uint64_t> f(8 * static_cast<std::size_t>(G));
    DUST2_CUDA(cudaMemcpy(f.data(), frng_.data(), f.size() * 8,
                          cudaMemcpyDeviceToHost));
    std::vector<std::uint64_t> p(4 * static_cast<std::size_t>(L.n_total));
    sys_->get_rng_state(p.data());
    std::size_t pos = 0;
    for (int g = 0; g < G; ++g) {
      for (int w = 0; w < 8; ++w) {
        out[pos++] = f[8 * g + w];
      }
      const std::size_t from = 4 * static_cast<std::size_t>(L.offset[g]);
      for (std::size_t w = 0; w < 4 * static_cast<std::size_t>(
             L.n_particles[g]); ++w) {
        out[pos++] = p[from + w];
      }
    }
  }

  void put_rng_state(const std::uint64_t* in) override {
    const auto& L = sys_->layout();
    const int G = L.n_groups;
    std::vector<std::uint64_t> f(8 * static_cast<std::size_t>(G));
    std::vector<std::uint64_t> p(4 * static_cast<std::size_t>(L.n_total));
    std::size_t pos = 0;
    for (int g = 0; g < G; ++g) {
      for (int w = 0; w < 8; ++w) {
        f[8 * g + w] = in[pos++];
      }
      const std::size_t to = 4 * static_cast<std::size_t>(L.offset[g]);
      for (std::size_t w = 0; w < 4 * static_cast<std::size_t>(
             L.n_particles[g]); ++w) {
        p[to + w] = in[pos++];
      }
    }
    DUST2_CUDA(cudaMemcpy(frng_.data(), f.data(), f.size() * 8,
                          cudaMemcpyHostToDevice));
    sys_->put_rng_state(p.data());
  }

  std::vector<int> select_random_particle() override {
    const auto& L = sys_->layout();
    const int G = L.n_groups;
    if (static_cast<int>(random_particle_.size()) != G) {
      random_particle_.assign(G, -1);
    }
    bool any = false;
    for (int g = 0; g < G; ++g) {
      any = any || random_particle_[g] < 0;
    }
    if (any) {
      std::vector<std::uint64_t> f(8 * static_cast<std::size_t>(G));
      DUST2_CUDA(cudaMemcpy(f.data(), frng_.data(), f.size() * 8,
                            cudaMemcpyDeviceToHost));
      for (int g = 0; g < G; ++g) {
        if (random_particle_[g] < 0) {
          random::rng_state r{};
          for (int w = 0; w < 4; ++w) {
            r.state[w] = f[8 * g + 4 + w];
          }
          const double u = random::random_real(r);
          random_particle_[g] =
            static_cast<int>(std::floor(u * L.n_particles[g]));
          for (int w = 0; w < 4; ++w) {
            f[8 * g + 4 + w] = r.state[w];
          }
        }
      }
      DUST2_CUDA(cudaMemcpy(frng_.data(), f.data(), f.size() * 8,
                            cudaMemcpyHostToDevice));
    }
    return random_particle_;
  }

  // The step kernel's launch shape before any tuning: one-warp tiles
  // that spread a small problem over the SM partitions (four per SM)
  // when its group tiles would fill fewer warps than there are
  // partitions, else the group tiles.
  step_shape default_shape() const {
    const auto& L = sys_->layout();
    const int parts = 4 * n_sms();
    long warps = 0;
    for (int n : L.n_particles) {
      warps += (n + 31) / 32;
    }
    if (warps < parts) {
      const int per = static_cast<int>((static_cast<long>(L.n_total) +
                                        parts - 1) / parts);
      if (per < 32) {
        return step_shape{32, std::max(1, per), false};
      }
    }
    return step_shape{L.tile_size, 0, false};
  }

  // Blocks of a persistent step launch: as many as fit on the device at
  // once (at most one per tile).
  int persistent_grid(int block, int n_tiles) const {
    int per_sm = 0;
    DUST2_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(
      &per_sm, k_step_compare_queue<T>, block, 0));
    return std::max(1, std::min(n_tiles, std::max(1, per_sm) * n_sms()));
  }

  // One step+compare launch of observation i in the current shape, on
  // the given state and generators (the filter's, or the autotuner's
  // scratch copies); `next_tile` is the zeroed work-queue counter of a
  // persistent launch.
  void launch_step(cudaStream_t s, const filter_view& f, double* state,
                   std::uint64_t* rng, const obs_step& st, std::size_t i,
                   int* next_tile) {
    auto& S = *sys_;
    system_view<T> v = S.view();
    v.state = state;
    v.rng = rng;
    v.tiles = step_tiles_.data();
    launch_step_shape(s, f, v, shape_, n_step_tiles_, step_grid_, st, i,
                      next_tile);
  }

  // `grid`: the blocks of a persistent launch (persistent_grid, found
  // before any graph capture).
  void launch_step_shape(cudaStream_t s, const filter_view& f,
                         const system_view<T>& v, const step_shape& sh,
                         int n_tiles, int grid, const obs_step& st,
                         std::size_t i, int* next_tile) {
    auto& S = *sys_;
    const auto* d = data_.data() + i * n_groups_data_;
    if (sh.persistent) {
      k_step_compare_queue<T><<<grid, sh.block, 0, s>>>(
        v, f, st.t0, S.dt(), st.n_steps, st.t_compare, d, n_groups_data_,
        n_tiles, next_tile);
    } else {
      k_step_compare<T><<<n_tiles, sh.block, 0, s>>>(
        v, f, st.t0, S.dt(), st.n_steps, st.t_compare, d, n_groups_data_);
    }
  }

  static int n_sms() {
    int dev = 0, sms = 0;
    DUST2_CUDA(cudaGetDevice(&dev));
    DUST2_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount,
                                      dev));
    return sms;
  }

  void set_shape(step_shape sh) {
    const auto& L = sys_->layout();
    if (sh.per_tile < 0 || sh.per_tile > 32 || sh.block < 32 ||
        sh.block % 32 != 0 || sh.block > default_tile_size<T>() ||
        (sh.per_tile > 0 && sh.block != 32)) {
      throw std::runtime_error("invalid step kernel shape");
    }
    const std::vector<tile> t = sh.per_tile > 0 ?
      warp_tiles(L, sh.per_tile) : group_layout(L.n_particles, sh.block).tiles;
    step_tiles_.resize(t.size());
    DUST2_CUDA(cudaMemcpyAsync(step_tiles_.data(), t.data(),
                               t.size() * sizeof(tile),
                               cudaMemcpyHostToDevice, sys_->stream()));
    n_step_tiles_ = static_cast<int>(t.size());
    step_grid_ = sh.persistent ? persistent_grid(sh.block, n_step_tiles_) :
      n_step_tiles_;
    shape_ = sh;
    graph_state_ptr_ = nullptr;  // force a re-capture
    DUST2_CUDA(cudaStreamSynchronize(sys_->stream()));
  }

  // Candidate shapes: group tiles of every block size up to the
  // system's, and for problems that fill fewer warps than the device has
  // SM partitions also one-warp tiles of 1 to 16 particles.
  std::vector<step_shape> candidates() const {
    const auto& L = sys_->layout();
    std::vector<step_shape> c;
    for (int b = 32; b <= default_tile_size<T>(); b *= 2) {
      c.push_back(step_shape{b, 0, false});
      c.push_back(step_shape{b, 0, true});
    }
    const long parts = 4L * n_sms();
    long warps = 0;
    for (int n : L.n_particles) {
      warps += (n + 31) / 32;
    }
    if (warps < parts) {
      for (int per = 1; per <= 16; per *= 2) {
        if (static_cast<long>(warp_tiles(L, per).size()) <= 4 * parts) {
          c.push_back(step_shape{32, per, false});
        }
      }
    }
    return c;
  }

  // Pick the fastest candidate shape by timing the step kernel on
  // scratch copies of the particles: initial conditions, advanced part
  // of the way into the schedule (the cost of a step depends on the
  // state), then one observation's steps per candidate, three times,
  // keeping each candidate's fastest.  The filter's own state,
  // generators and error records are not touched; its weights and group
  // reductions are reset by the run that follows.  Skipped when the
  // scratch copies would take more than a quarter of the free memory.
  void autotune() {
    tuned_ = true;
    auto& S = *sys_;
    const auto& L = S.layout();
    const auto cand = candidates();
    n_candidates_ = static_cast<int>(cand.size());
    if (cand.size() < 2 || schedule_.empty()) {
      return;
    }
    const std::size_t n_st = static_cast<std::size_t>(S.n_state()) *
      L.stride;
    const std::size_t bytes = 2 * n_st * sizeof(double) +
      8 * static_cast<std::size_t>(L.stride) * sizeof(std::uint64_t) +
      L.n_total * sizeof(particle_error);
    std::size_t free_b = 0, total_b = 0;
    DUST2_CUDA(cudaMemGetInfo(&free_b, &total_b));
    if (bytes > free_b / 4) {
      return;
    }
    auto s = S.stream();
    device_array<double> base(n_st), work(n_st);
    device_array<std::uint64_t> rng_base(4 * L.stride), rng_work(4 * L.stride);
    device_array<particle_error> err(L.n_total);
    device_array<int> any(1);
    system_view<T> v = S.run_view();
    DUST2_CUDA(cudaMemcpyAsync(base.data(), v.state, n_st * sizeof(double),
                               cudaMemcpyDeviceToDevice, s));
    DUST2_CUDA(cudaMemcpyAsync(rng_base.data(), v.rng,
                               4 * L.stride * sizeof(std::uint64_t),
                               cudaMemcpyDeviceToDevice, s));
    v.state = base.data();
    v.rng = rng_base.data();
    v.errors = err.data();
    v.any_error = any.data();
    const int run_tiles = S.n_run_tiles();
    k_initial<T><<<run_tiles, L.tile_size, 0, s>>>(v, nullptr, time_start_);
    // part of the way in: half the schedule's steps, at most 400 (the
    // cost of a step depends on the state, and early states are cheap)
    const std::size_t mid = schedule_.size() / 2;
    int steps = 0;
    for (std::size_t i = 0; i < mid; ++i) {
      steps += schedule_[i].n_steps;
    }
    steps = std::min(steps, 400);
    if (steps > 0) {
      k_run<T><<<run_tiles, L.tile_size, 0, s>>>(v, time_start_, S.dt(),
                                                 steps);
    }
    DUST2_CUDA(cudaGetLastError());
    const double t0 = time_start_ + steps * S.dt();
    const int n_steps = std::max(1, schedule_[mid].n_steps);
    const obs_step trial{t0, n_steps, t0 + n_steps * S.dt()};
    device_array<int> counter(1);
    filter_view f = view();
    active_host_.assign(L.n_groups, 1);
    DUST2_CUDA(cudaMemcpyAsync(active_.data(), active_host_.data(),
                               L.n_groups * sizeof(int),
                               cudaMemcpyHostToDevice, s));
    std::vector<device_array<tile>> tiles(cand.size());
    std::vector<int> n_tiles(cand.size());
    std::vector<int> grids(cand.size());
    for (std::size_t c = 0; c < cand.size(); ++c) {
      const std::vector<tile> t = cand[c].per_tile > 0 ?
        warp_tiles(L, cand[c].per_tile) :
        group_layout(L.n_particles, cand[c].block).tiles;
      tiles[c].resize(t.size());
      DUST2_CUDA(cudaMemcpyAsync(tiles[c].data(), t.data(),
                                 t.size() * sizeof(tile),
                                 cudaMemcpyHostToDevice, s));
      n_tiles[c] = static_cast<int>(t.size());
      grids[c] = cand[c].persistent ?
        persistent_grid(cand[c].block, n_tiles[c]) : n_tiles[c];
    }
    constexpr int REPS = 3;
    std::vector<cudaEvent_t> ev(2 * REPS * cand.size());
    for (auto& e : ev) {
      DUST2_CUDA(cudaEventCreate(&e));
    }
    system_view<T> w = S.view();
    w.state = work.data();
    w.rng = rng_work.data();
    w.errors = err.data();
    w.any_error = any.data();
    for (int r = 0; r < REPS; ++r) {
      for (std::size_t c = 0; c < cand.size(); ++c) {
        DUST2_CUDA(cudaMemcpyAsync(work.data(), base.data(),
                                   n_st * sizeof(double),
                                   cudaMemcpyDeviceToDevice, s));
        DUST2_CUDA(cudaMemcpyAsync(rng_work.data(), rng_base.data(),
                                   4 * L.stride * sizeof(std::uint64_t),
                                   cudaMemcpyDeviceToDevice, s));
        DUST2_CUDA(cudaMemsetAsync(counter.data(), 0, sizeof(int), s));
        w.tiles = tiles[c].data();
        const std::size_t e = 2 * (r * cand.size() + c);
        DUST2_CUDA(cudaEventRecord(ev[e], s));
        launch_step_shape(s, f, w, cand[c], n_tiles[c], grids[c], trial,
                          mid, counter.data());
        DUST2_CUDA(cudaEventRecord(ev[e + 1], s));
      }
    }
    DUST2_CUDA(cudaGetLastError());
    DUST2_CUDA(cudaStreamSynchronize(s));
    std::vector<double> best(cand.size(), 1e300);
    for (int r = 0; r < REPS; ++r) {
      for (std::size_t c = 0; c < cand.size(); ++c) {
        const std::size_t e = 2 * (r * cand.size() + c);
        float ms = 0;
        DUST2_CUDA(cudaEventElapsedTime(&ms, ev[e], ev[e + 1]));
        best[c] = std::min(best[c], static_cast<double>(ms));
      }
    }
    for (auto e : ev) {
      cudaEventDestroy(e);
    }
    const std::size_t pick = static_cast<std::size_t>(
      std::min_element(best.begin(), best.end()) - best.begin());
    best_ms_ = best[pick];
    set_shape(cand[pick]);
  }

  void set_autotune(bool enable) override {
    if (pending_) {
      finish(nullptr);
    }
    autotune_ = enable;
  }

  void set_step_shape(int block, int per_tile, bool persistent) override {
    if (pending_) {
      finish(nullptr);
    }
    if constexpr (is_continuous<T>()) {
      throw std::runtime_error("the step shape applies to discrete-time "
                               "filters");
    } else {
      set_shape(step_shape{block, per_tile, persistent});
      autotune_ = false;
      tuned_ = true;
    }
  }

  void step_shape_info(int* block, int* per_tile, int* persistent,
                       int* n_candidates, double* best_ms) override {
    *block = shape_.block;
    *per_tile = shape_.per_tile;
    *persistent = shape_.persistent ? 1 : 0;
    *n_candidates = n_candidates_;
    *best_ms = best_ms_;
  }

  ~filter_engine() override {
    cudaStreamSynchronize(sys_->stream());
    for (auto e : ev_step_) {
      cudaEventDestroy(e);
    }
    for (auto e : ev_run_) {
      cudaEventDestroy(e);
    }
    for (auto e : ev_reorder_) {
      cudaEventDestroy(e);
    }
    if (graph_exec_ != nullptr) {
      cudaGraphExecDestroy(graph_exec_);
    }
    if (graph_ != nullptr) {
      cudaGraphDestroy(graph_);
    }
  }

private:
  // The launch sequence of one run; captured into a graph or issued
  // directly.
  void enqueue() {
    auto& S = *sys_;
    const auto& L = S.layout();
    auto s = S.stream();
    const int G = L.n_groups;
    const int NT = L.n_tiles();
    const int TS = L.tile_size;
    filter_view f = view();
    f.gflag = gflag_.data();
    if (timing_) {
      ensure_events();
      record(ev_run_[0]);
    }
    k_filter_reset<<<n_blocks(G, 128), 128, 0, s>>>(f, G);
    if constexpr (!is_continuous<T>()) {
      if (shape_.persistent) {
        // one work-queue counter per data time, all zero before the run
        DUST2_CUDA(cudaMemsetAsync(queue_.data(), 0,
                                   schedule_.size() * sizeof(int), s));
      }
    }
    DUST2_CUDA(cudaMemsetAsync(fallback_count_.data(), 0, G * sizeof(int), s));
    system_view<T> v = S.view();
    k_initial_flagged<T><<<NT, TS, 0, s>>>(v, set_initial_.data(),
                                           time_start_);
    double* cur = S.state_ptr();
    double* other = S.state_other_ptr();
    for (std::size_t i = 0; i < schedule_.size(); ++i) {
      const auto& st = schedule_[i];
      v.state = cur;
      if (timing_) {
        record(ev_step_[2 * i]);
      }
      if constexpr (is_continuous<T>()) {
        k_step_compare_mixed<T><<<NT, TS, 0, s>>>(
          v, owner_->view_ode(), owner_->control_dev(), f, st.t0,
          st.t_compare, owner_->dt(), i == 0 ? 1 : 0,
          data_.data() + i * n_groups_data_, n_groups_data_);
      } else {
        launch_step(s, f, v.state, v.rng, st, i, queue_.data() + i);
      }
      if (timing_) {
        record(ev_step_[2 * i + 1]);
      }
      if (fused_tail_) {
        k_tail_cluster<<<G * TAIL_CLUSTER, TAIL_BLOCK, 0, s>>>(
          f, fallback_count_.data(), cur, other, L.stride, S.n_state());
      } else {
        k_weights<<<NT, TS, 0, s>>>(f);
        k_group<<<G, group_threads_, 0, s>>>(f, G);
        k_resample<<<NT, TS, 0, s>>>(f);
        k_fallback_counted(f, s);
        if (timing_) {
          record(ev_reorder_[2 * i]);
        }
        k_reorder<<<NT, TS, 0, s>>>(cur, other, L.stride, S.n_state(),
                                    L.tiles.empty() ? nullptr :
                                    S.tiles_dev(), offset_.data(),
                                    idx_.data(), mode_.data());
        if (timing_) {
          record(ev_reorder_[2 * i + 1]);
        }
      }
      if constexpr (is_continuous<T>()) {
        owner_->enqueue_reorder_record(S.tiles_dev(), NT, TS, offset_.data(),
                                       idx_.data(), mode_.data(), s);
      }
      std::swap(cur, other);
      const std::size_t stride = L.stride;
      if (save_traj_ || !snap_obs_.empty()) {
        k_save_history<<<NT, TS, 0, s>>>(
          cur, L.stride, traj_index_dev_.data(),
          save_traj_ ? n_trajectory_state() : 0, S.tiles_dev(),
          active_.data(), mode_.data(), idx_.data(),
          save_traj_ ? hist_state_.data() + i * traj_index_.size() * stride :
          nullptr, hist_order_.data() + i * stride);
      }
      for (std::size_t sn = 0; sn < snap_obs_.size(); ++sn) {
        if (snap_obs_[sn] == static_cast<int>(i)) {
          k_save_history<<<NT, TS, 0, s>>>(
            cur, L.stride, all_state_dev_.data(), S.n_state(),
            S.tiles_dev(), active_.data(), mode_.data(), idx_.data(),
            snap_state_.data() + sn * S.n_state() * stride, nullptr);
        }
      }
    }
    if (cur != S.state_ptr()) {
      DUST2_CUDA(cudaMemcpyAsync(S.state_ptr(), cur,
                                 static_cast<std::size_t>(S.n_state()) *
                                 L.stride * sizeof(double),
                                 cudaMemcpyDeviceToDevice, s));
    }
    if (timing_) {
      record(ev_run_[1]);
    }
    DUST2_CUDA(cudaGetLastError());
  }

  void ensure_events() {
    const std::size_t need = 2 * schedule_.size();
    while (ev_step_.size() < need) {
      cudaEvent_t e;
      DUST2_CUDA(cudaEventCreate(&e));
      ev_step_.push_back(e);
    }
    while (ev_reorder_.size() < need) {
      cudaEvent_t e;
      DUST2_CUDA(cudaEventCreate(&e));
      ev_reorder_.push_back(e);
    }
    while (ev_run_.size() < 2) {
      cudaEvent_t e;
      DUST2_CUDA(cudaEventCreate(&e));
      ev_run_.push_back(e);
    }
  }

  void record(cudaEvent_t e) {
    DUST2_CUDA(cudaEventRecordWithFlags(
      e, sys_->stream(), capturing_ ? cudaEventRecordExternal :
      cudaEventRecordDefault));
  }

  void accumulate_timing() {
    for (std::size_t i = 0; i < schedule_.size(); ++i) {
      float ms = 0;
      DUST2_CUDA(cudaEventElapsedTime(&ms, ev_step_[2 * i],
                                      ev_step_[2 * i + 1]));
      step_ms_ += ms;
      n_step_launches_++;
      if (!fused_tail_) {
        DUST2_CUDA(cudaEventElapsedTime(&ms, ev_reorder_[2 * i],
                                        ev_reorder_[2 * i + 1]));
        reorder_ms_ += ms;
        n_reorder_launches_++;
      }
    }
    float ms = 0;
    DUST2_CUDA(cudaEventElapsedTime(&ms, ev_run_[0], ev_run_[1]));
    run_ms_ += ms;
    n_timed_runs_++;
  }

  void k_fallback_counted(filter_view f, cudaStream_t s);

  void capture() {
    auto s = sys_->stream();
    if (graph_exec_ != nullptr) {
      cudaGraphExecDestroy(graph_exec_);
      graph_exec_ = nullptr;
    }
    if (graph_ != nullptr) {
      cudaGraphDestroy(graph_);
      graph_ = nullptr;
    }
    DUST2_CUDA(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
    capturing_ = true;
    try {
      enqueue();
    } catch (...) {
      capturing_ = false;
      cudaGraph_t g = nullptr;
      cudaStreamEndCapture(s, &g);
      if (g != nullptr) {
        cudaGraphDestroy(g);
      }
      throw;
    }
    capturing_ = false;
    DUST2_CUDA(cudaStreamEndCapture(s, &graph_));
    DUST2_CUDA(cudaGraphInstantiate(&graph_exec_, graph_, 0));
    graph_state_ptr_ = sys_->state_ptr();
  }

  static discrete_system<T>& base_of(discrete_system<T>& s) {
    return s;
  }
  static discrete_system<T>& base_of(continuous_system<T>& s) {
    return s.base();
  }

  std::unique_ptr<system_type> owner_;
  discrete_system<T>* sys_;
  double time_start_;
  std::vector<double> times_;
  int n_groups_data_;
  std::vector<obs_step> schedule_;
  std::vector<int> random_particle_;
  bool has_run_ = false;
  bool use_graph_ = true;
  bool fused_tail_ = false;  // k_tail_cluster instead of separate kernels
  int group_threads_ = 32;   // block size of k_group
  bool pending_ = false;
  bool capturing_ = false;
  bool timing_ = false;
  bool save_traj_ = false;
  bool traj_current_ = false;
  std::vector<int> traj_index_;
  device_array<int> traj_index_dev_;
  device_array<double> hist_state_;
  device_array<int> hist_order_;
  std::vector<int> snap_obs_;
  bool snap_current_ = false;
  device_array<int> snap_obs_dev_;
  device_array<int> all_state_dev_;
  device_array<double> snap_state_;
  long n_fallbacks_ = 0;
  std::vector<int> active_host_;
  int set_initial_host_ = 1;
  std::vector<int> fallback_host_;
  std::vector<cudaEvent_t> ev_step_;
  std::vector<cudaEvent_t> ev_run_;
  std::vector<cudaEvent_t> ev_reorder_;
  double step_ms_ = 0;
  double run_ms_ = 0;
  double reorder_ms_ = 0;
  long n_step_launches_ = 0;
  long n_reorder_launches_ = 0;
  long n_timed_runs_ = 0;

  device_array<int> active_, n_part_, offset_, chunk_first_, chunk_count_;
  device_array<double> w_, ew_, pre_, chunk_sum_, chunk_off_;
  device_array<unsigned long long> gkey_;
  device_array<int> gnz_, gflag_, mode_;
  device_array<double> ll_, gu_, guu0_, gdu_, gtot_;
  device_array<int> idx_;
  device_array<std::uint64_t> frng_;
  device_array<int> set_initial_;
  device_array<int> fallback_count_;
  device_array<int> force_serial_;
  device_array<data_type> data_;

  // launch shape of the step kernel (discrete-time systems)
  step_shape shape_{};
  int step_grid_ = 0;
  device_array<tile> step_tiles_;
  device_array<int> queue_;  // [n_times] work-queue counters
  int n_step_tiles_ = 0;
  bool autotune_ = true;
  bool tuned_ = false;
  int n_candidates_ = 0;
  double best_ms_ = 0;

  cudaGraph_t graph_ = nullptr;
  cudaGraphExec_t graph_exec_ = nullptr;
  const double* graph_state_ptr_ = nullptr;
};

// Serial fallback, counting how many groups needed it.
__global__ void k_fallback_count(filter_view f, int* count);

template <typename T>
void filter_engine<T>::k_fallback_counted(filter_view f, cudaStream_t s) {
  const int G = sys_->layout().n_groups;
  k_fallback_count<<<G, FALLBACK_THREADS, 0, s>>>(f, fallback_count_.data());
}

}  // namespace engine
}  // namespace dust2gpu
