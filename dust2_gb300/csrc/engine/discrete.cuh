// Discrete-time system engine on the GPU: the counterpart of
// dust2::dust_discrete<T> (inst/include/dust2/discrete/system.hpp:21-485).
//
// One thread advances one particle.  A particle's state and generator are
// loaded from structure-of-arrays device memory into registers, stepped
// `n_steps` times with the system's `update` (ping-pong between two
// register arrays, exactly as the reference swaps `state` and
// `state_next` pointers, :404-423), and written back once.  The group's
// `shared_state` and `zero_every` table are staged in shared memory.
//
// Semantics kept from the reference:
//   n_steps = round(max(0, t - time) / dt)                        (:62)
//   step i starts at time + i * dt; zero_every entries whose period
//   divides that time are reset first                         (:412-418)
//   time advances by n_steps * dt                                  (:91)
//   per-particle errors are collected and reported together, and leave
//   the system in an "errors pending" state                  (:82-87)
#pragma once

#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <memory>
#include <string>
#include <vector>

#include "../dust2gpu/system.hpp"
#include "api.hpp"
#include "device.cuh"
#include "kernels_common.cuh"
#include "layout.hpp"

namespace dust2gpu {
namespace engine {

// Everything a per-particle kernel needs to reach a system's device data.
template <typename T>
struct system_view {
  double* state;                 // [n_state][stride]
  std::uint64_t* rng;            // [4][stride]
  const typename T::shared_state* shared;  // [n_groups]
  const zero_every_spec* zero_every;       // [n_groups]
  const tile* tiles;
  particle_error* errors;        // [n_total]
  int* any_error;
  int stride;
  int n_state;
  bool deterministic;
  const int* particle_group;     // [n_total], for packed tiles
};

// Group of particle k of tile tl (a packed tile's particles may belong to
// different groups).
template <typename T>
__device__ __forceinline__ int group_of(const system_view<T>& v,
                                        const tile& tl, int k) {
  return tl.group >= 0 ? tl.group : v.particle_group[k];
}

// Steps of one launch whose zero_every test is precomputed per block.
constexpr int ZERO_STEPS_CACHED = 64;

template <typename T>
struct shared_smem {
  alignas(16) unsigned char shared_buf[sizeof(typename T::shared_state)];
  zero_every_spec zero;
  // bit i of zero_steps[e]: fmod(time + i * dt, period[e]) == 0
  std::uint64_t zero_steps[ZERO_EVERY_MAX];

  __device__ const typename T::shared_state& shared() const {
    return *reinterpret_cast<const typename T::shared_state*>(shared_buf);
  }
  __device__ void load(const system_view<T>& v, int group) {
    block_load(reinterpret_cast<typename T::shared_state*>(shared_buf),
               v.shared + group);
    block_load(&zero, v.zero_every + group);
  }
  // Evaluate the zero_every test of the first ZERO_STEPS_CACHED steps
  // once per block instead of once per particle and step (warp 0, one
  // step per lane; the expression is the one run_particle would use).
  // Called by every thread, before the barrier that follows load(); tiles
  // are whole warps (a multiple of 32 threads), so warp 0 is complete.
  __device__ void load_zero_steps(const system_view<T>& v, int group,
                                  double time, double dt, int n_steps) {
    if (threadIdx.x >= 32) {
      return;
    }
    const zero_every_spec& z = v.zero_every[group];
    const int lane = threadIdx.x;
    for (int e = 0; e < z.n; ++e) {
      std::uint64_t mask = 0;
      for (int base = 0; base < ZERO_STEPS_CACHED && base < n_steps;
           base += 32) {
        const int i = base + lane;
        const double t = time + static_cast<double>(i) * dt;
        const bool hit = i < n_steps && fmod(t, z.period[e]) == 0;
        mask |= static_cast<std::uint64_t>(__ballot_sync(0xffffffffu, hit))
          << base;
      }
      if (lane == 0) {
        zero_steps[e] = mask;
      }
    }
  }
};

template <typename T>
__device__ __forceinline__ void load_state(const system_view<T>& v, int k,
                                           double* x) {
#pragma unroll
  for (int s = 0; s < T::n_state_max; ++s) {
    if (s < v.n_state) {
      x[s] = v.state[static_cast<long>(s) * v.stride + k];
    }
  }
}

template <typename T>
__device__ __forceinline__ void store_state(const system_view<T>& v, int k,
                                            const double* x) {
#pragma unroll
  for (int s = 0; s < T::n_state_max; ++s) {
    if (s < v.n_state) {
      v.state[static_cast<long>(s) * v.stride + k] = x[s];
    }
  }
}

// Reset the zero_every entries due at step `step` (time `time`): the
// first ZERO_STEPS_CACHED steps read the block's precomputed masks.
template <typename T>
__device__ __forceinline__ void apply_zero_every(
    const zero_every_spec& z, const std::uint64_t* zero_steps, int step,
    double time, double* x) {
  for (int i = 0; i < z.n; ++i) {
    const bool hit = (zero_steps != nullptr && step < ZERO_STEPS_CACHED) ?
      ((zero_steps[i] >> step) & 1) != 0 : fmod(time, z.period[i]) == 0;
    if (hit) {
      if constexpr (T::n_state_max > 32) {
        // a large state lives in local memory: walk the mask's set bits
        // (an unrolled test of every entry made the compiler keep entries
        // in registers and spill around the samplers; SEIR: 2.5 KB of
        // spill code before, 0.24 KB after)
        for (int w = 0; w < ZERO_EVERY_WORDS; ++w) {
          std::uint64_t bits = z.mask[i][w];
          while (bits != 0) {
            const int s = w * 64 + __ffsll(static_cast<long long>(bits)) - 1;
            bits &= bits - 1;
            if (s < T::n_state_max) {
              x[s] = 0;
            }
          }
        }
      } else {
#pragma unroll
        for (int s = 0; s < T::n_state_max; ++s) {
          if (z.has(i, s)) {
            x[s] = 0;
          }
        }
      }
    }
  }
}

// States updated in place.  A system may declare `static constexpr bool
// update_in_place = true` when its `update` is correct with `state_next
// == state`: it reads each state entry before it writes that entry of
// state_next and never reads an entry after writing it.  Its particles
// then keep one state array instead of two, and the copy after each step
// goes (for a state too large for registers, both arrays live in local
// memory).  The arithmetic, and so every result, is the same.
template <typename T, typename = void>
struct update_in_place_of : std::false_type {};
template <typename T>
struct update_in_place_of<T, std::void_t<decltype(T::update_in_place)>>
  : std::integral_constant<bool, T::update_in_place> {};

// Advance one particle n_steps; on return the state is in x.  The
// reference swaps the two state pointers after each step; since `update`
// writes every entry of `state_next`, copying y back into x (register
// moves) is equivalent and keeps a single inlined copy of `update` in the
// loop (the samplers make it large; instruction-cache misses showed up as
// "no instruction" stalls when the loop held three copies).  A system
// updated in place steps x itself (y is unused).
template <typename T>
__device__ __forceinline__ void run_particle(
    double time, double dt, int n_steps,
    const typename T::shared_state& shared,
    typename T::internal_state& internal, const zero_every_spec& z,
    const std::uint64_t* zero_steps, random::rng_state& rng, double* x,
    double* y) {
  for (int i = 0; i < n_steps; ++i) {
    const double t = time + static_cast<double>(i) * dt;
    apply_zero_every<T>(z, zero_steps, i, t, x);
    if constexpr (update_in_place_of<T>::value) {
      T::update(t, dt, x, shared, internal, rng, x);
    } else {
      T::update(t, dt, x, shared, internal, rng, y);
#pragma unroll
      for (int s = 0; s < T::n_state_max; ++s) {
        x[s] = y[s];
      }
    }
  }
}

// Pick a block size for a system: big states need more registers per
// thread, so fewer threads per block keep occupancy sane.  Every kernel
// over a system's particles runs with this block size.
template <typename T>
constexpr int default_tile_size() {
  return T::n_state_max > 32 ? 128 : 256;
}

// The tile size for a set of groups: the system's block size, halved
// (down to one warp) while that leaves fewer than two tiles per SM, so
// that small problems spread over more of the GPU.  Results do not depend
// on it: per-group sums use a fixed chunk structure (filter.cuh).
template <typename T>
int choose_tile_size(const std::vector<int>& n_particles) {
  int dev = 0, sms = 0;
  DUST2_CUDA(cudaGetDevice(&dev));
  DUST2_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount,
                                    dev));
  auto n_tiles = [&](int ts) {
    long n = 0;
    for (int np : n_particles) {
      n += (np + ts - 1) / ts;
    }
    return n;
  };
  int t = default_tile_size<T>();
  while (t > 32 && n_tiles(t) < 2L * sms) {
    t /= 2;
  }
  return t;
}

// Blocks per SM the per-particle kernels of a system must fit, which caps
// registers per thread at 65536 / (tile size * blocks): a system may
// declare `static constexpr int min_blocks_per_sm`; the default, 2, allows
// 128 registers at 256 threads and 255 at 128.
template <typename T, typename = void>
struct min_blocks_of {
  static constexpr int value = 2;
};
template <typename T>
struct min_blocks_of<T, std::void_t<decltype(T::min_blocks_per_sm)>> {
  static constexpr int value = T::min_blocks_per_sm;
};

#define DUST2_PARTICLE_KERNEL(T)                                          \
  __global__ void __launch_bounds__(default_tile_size<T>(),               \
                                    min_blocks_of<T>::value)

// The per-particle kernels below run over a layout's run tiles: a block
// whose particles share one group stages that group's shared state in
// shared memory; in a packed tile each thread reads its own group's from
// global memory.
template <typename T>
DUST2_PARTICLE_KERNEL(T) k_initial(system_view<T> v, const int* active,
                                   double time) {
  __shared__ shared_smem<T> sm;
  const tile tl = v.tiles[blockIdx.x];
  const bool mixed = tl.group < 0;
  if (!mixed) {
    sm.load(v, tl.group);
  }
  __syncthreads();
  if (static_cast<int>(threadIdx.x) >= tl.count) {
    return;
  }
  const int k = tl.start + threadIdx.x;
  const int g = group_of(v, tl, k);
  if (active != nullptr && !active[g]) {
    return;
  }
  const auto& shared = mixed ? v.shared[g] : sm.shared();
  auto rng = load_rng(v.rng, v.stride, k, v.deterministic);
  typename T::internal_state internal{};
  double x[T::n_state_max];
  load_state<T>(v, k, x);
  T::initial(time, shared, internal, rng, x);
  store_state<T>(v, k, x);
  store_rng(v.rng, v.stride, k, rng);
  capture_error(v.errors, v.any_error, k, rng);
}

template <typename T>
DUST2_PARTICLE_KERNEL(T) k_run(system_view<T> v, double time, double dt,
                               int n_steps) {
  __shared__ shared_smem<T> sm;
  const tile tl = v.tiles[blockIdx.x];
  const bool mixed = tl.group < 0;
  if (!mixed) {
    sm.load(v, tl.group);
    sm.load_zero_steps(v, tl.group, time, dt, n_steps);
  }
  __syncthreads();
  if (static_cast<int>(threadIdx.x) >= tl.count) {
    return;
  }
  const int k = tl.start + threadIdx.x;
  const int g = group_of(v, tl, k);
  const auto& shared = mixed ? v.shared[g] : sm.shared();
  const zero_every_spec& zero = mixed ? v.zero_every[g] : sm.zero;
  auto rng = load_rng(v.rng, v.stride, k, v.deterministic);
  typename T::internal_state internal{};
  double x[T::n_state_max];
  double y[update_in_place_of<T>::value ? 1 : T::n_state_max];
  load_state<T>(v, k, x);
  run_particle<T>(time, dt, n_steps, shared, internal, zero,
                  mixed ? nullptr : sm.zero_steps, rng, x, y);
  store_state<T>(v, k, x);
  store_rng(v.rng, v.stride, k, rng);
  capture_error(v.errors, v.any_error, k, rng);
}

// out[k] = compare_data(time, state_k, data[group or 0]); data is
// [n_groups_data] of the system's data_type.
template <typename T>
DUST2_PARTICLE_KERNEL(T) k_compare(system_view<T> v, double time,
                          const typename T::data_type* data,
                          int n_groups_data, double* out) {
  __shared__ shared_smem<T> sm;
  const tile tl = v.tiles[blockIdx.x];
  const bool mixed = tl.group < 0;
  if (!mixed) {
    sm.load(v, tl.group);
  }
  __syncthreads();
  if (static_cast<int>(threadIdx.x) >= tl.count) {
    return;
  }
  if constexpr (has_compare_data<T>::value) {
    const int k = tl.start + threadIdx.x;
    const int g = group_of(v, tl, k);
    const auto& shared = mixed ? v.shared[g] : sm.shared();
    auto rng = load_rng(v.rng, v.stride, k, v.deterministic);
    typename T::internal_state internal{};
    double x[T::n_state_max];
    load_state<T>(v, k, x);
    const auto& d = data[n_groups_data == 1 ? 0 : g];
    out[k] = T::compare_data(time, x, d, shared, internal, rng);
    store_rng(v.rng, v.stride, k, rng);
    capture_error(v.errors, v.any_error, k, rng);
  }
}

// The device-resident discrete-time system.
template <typename T>
class discrete_system : public system_api {
public:
  using shared_state = typename T::shared_state;
  using data_type = typename T::data_type;
  static_assert(check_system<T>(), "invalid system");

  // rng_words: 4 words per particle stream, particles in global
  // (group-major) order.
  discrete_system(std::vector<shared_state> shared, double time, double dt,
                  const std::vector<int>& n_particles,
                  const std::vector<std::uint64_t>& rng_words,
                  bool deterministic, int tile_size = 0) :
    shared_(std::move(shared)),
    layout_(n_particles,
            tile_size > 0 ? tile_size : choose_tile_size<T>(n_particles)),
    n_state_(T::n_state(shared_[0])),
    time_(time), dt_(dt), deterministic_(deterministic) {
    if (static_cast<int>(shared_.size()) != layout_.n_groups) {
      throw std::runtime_error("shared state does not match group count");
    }
    if (layout_.tile_size > default_tile_size<T>()) {
      // the kernels are compiled for at most this many threads per block
      throw std::runtime_error("tile size above the system's block size");
    }
    for (std::size_t g = 1; g < shared_.size(); ++g) {
      const int n_g = T::n_state(shared_[g]);
      if (n_g != n_state_) {
        throw std::runtime_error(
          "State length for group " + std::to_string(g + 1) +
          " was different to previous groups; total length was expected "
          "to be " + std::to_string(n_state_) + " but it was " +
          std::to_string(n_g));
      }
    }
    if (n_state_ > T::n_state_max) {
      throw std::runtime_error("state larger than the system's n_state_max");
    }
    DUST2_CUDA(cudaStreamCreateWithFlags(&stream_, cudaStreamNonBlocking));
    const int stride = layout_.stride;
    state_.resize(static_cast<std::size_t>(n_state_) * stride);
    state_other_.resize(static_cast<std::size_t>(n_state_) * stride);
    rng_.resize(4 * static_cast<std::size_t>(stride));
    shared_dev_.resize(shared_.size());
    zero_dev_.resize(shared_.size());
    tiles_.resize(layout_.tiles.size());
    if (layout_.use_packed) {
      packed_.resize(layout_.packed.size());
      particle_group_.resize(layout_.n_total);
    }
    offsets_dev_.resize(layout_.n_groups);
    errors_.resize(layout_.n_total);
    any_error_.resize(1);
    DUST2_CUDA(cudaMemsetAsync(state_.data(), 0,
                               state_.size() * sizeof(double), stream_));
    DUST2_CUDA(cudaMemsetAsync(state_other_.data(), 0,
                               state_other_.size() * sizeof(double), stream_));
    upload_shared();
    std::vector<zero_every_spec> z;
    for (auto& s : shared_) {
      z.push_back(T::zero_every(s));
    }
    DUST2_CUDA(cudaMemcpyAsync(zero_dev_.data(), z.data(),
                               z.size() * sizeof(zero_every_spec),
                               cudaMemcpyHostToDevice, stream_));
    if (layout_.use_packed) {
      DUST2_CUDA(cudaMemcpyAsync(packed_.data(), layout_.packed.data(),
                                 layout_.packed.size() * sizeof(tile),
                                 cudaMemcpyHostToDevice, stream_));
      DUST2_CUDA(cudaMemcpyAsync(particle_group_.data(),
                                 layout_.particle_group.data(),
                                 layout_.n_total * sizeof(int),
                                 cudaMemcpyHostToDevice, stream_));
    }
    DUST2_CUDA(cudaMemcpyAsync(tiles_.data(), layout_.tiles.data(),
                               layout_.tiles.size() * sizeof(tile),
                               cudaMemcpyHostToDevice, stream_));
    DUST2_CUDA(cudaMemcpyAsync(offsets_dev_.data(), layout_.offset.data(),
                               layout_.offset.size() * sizeof(int),
                               cudaMemcpyHostToDevice, stream_));
    reset_errors();
    put_rng_state(rng_words.data());
    sync();
  }

  ~discrete_system() override {
    if (stream_ != nullptr) {
      cudaStreamSynchronize(stream_);
      cudaStreamDestroy(stream_);
    }
  }

  const char* name() const override {
    return T::name;
  }
  bool is_continuous() const override {
    return false;
  }
  bool has_compare() const override {
    return has_compare_data<T>::value;
  }
  int n_state() const override {
    return n_state_;
  }
  int n_groups() const override {
    return layout_.n_groups;
  }
  int n_particles_total() const override {
    return layout_.n_total;
  }
  const std::vector<int>& n_particles() const override {
    return layout_.n_particles;
  }
  std::vector<packing_entry> packing_state() const override {
    return T::packing_state(shared_[0]);
  }
  double time() const override {
    return time_;
  }
  double dt() const override {
    return dt_;
  }
  void set_time(double time) override {
    time_ = time;
  }
  bool errors_pending() const override {
    return errors_pending_;
  }
  int n_pars() const override {
    return parameter_length<T>();
  }
  int n_data() const override {
    if constexpr (has_compare_data<T>::value) {
      return static_cast<int>(sizeof(data_type) / sizeof(double));
    } else {
      return 0;
    }
  }

  system_view<T> view() {
    return system_view<T>{state_.data(), rng_.data(), shared_dev_.data(),
                          zero_dev_.data(), tiles_.data(), errors_.data(),
                          any_error_.data(), layout_.stride, n_state_,
                          deterministic_};
  }

  const group_layout& layout() const {
    return layout_;
  }
  cudaStream_t stream() const {
    return stream_;
  }
  double* state_ptr() {
    return state_.data();
  }
  double* state_other_ptr() {
    return state_other_.data();
  }
  const int* group_offsets_dev() const {
    return offsets_dev_.data();
  }
  // The view of the per-particle kernels (k_initial, k_run, k_compare and
  // the ODE kernels): over the layout's run tiles.
  system_view<T> run_view() {
    system_view<T> v = view();
    if (layout_.use_packed) {
      v.tiles = packed_.data();
      v.particle_group = particle_group_.data();
    }
    return v;
  }
  int n_run_tiles() const {
    return static_cast<int>(layout_.run_tiles().size());
  }

  const tile* tiles_dev() const {
    return tiles_.data();
  }
  void swap_state() {
    std::swap(state_, state_other_);
  }
  std::vector<shared_state>& shared_host() {
    return shared_;
  }

  // n_steps for a run from the current time to `time`
  // (discrete/system.hpp:62).
  int n_steps_to(double time) const {
    return static_cast<int>(std::round(std::max(0.0, time - time_) / dt_));
  }

  void run_to_time(double time) override {
    const int n_steps = n_steps_to(time);
    launch_run(time_, n_steps);
    check_errors_after();
    time_ = time_ + n_steps * dt_;
  }

  void launch_run(double t0, int n_steps) {
    if constexpr (has_update<T>::value && !dust2gpu::is_continuous<T>()) {
      if (n_steps > 0) {
        k_run<T><<<n_run_tiles(), layout_.tile_size, 0, stream_>>>(
          run_view(), t0, dt_, n_steps);
        DUST2_CUDA(cudaGetLastError());
      }
    } else {
      throw std::runtime_error("continuous-time system has no update()");
    }
  }

  void launch_initial(const int* active) {
    k_initial<T><<<n_run_tiles(), layout_.tile_size, 0, stream_>>>(
      run_view(), active, time_);
    DUST2_CUDA(cudaGetLastError());
  }

  void set_state_initial() override {
    reset_errors();
    launch_initial(nullptr);
    check_errors_after();
  }

  void get_state(double* out) override {
    const long n = static_cast<long>(layout_.n_total) * n_state_;
    ensure_scratch(n);
    k_gather_state<<<n_blocks(n, 256), 256, 0, stream_>>>(
      state_.data(), layout_.stride, layout_.n_total, nullptr, n_state_,
      scratch_.data());
    DUST2_CUDA(cudaGetLastError());
    DUST2_CUDA(cudaMemcpyAsync(out, scratch_.data(), n * sizeof(double),
                               cudaMemcpyDeviceToHost, stream_));
    sync();
  }

  void put_state(const double* in) override {
    reset_errors();
    const long n = static_cast<long>(layout_.n_total) * n_state_;
    ensure_scratch(n);
    DUST2_CUDA(cudaMemcpyAsync(scratch_.data(), in, n * sizeof(double),
                               cudaMemcpyHostToDevice, stream_));
    k_scatter_state<<<n_blocks(n, 256), 256, 0, stream_>>>(
      scratch_.data(), layout_.stride, layout_.n_total, n_state_,
      state_.data());
    DUST2_CUDA(cudaGetLastError());
    sync();
  }

  void get_rng_state(std::uint64_t* out) override {
    const int stride = layout_.stride;
    std::vector<std::uint64_t> soa(4 * static_cast<std::size_t>(stride));
    DUST2_CUDA(cudaMemcpyAsync(soa.data(), rng_.data(),
                               soa.size() * sizeof(std::uint64_t),
                               cudaMemcpyDeviceToHost, stream_));
    sync();
    for (int k = 0; k < layout_.n_total; ++k) {
      for (int w = 0; w < 4; ++w) {
        out[4 * static_cast<std::size_t>(k) + w] =
          soa[static_cast<std::size_t>(w) * stride + k];
      }
    }
  }

  void put_rng_state(const std::uint64_t* in) override {
    const int stride = layout_.stride;
    std::vector<std::uint64_t> soa(4 * static_cast<std::size_t>(stride), 0);
    for (int k = 0; k < layout_.n_total; ++k) {
      for (int w = 0; w < 4; ++w) {
        soa[static_cast<std::size_t>(w) * stride + k] =
          in[4 * static_cast<std::size_t>(k) + w];
      }
    }
    DUST2_CUDA(cudaMemcpyAsync(rng_.data(), soa.data(),
                               soa.size() * sizeof(std::uint64_t),
                               cudaMemcpyHostToDevice, stream_));
    sync();
  }

  void update_pars(const double* pars, const int* index_group,
                   int n_index_group) override {
    const int np = parameter_length<T>();
    if (index_group == nullptr) {
      for (int g = 0; g < layout_.n_groups; ++g) {
        T::update_shared(pars + static_cast<std::size_t>(g) * np, shared_[g]);
      }
    } else {
      for (int i = 0; i < n_index_group; ++i) {
        T::update_shared(pars + static_cast<std::size_t>(i) * np,
                         shared_[index_group[i]]);
      }
    }
    upload_shared();
    sync();
  }

  void simulate(const double* times, int n_times, const int* index_state,
                int n_index_state, double* out) override {
    const int n_save = index_state == nullptr ? n_state_ : n_index_state;
    const long per_time = static_cast<long>(layout_.n_total) * n_save;
    device_array<int> idx;
    if (index_state != nullptr) {
      idx.resize(n_index_state);
      DUST2_CUDA(cudaMemcpyAsync(idx.data(), index_state,
                                 n_index_state * sizeof(int),
                                 cudaMemcpyHostToDevice, stream_));
    }
    device_array<double> buf(static_cast<std::size_t>(per_time) * n_times);
    for (int i = 0; i < n_times; ++i) {
      const int n_steps = n_steps_to(times[i]);
      launch_run(time_, n_steps);
      time_ = time_ + n_steps * dt_;
      k_gather_state<<<n_blocks(per_time, 256), 256, 0, stream_>>>(
        state_.data(), layout_.stride, layout_.n_total, idx.data(), n_save,
        buf.data() + static_cast<std::size_t>(i) * per_time);
      DUST2_CUDA(cudaGetLastError());
    }
    DUST2_CUDA(cudaMemcpyAsync(out, buf.data(),
                               buf.size() * sizeof(double),
                               cudaMemcpyDeviceToHost, stream_));
    check_errors_after();
  }

  void simulate_device(const double* times, int n_times,
                       double* out_dev) override {
    const long per_time = static_cast<long>(layout_.n_total) * n_state_;
    for (int i = 0; i < n_times; ++i) {
      const int n_steps = n_steps_to(times[i]);
      launch_run(time_, n_steps);
      time_ = time_ + n_steps * dt_;
      k_gather_state<<<n_blocks(per_time, 256), 256, 0, stream_>>>(
        state_.data(), layout_.stride, layout_.n_total, nullptr, n_state_,
        out_dev + static_cast<std::size_t>(i) * per_time);
      DUST2_CUDA(cudaGetLastError());
    }
    check_errors_after();
  }

  void* stream_handle() override {
    return static_cast<void*>(stream_);
  }

  void reorder(const int* index) override {
    device_array<int> idx(layout_.n_total);
    DUST2_CUDA(cudaMemcpyAsync(idx.data(), index,
                               layout_.n_total * sizeof(int),
                               cudaMemcpyHostToDevice, stream_));
    k_reorder<<<layout_.n_tiles(), layout_.tile_size, 0, stream_>>>(
      state_.data(), state_other_.data(), layout_.stride, n_state_,
      tiles_.data(), offsets_dev_.data(), idx.data(), nullptr);
    DUST2_CUDA(cudaGetLastError());
    sync();
    swap_state();
  }

  void compare_data(const double* data, int n_groups_data,
                    double* out) override {
    if constexpr (has_compare_data<T>::value) {
      const int nd = n_data();
      std::vector<data_type> d;
      for (int g = 0; g < n_groups_data; ++g) {
        d.push_back(build_data_of<T>(data + static_cast<std::size_t>(g) * nd,
                                     shared_[n_groups_data == 1 ? 0 : g]));
      }
      device_array<data_type> d_dev(d.size());
      device_array<double> o(layout_.n_total);
      DUST2_CUDA(cudaMemcpyAsync(d_dev.data(), d.data(),
                                 d.size() * sizeof(data_type),
                                 cudaMemcpyHostToDevice, stream_));
      k_compare<T><<<n_run_tiles(), layout_.tile_size, 0, stream_>>>(
        run_view(), time_, d_dev.data(), n_groups_data, o.data());
      DUST2_CUDA(cudaGetLastError());
      DUST2_CUDA(cudaMemcpyAsync(out, o.data(),
                                 layout_.n_total * sizeof(double),
                                 cudaMemcpyDeviceToHost, stream_));
      check_errors_after();
    } else {
      throw std::runtime_error("system does not support compare_data");
    }
  }

  std::vector<ode_internals_row> ode_internals() override {
    return {};
  }
  std::vector<std::vector<double>> ode_step_times() override {
    return {};
  }

  void reset_errors() {
    DUST2_CUDA(cudaMemsetAsync(errors_.data(), 0,
                               errors_.size() * sizeof(particle_error),
                               stream_));
    DUST2_CUDA(cudaMemsetAsync(any_error_.data(), 0, sizeof(int), stream_));
    errors_pending_ = false;
  }

  // Synchronise, then turn any captured device errors into an exception.
  void check_errors_after() {
    int any = 0;
    DUST2_CUDA(cudaMemcpyAsync(&any, any_error_.data(), sizeof(int),
                               cudaMemcpyDeviceToHost, stream_));
    sync();
    if (any) {
      std::vector<particle_error> e(errors_.size());
      DUST2_CUDA(cudaMemcpy(e.data(), errors_.data(),
                            e.size() * sizeof(particle_error),
                            cudaMemcpyDeviceToHost));
      errors_pending_ = true;
      throw std::runtime_error(format_errors(e));
    }
  }

  void sync() {
    DUST2_CUDA(cudaStreamSynchronize(stream_));
  }

  void upload_shared() {
    DUST2_CUDA(cudaMemcpyAsync(shared_dev_.data(), shared_.data(),
                               shared_.size() * sizeof(shared_state),
                               cudaMemcpyHostToDevice, stream_));
  }

  int* any_error_dev() {
    return any_error_.data();
  }

private:
  void ensure_scratch(long n) {
    if (scratch_.size() < static_cast<std::size_t>(n)) {
      scratch_.resize(n);
    }
  }

  std::vector<shared_state> shared_;
  group_layout layout_;
  int n_state_;
  double time_;
  double dt_;
  bool deterministic_;
  bool errors_pending_ = false;
  cudaStream_t stream_ = nullptr;
  device_array<double> state_;
  device_array<double> state_other_;
  device_array<std::uint64_t> rng_;
  device_array<shared_state> shared_dev_;
  device_array<zero_every_spec> zero_dev_;
  device_array<tile> tiles_;
  device_array<tile> packed_;
  device_array<int> particle_group_;
  device_array<int> offsets_dev_;
  device_array<particle_error> errors_;
  device_array<int> any_error_;
  device_array<double> scratch_;
};

}  // namespace engine
}  // namespace dust2gpu
