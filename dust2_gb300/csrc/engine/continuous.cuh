// Continuous-time system engine on the GPU: the counterpart of
// dust2::dust_continuous<T> (inst/include/dust2/continuous/system.hpp
// :25-586) for pure-ODE systems (no mixed time, delays or events).
//
// One thread integrates one particle with the dopri5 solver of
// engine/dopri5.cuh.  Between calls each particle's solver record (the
// derivative, the dense-output coefficients of the last step, step size,
// error and step counters; `ode::internals`, solver.hpp:35-73) lives in
// structure-of-arrays device memory; during a call it lives in registers.
// `simulate` integrates through all output times inside one kernel, so a
// particle's record is loaded and stored once per call however many
// outputs are requested.
//
// Semantics kept from the reference:
//   the solver is (re)initialised at the start of a run for groups whose
//   state, parameters or time changed                       (:444-482)
//   run_to_time integrates [time, t] and sets time = t      (:80-106)
//   reorder moves the solver record with the state          (:175-204)
//   output variables are refreshed before state is read     (:206-209)
#pragma once

#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <memory>
#include <string>
#include <vector>

#include "../dust2gpu/system.hpp"
#include "api.hpp"
#include "device.cuh"
#include "discrete.cuh"
#include "dopri5.cuh"
#include "kernels_common.cuh"
#include "layout.hpp"

namespace dust2gpu {
namespace engine {

template <typename T>
constexpr int n_var_max() {
  return T::n_state_max - T::n_output;
}

struct ode_view {
  double* dydt;     // [NV][stride]
  double* c;        // [5][NV][stride]: c1..c5
  double* t0;
  double* t1;
  double* h;
  double* step_size;
  double* error;
  int* n_steps;
  int* n_steps_accepted;
  int* n_steps_rejected;
  int stride;
};

template <int NV>
__device__ __forceinline__ void load_ode(const ode_view& o, int k, int n_var,
                                         dopri5::state<NV>& st) {
  const long S = o.stride;
#pragma unroll
  for (int i = 0; i < NV; ++i) {
    if (i < n_var) {
      st.dydt[i] = o.dydt[i * S + k];
      st.c1[i] = o.c[(0 * NV + i) * S + k];
      st.c2[i] = o.c[(1 * NV + i) * S + k];
      st.c3[i] = o.c[(2 * NV + i) * S + k];
      st.c4[i] = o.c[(3 * NV + i) * S + k];
      st.c5[i] = o.c[(4 * NV + i) * S + k];
    }
  }
  st.t0 = o.t0[k];
  st.t1 = o.t1[k];
  st.h = o.h[k];
  st.step_size = o.step_size[k];
  st.error = o.error[k];
  st.n_steps = o.n_steps[k];
  st.n_steps_accepted = o.n_steps_accepted[k];
  st.n_steps_rejected = o.n_steps_rejected[k];
  st.err = 0;
}

template <int NV>
__device__ __forceinline__ void store_ode(const ode_view& o, int k, int n_var,
                                          const dopri5::state<NV>& st) {
  const long S = o.stride;
#pragma unroll
  for (int i = 0; i < NV; ++i) {
    if (i < n_var) {
      o.dydt[i * S + k] = st.dydt[i];
      o.c[(0 * NV + i) * S + k] = st.c1[i];
      o.c[(1 * NV + i) * S + k] = st.c2[i];
      o.c[(2 * NV + i) * S + k] = st.c3[i];
      o.c[(3 * NV + i) * S + k] = st.c4[i];
      o.c[(4 * NV + i) * S + k] = st.c5[i];
    }
  }
  o.t0[k] = st.t0;
  o.t1[k] = st.t1;
  o.h[k] = st.h;
  o.step_size[k] = st.step_size;
  o.error[k] = st.error;
  o.n_steps[k] = st.n_steps;
  o.n_steps_accepted[k] = st.n_steps_accepted;
  o.n_steps_rejected[k] = st.n_steps_rejected;
}

template <typename T>
__device__ __forceinline__ void refresh_output(
    double time, double* y, const typename T::shared_state& shared,
    typename T::internal_state& internal) {
  if constexpr (has_output<T>::value) {
    T::output(time, y, shared, internal);
  }
}

// Advance one particle from t to t_end.  Pure ODE systems (and mixed-time
// systems run without a dt) integrate with the solver.  Mixed-time
// systems with dt > 0 follow run_to_time1 (continuous/system.hpp:544-585)
// exactly: n_steps = (t_end - t) / dt truncated (none when t_end - t <
// dt, and then nothing happens); step s integrates from where the last one
// ended to t + s dt, the last step to t_end, so the first step is empty
// and, with several steps, the last spans two intervals; after each, the
// update runs at time t_end on a copy of the rest of the state and with a
// copy of the particle's generator (update_ takes it by value, :408-416,
// so the stream never advances); when the update changed the state the
// solver is re-initialised at t.  Returns the generator's error code from
// an update, or 0.
template <typename T, int NV>
__device__ __forceinline__ int advance(
    dopri5::solver<T, NV>& sol, double t, double t_end, double dt, double* y,
    const zero_every_spec& zero, dopri5::state<NV>& st,
    dopri5::scratch<NV>& s, const random::rng_state& rng,
    const typename T::shared_state& shared,
    typename T::internal_state& internal) {
  if constexpr (is_mixed_time<T>()) {
    if (dt > 0) {
      if (!(t_end > t)) {
        return 0;
      }
      const long n_steps = static_cast<long>((t_end - t) / dt);
      const int n_variables = sol.n_var + sol.n_special;
      double y_other[T::n_state_max];
      double t1 = t;
      for (long step = 0; step < n_steps && st.err == 0; ++step) {
        const double t0 = t1;
        t1 = (step == n_steps - 1) ? t_end :
          t + static_cast<double>(step) * dt;
        sol.run(t0, t1, y, zero, st, s);
        if (st.err != 0) {
          break;
        }
        for (int i = 0; i < n_variables; ++i) {
          y_other[i] = y[i];
        }
        random::rng_state r = rng;
        T::update(t_end, dt, y, shared, internal, r, y_other);
        if (r.err != 0) {
          return r.err;
        }
        bool changed = false;
        for (int i = 0; i < n_variables; ++i) {
          changed = changed || !(y_other[i] == y[i]);
          y[i] = y_other[i];
        }
        if (changed) {
          sol.initialise(t, y, st, s);
        }
      }
      return 0;
    }
  }
  sol.run(t, t_end, y, zero, st, s);
  return 0;
}

// Integrate every particle through `times` (n_times >= 1), writing the
// state at each time to out[(i * n_total + k) * n_out + j] (j over
// index_out, or over all state when index_out is null) when out is set.
template <typename T>
__global__ void k_ode_run(system_view<T> v, ode_view o,
                          dopri5::control_dev ctl, double time0, double dt,
                          const double* times, int n_times,
                          const int* requires_init, int n_total,
                          double* out, const int* index_out, int n_out) {
  constexpr int NV = n_var_max<T>();
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
  const auto& shared = mixed ? v.shared[g] : sm.shared();
  const zero_every_spec& zero = mixed ? v.zero_every[g] : sm.zero;
  const int n_var = v.n_state - T::n_output - n_special<T>();
  typename T::internal_state internal{};
  double y[T::n_state_max];
  load_state<T>(v, k, y);
  const auto rng = load_rng(v.rng, v.stride, k, v.deterministic);
  int update_err = 0;
  dopri5::state<NV> st;
  dopri5::scratch<NV> s;
  load_ode<NV>(o, k, n_var, st);
  dopri5::solver<T, NV> sol{ctl, shared, internal, n_var, k};
  sol.n_special = n_special<T>();
  if (requires_init[g]) {
    sol.initialise(time0, y, st, s);
  }
  double t = time0;
  for (int i = 0; i < n_times; ++i) {
    const double t_end = times[i];
    if (st.err == 0 && update_err == 0) {
      update_err = advance<T, NV>(sol, t, t_end, dt, y, zero, st, s, rng,
                                  shared, internal);
    }
    t = t_end;
    if (out != nullptr) {
      refresh_output<T>(t_end, y, shared, internal);
      double* dst = out + (static_cast<long>(i) * n_total + k) * n_out;
      for (int j = 0; j < n_out; ++j) {
        const int sj = index_out == nullptr ? j : index_out[j];
#pragma unroll
        for (int q = 0; q < T::n_state_max; ++q) {
          if (q == sj) {
            dst[j] = y[q];
          }
        }
      }
    }
  }
  refresh_output<T>(t, y, shared, internal);
  store_state<T>(v, k, y);
  store_ode<NV>(o, k, n_var, st);
  if (st.err != 0 || update_err != 0) {
    random::rng_state r{};
    r.err = st.err != 0 ? st.err : update_err;
    capture_error(v.errors, v.any_error, k, r);
  }
}

// Refresh output variables of every particle (state() in the reference).
template <typename T>
__global__ void k_ode_output(system_view<T> v, double time) {
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
  const auto& shared = mixed ? v.shared[group_of(v, tl, k)] : sm.shared();
  typename T::internal_state internal{};
  double y[T::n_state_max];
  load_state<T>(v, k, y);
  refresh_output<T>(time, y, shared, internal);
  store_state<T>(v, k, y);
}

template <typename T>
class continuous_system : public system_api {
public:
  using shared_state = typename T::shared_state;
  using data_type = typename T::data_type;
  static constexpr int NV = n_var_max<T>();
  static_assert(check_system<T>(), "invalid system");

  // dt: the update interval of a mixed-time system (0: no updates; always
  // 0 for a pure ODE).
  continuous_system(std::vector<shared_state> shared, double time,
                    const ode_control& control,
                    const std::vector<int>& n_particles,
                    const std::vector<std::uint64_t>& rng_words,
                    bool deterministic, int tile_size = 0, double dt = 0) :
    base_(std::move(shared), time, 0.0, n_particles, rng_words,
          deterministic, tile_size > 0 ? tile_size : 128),
    control_(control), dt_(dt),
    requires_initialise_(base_.n_groups(), 1) {
    const auto& L = base_.layout();
    const std::size_t S = L.stride;
    dydt_.resize(NV * S);
    c_.resize(5 * NV * S);
    t0_.resize(S);
    t1_.resize(S);
    h_.resize(S);
    step_size_.resize(S);
    error_.resize(S);
    n_steps_.resize(S);
    n_acc_.resize(S);
    n_rej_.resize(S);
    zero_ode(false);
    critical_.resize(std::max<std::size_t>(1, control_.critical_times.size()));
    if (!control_.critical_times.empty()) {
      DUST2_CUDA(cudaMemcpy(critical_.data(), control_.critical_times.data(),
                            control_.critical_times.size() * sizeof(double),
                            cudaMemcpyHostToDevice));
    }
    if (control_.debug_record_step_times) {
      step_times_.resize(static_cast<std::size_t>(L.n_total) * step_times_cap);
      n_step_times_.resize(L.n_total);
      DUST2_CUDA(cudaMemset(n_step_times_.data(), 0, L.n_total * sizeof(int)));
    }
    requires_init_dev_.resize(base_.n_groups());
    other_.resize((6 * NV + 8) * S);
  }

  const char* name() const override {
    return T::name;
  }
  bool is_continuous() const override {
    return true;
  }
  bool has_compare() const override {
    return has_compare_data<T>::value;
  }
  int n_state() const override {
    return base_.n_state();
  }
  int n_groups() const override {
    return base_.n_groups();
  }
  int n_particles_total() const override {
    return base_.n_particles_total();
  }
  const std::vector<int>& n_particles() const override {
    return base_.n_particles();
  }
  std::vector<packing_entry> packing_state() const override {
    return base_.packing_state();
  }
  double time() const override {
    return base_.time();
  }
  double dt() const override {
    return dt_;
  }
  bool errors_pending() const override {
    return base_.errors_pending();
  }
  int n_pars() const override {
    return base_.n_pars();
  }
  int n_data() const override {
    return base_.n_data();
  }

  void set_time(double time) override {
    base_.set_time(time);
    mark_all();
  }

  void run_to_time(double time) override {
    const double t = time;
    launch_run(&t, 1, nullptr, nullptr, 0);
    base_.check_errors_after();
    base_.set_time(time);
  }

  void set_state_initial() override {
    base_.set_state_initial();
    mark_all();
  }

  void get_state(double* out) override {
    refresh_outputs();
    base_.get_state(out);
  }

  void put_state(const double* in) override {
    base_.put_state(in);
    mark_all();
  }

  void get_rng_state(std::uint64_t* out) override {
    base_.get_rng_state(out);
  }

  void put_rng_state(const std::uint64_t* in) override {
    base_.put_rng_state(in);
  }

  void update_pars(const double* pars, const int* index_group,
                   int n_index_group) override {
    base_.update_pars(pars, index_group, n_index_group);
    if (index_group == nullptr) {
      mark_all();
    } else {
      for (int i = 0; i < n_index_group; ++i) {
        requires_initialise_[index_group[i]] = 1;
      }
    }
  }

  discrete_system<T>& base() {
    return base_;
  }

  // Launch a whole-run kernel of the unfilter (engine/unfilter.cuh) with
  // this system's solver record: kernel(view, ode view, control, time,
  // dt, times, n_times, requires_init, active, data, n_groups_data, ll,
  // save) with `save` saying what to keep at each data time.
  template <typename K, typename D, typename S>
  void launch_unfilter(const double* times_dev, int n_times,
                       const int* active, const D* data, int n_groups_data,
                       double* ll, K kernel, const S& save) {
    const auto& L = base_.layout();
    auto s = base_.stream();
    DUST2_CUDA(cudaMemcpyAsync(requires_init_dev_.data(),
                               requires_initialise_.data(),
                               requires_initialise_.size() * sizeof(int),
                               cudaMemcpyHostToDevice, s));
    kernel<<<base_.n_run_tiles(), L.tile_size, 0, s>>>(
      base_.run_view(), view_ode(), control_dev(), base_.time(), dt_,
      times_dev, n_times, requires_init_dev_.data(), active, data,
      n_groups_data, ll, save);
    DUST2_CUDA(cudaGetLastError());
    std::fill(requires_initialise_.begin(), requires_initialise_.end(), 0);
  }

  void simulate(const double* times, int n_times, const int* index_state,
                int n_index_state, double* out) override {
    const auto& L = base_.layout();
    const int n_out = index_state == nullptr ? base_.n_state() : n_index_state;
    device_array<int> idx;
    if (index_state != nullptr) {
      idx.resize(n_index_state);
      DUST2_CUDA(cudaMemcpy(idx.data(), index_state,
                            n_index_state * sizeof(int),
                            cudaMemcpyHostToDevice));
    }
    // The output times are integrated in up to 8 consecutive launches
    // (each continuing from the last one's state and solver record, so the
    // result is that of one launch), all enqueued first; each chunk of
    // outputs is then copied to the host on a second stream as soon as its
    // launch is done, while the next chunk integrates.
    const std::size_t per_time = static_cast<std::size_t>(L.n_total) * n_out;
    if (sim_buf_.size() < per_time * n_times) {
      sim_buf_.resize(per_time * n_times);
    }
    if (copy_stream_ == nullptr) {
      DUST2_CUDA(cudaStreamCreateWithFlags(&copy_stream_,
                                           cudaStreamNonBlocking));
      for (auto& e : chunk_done_) {
        DUST2_CUDA(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
      }
    }
    const int n_chunks = std::min(n_times, n_sim_chunks);
    std::vector<int> first(n_chunks + 1);
    for (int c = 0; c <= n_chunks; ++c) {
      first[c] = static_cast<int>(static_cast<long>(n_times) * c / n_chunks);
    }
    for (int c = 0; c < n_chunks; ++c) {
      if (c > 0) {
        base_.set_time(times[first[c] - 1]);
      }
      launch_run(times + first[c], first[c + 1] - first[c],
                 sim_buf_.data() + first[c] * per_time, idx.data(), n_out);
      DUST2_CUDA(cudaEventRecord(chunk_done_[c], base_.stream()));
    }
    for (int c = 0; c < n_chunks; ++c) {
      DUST2_CUDA(cudaStreamWaitEvent(copy_stream_, chunk_done_[c], 0));
      DUST2_CUDA(cudaMemcpyAsync(
        out + first[c] * per_time, sim_buf_.data() + first[c] * per_time,
        (first[c + 1] - first[c]) * per_time * sizeof(double),
        cudaMemcpyDeviceToHost, copy_stream_));
    }
    DUST2_CUDA(cudaStreamSynchronize(copy_stream_));
    base_.check_errors_after();
    base_.set_time(times[n_times - 1]);
  }

  ~continuous_system() override {
    if (copy_stream_ != nullptr) {
      cudaStreamSynchronize(copy_stream_);
      for (auto e : chunk_done_) {
        cudaEventDestroy(e);
      }
      cudaStreamDestroy(copy_stream_);
    }
  }

  // Run through `times` leaving outputs in a caller-provided device
  // buffer.
  void simulate_device(const double* times, int n_times,
                       double* out_dev) override {
    launch_run(times, n_times, out_dev, nullptr, base_.n_state());
    base_.check_errors_after();
    base_.set_time(times[n_times - 1]);
  }

  void* stream_handle() override {
    return base_.stream_handle();
  }

  void reorder(const int* index) override {
    const auto& L = base_.layout();
    device_array<int> idx(L.n_total);
    DUST2_CUDA(cudaMemcpyAsync(idx.data(), index, L.n_total * sizeof(int),
                               cudaMemcpyHostToDevice, base_.stream()));
    auto s = base_.stream();
    const int S = L.stride;
    auto move = [&](double* a, int n_rows) {
      k_reorder<<<L.n_tiles(), L.tile_size, 0, s>>>(
        a, other_.data(), S, n_rows, base_.tiles_dev(),
        base_.group_offsets_dev(), idx.data(), nullptr);
      DUST2_CUDA(cudaMemcpyAsync(a, other_.data(),
                                 static_cast<std::size_t>(n_rows) * S *
                                 sizeof(double),
                                 cudaMemcpyDeviceToDevice, s));
    };
    move(dydt_.data(), NV);
    move(c_.data(), 5 * NV);
    move(t0_.data(), 1);
    move(t1_.data(), 1);
    move(h_.data(), 1);
    move(step_size_.data(), 1);
    move(error_.data(), 1);
    DUST2_CUDA(cudaGetLastError());
    base_.sync();
    // integer counters: reorder on the host (small)
    auto reorder_int = [&](device_array<int>& a) {
      std::vector<int> h(L.n_total), r(L.n_total);
      DUST2_CUDA(cudaMemcpy(h.data(), a.data(), L.n_total * sizeof(int),
                            cudaMemcpyDeviceToHost));
      for (int g = 0; g < L.n_groups; ++g) {
        for (int j = 0; j < L.n_particles[g]; ++j) {
          const int k = L.offset[g] + j;
          r[k] = h[L.offset[g] + index[k]];
        }
      }
      DUST2_CUDA(cudaMemcpy(a.data(), r.data(), L.n_total * sizeof(int),
                            cudaMemcpyHostToDevice));
    };
    reorder_int(n_steps_);
    reorder_int(n_acc_);
    reorder_int(n_rej_);
    base_.reorder(index);
  }

  void compare_data(const double* data, int n_groups_data,
                    double* out) override {
    base_.compare_data(data, n_groups_data, out);
  }

  std::vector<ode_internals_row> ode_internals() override {
    const auto& L = base_.layout();
    const int N = L.n_total;
    std::vector<double> ss(N), er(N);
    std::vector<int> ns(N), na(N), nr(N);
    DUST2_CUDA(cudaMemcpy(ss.data(), step_size_.data(), N * sizeof(double),
                          cudaMemcpyDeviceToHost));
    DUST2_CUDA(cudaMemcpy(er.data(), error_.data(), N * sizeof(double),
                          cudaMemcpyDeviceToHost));
    DUST2_CUDA(cudaMemcpy(ns.data(), n_steps_.data(), N * sizeof(int),
                          cudaMemcpyDeviceToHost));
    DUST2_CUDA(cudaMemcpy(na.data(), n_acc_.data(), N * sizeof(int),
                          cudaMemcpyDeviceToHost));
    DUST2_CUDA(cudaMemcpy(nr.data(), n_rej_.data(), N * sizeof(int),
                          cudaMemcpyDeviceToHost));
    std::vector<ode_internals_row> ret(N);
    for (int k = 0; k < N; ++k) {
      ret[k] = ode_internals_row{ss[k], er[k], ns[k], na[k], nr[k]};
    }
    return ret;
  }

  std::vector<std::vector<double>> ode_step_times() override {
    const auto& L = base_.layout();
    const int N = L.n_total;
    std::vector<std::vector<double>> ret(N);
    if (!control_.debug_record_step_times) {
      return ret;
    }
    std::vector<int> n(N);
    std::vector<double> t(static_cast<std::size_t>(N) * step_times_cap);
    DUST2_CUDA(cudaMemcpy(n.data(), n_step_times_.data(), N * sizeof(int),
                          cudaMemcpyDeviceToHost));
    DUST2_CUDA(cudaMemcpy(t.data(), step_times_.data(),
                          t.size() * sizeof(double), cudaMemcpyDeviceToHost));
    for (int k = 0; k < N; ++k) {
      const int nk = std::min(n[k], step_times_cap);
      ret[k].assign(t.begin() + static_cast<long>(k) * step_times_cap,
                    t.begin() + static_cast<long>(k) * step_times_cap + nk);
    }
    return ret;
  }

  cudaStream_t stream() const {
    return base_.stream();
  }

  static constexpr int step_times_cap = 4096;

  dopri5::control_dev control_dev() {
    dopri5::control_dev c;
    c.max_steps = control_.max_steps;
    c.atol = control_.atol;
    c.rtol = control_.rtol;
    c.step_size_min = control_.step_size_min;
    c.step_size_max = control_.step_size_max;
    c.factor_safe = control_.factor_safe;
    c.facc1 = 1 / control_.factor_min;
    c.facc2 = 1 / control_.factor_max;
    c.beta = control_.beta;
    c.constant = control_.constant;
    c.critical = critical_.data();
    c.n_critical = static_cast<int>(control_.critical_times.size());
    c.step_times = control_.debug_record_step_times ? step_times_.data() :
      nullptr;
    c.n_step_times = control_.debug_record_step_times ?
      n_step_times_.data() : nullptr;
    c.step_times_cap = step_times_cap;
    return c;
  }

  ode_view view_ode() {
    return ode_view{dydt_.data(), c_.data(), t0_.data(), t1_.data(),
                    h_.data(), step_size_.data(), error_.data(),
                    n_steps_.data(), n_acc_.data(), n_rej_.data(),
                    base_.layout().stride};
  }

  // Enqueue the reordering of every particle's solver record on stream s
  // (continuous/system.hpp:199-203, ode_internals moved with the state);
  // arguments as k_reorder's.
  void enqueue_reorder_record(const tile* tiles, int n_tiles, int tile_size,
                              const int* group_offset, const int* index,
                              const int* group_mode, cudaStream_t s) {
    const int S = base_.layout().stride;
    auto move = [&](double* a, int n_rows) {
      k_reorder<<<n_tiles, tile_size, 0, s>>>(a, other_.data(), S, n_rows,
                                              tiles, group_offset, index,
                                              group_mode);
      DUST2_CUDA(cudaMemcpyAsync(a, other_.data(),
                                 static_cast<std::size_t>(n_rows) * S *
                                 sizeof(double),
                                 cudaMemcpyDeviceToDevice, s));
    };
    move(dydt_.data(), NV);
    move(c_.data(), 5 * NV);
    move(t0_.data(), 1);
    move(t1_.data(), 1);
    move(h_.data(), 1);
    move(step_size_.data(), 1);
    move(error_.data(), 1);
    int* tmp = reinterpret_cast<int*>(other_.data());
    for (int* a : {n_steps_.data(), n_acc_.data(), n_rej_.data()}) {
      k_reorder_int<<<n_tiles, tile_size, 0, s>>>(a, tmp, S, tiles,
                                                  group_offset, index,
                                                  group_mode);
      DUST2_CUDA(cudaMemcpyAsync(a, tmp, static_cast<std::size_t>(S) *
                                 sizeof(int), cudaMemcpyDeviceToDevice, s));
    }
    DUST2_CUDA(cudaGetLastError());
  }

private:

  void launch_run(const double* times, int n_times, double* out_dev,
                  const int* index_dev, int n_out) {
    const auto& L = base_.layout();
    auto s = base_.stream();
    if (times_dev_.size() < static_cast<std::size_t>(n_times)) {
      times_dev_.resize(n_times);
    }
    DUST2_CUDA(cudaMemcpyAsync(times_dev_.data(), times,
                               n_times * sizeof(double),
                               cudaMemcpyHostToDevice, s));
    DUST2_CUDA(cudaMemcpyAsync(requires_init_dev_.data(),
                               requires_initialise_.data(),
                               requires_initialise_.size() * sizeof(int),
                               cudaMemcpyHostToDevice, s));
    k_ode_run<T><<<base_.n_run_tiles(), L.tile_size, 0, s>>>(
      base_.run_view(), view_ode(), control_dev(), base_.time(), dt_,
      times_dev_.data(), n_times, requires_init_dev_.data(), L.n_total,
      out_dev, index_dev, n_out);
    DUST2_CUDA(cudaGetLastError());
    std::fill(requires_initialise_.begin(), requires_initialise_.end(), 0);
  }

  void refresh_outputs() {
    if constexpr (has_output<T>::value) {
      const auto& L = base_.layout();
      k_ode_output<T><<<base_.n_run_tiles(), L.tile_size, 0,
                        base_.stream()>>>(base_.run_view(), base_.time());
      DUST2_CUDA(cudaGetLastError());
    }
  }

  void mark_all() {
    std::fill(requires_initialise_.begin(), requires_initialise_.end(), 1);
  }

  void zero_ode(bool) {
    auto z = [](auto& a) {
      DUST2_CUDA(cudaMemset(a.data(), 0, a.size() * sizeof(*a.data())));
    };
    z(dydt_);
    z(c_);
    z(t0_);
    z(t1_);
    z(h_);
    z(step_size_);
    z(error_);
    z(n_steps_);
    z(n_acc_);
    z(n_rej_);
  }

  // The discrete engine supplies state, generator, parameters, tiles,
  // errors and the state verbs; this class adds the solver record.
  discrete_system<T> base_;
  ode_control control_;
  double dt_ = 0;
  std::vector<int> requires_initialise_;
  device_array<double> dydt_, c_, t0_, t1_, h_, step_size_, error_;
  device_array<int> n_steps_, n_acc_, n_rej_;
  device_array<double> critical_;
  device_array<double> step_times_;
  device_array<int> n_step_times_;
  device_array<int> requires_init_dev_;
  device_array<double> times_dev_;
  device_array<double> other_;
  // simulate(): output buffer and the stream its chunks are copied on
  static constexpr int n_sim_chunks = 8;
  device_array<double> sim_buf_;
  cudaStream_t copy_stream_ = nullptr;
  cudaEvent_t chunk_done_[n_sim_chunks] = {};
};

}  // namespace engine
}  // namespace dust2gpu
