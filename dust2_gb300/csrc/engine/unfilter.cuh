// Deterministic likelihood ("unfilter"): the counterpart of
// dust2::unfilter (inst/include/dust2/unfilter.hpp:10-73) for discrete-
// and continuous-time systems.
//
// The reference runs its deterministic system to each data time in turn
// (run_to_time, :55), compares every particle with that time's data
// (compare_data, :56) and adds the result to a per-particle
// log-likelihood (:57-59); nothing couples particles, so there is no
// resampling.  Here one kernel does the whole run: each thread advances
// its particle through all data times (update steps, or the dopri5 solver
// for continuous systems), calling compare_data after each and keeping
// the running sum in a register; the state and solver record are loaded
// and stored once.  The system is created deterministic with the
// reference's fixed seed 42 (r/discrete/unfilter.hpp:37-39), so every
// sampler returns its expectation.
//
// The continuous reference compares against the state as it is after
// run_to_time, whose output variables are not recomputed
// (continuous/system.hpp:100-106, 279-305), so the compare here sees the
// same, and outputs are refreshed only when the run ends (as state() does,
// :206-209).
#pragma once

#include <cuda_runtime.h>

#include <memory>
#include <vector>

#include "api.hpp"
#include "continuous.cuh"
#include "device.cuh"
#include "discrete.cuh"
#include "filter.cuh"

namespace dust2gpu {
namespace engine {

template <typename T>
DUST2_PARTICLE_KERNEL(T) k_unfilter_discrete(
    system_view<T> v, const int* active, const obs_step* sched,
    int n_times, double dt, const typename T::data_type* data,
    int n_groups_data, double* ll) {
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
  if (!active[g]) {
    return;
  }
  if constexpr (has_compare_data<T>::value) {
    const auto& shared = mixed ? v.shared[g] : sm.shared();
    const zero_every_spec& zero = mixed ? v.zero_every[g] : sm.zero;
    auto rng = load_rng(v.rng, v.stride, k, v.deterministic);
    typename T::internal_state internal{};
    double x[T::n_state_max];
    double y[T::n_state_max];
    load_state<T>(v, k, x);
    double acc = 0;
    for (int i = 0; i < n_times; ++i) {
      const obs_step st = sched[i];
      run_particle<T>(st.t0, dt, st.n_steps, shared, internal, zero, nullptr,
                      rng, x, y);
      const auto& d = data[static_cast<long>(i) * n_groups_data +
                           (n_groups_data == 1 ? 0 : g)];
      acc += T::compare_data(st.t_compare, x, d, shared, internal, rng);
    }
    store_state<T>(v, k, x);
    store_rng(v.rng, v.stride, k, rng);
    capture_error(v.errors, v.any_error, k, rng);
    ll[k] = acc;
  }
}

template <typename T>
DUST2_PARTICLE_KERNEL(T) k_unfilter_ode(
    system_view<T> v, ode_view o, dopri5::control_dev ctl, double time0,
    const double* times, int n_times, const int* requires_init,
    const int* active, const typename T::data_type* data, int n_groups_data,
    double* ll) {
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
  if (!active[g]) {
    return;
  }
  if constexpr (has_compare_data<T>::value) {
    const auto& shared = mixed ? v.shared[g] : sm.shared();
    const zero_every_spec& zero = mixed ? v.zero_every[g] : sm.zero;
    const int n_var = v.n_state - T::n_output;
    auto rng = load_rng(v.rng, v.stride, k, v.deterministic);
    typename T::internal_state internal{};
    double y[T::n_state_max];
    load_state<T>(v, k, y);
    dopri5::state<NV> st;
    dopri5::scratch<NV> s;
    load_ode<NV>(o, k, n_var, st);
    dopri5::solver<T, NV> sol{ctl, shared, internal, n_var, k};
    if (requires_init[g]) {
      sol.initialise(time0, y, st, s);
    }
    double t = time0;
    double acc = 0;
    for (int i = 0; i < n_times; ++i) {
      const double t_end = times[i];
      if (st.err == 0) {
        sol.run(t, t_end, y, zero, st, s);
      }
      t = t_end;
      const auto& d = data[static_cast<long>(i) * n_groups_data +
                           (n_groups_data == 1 ? 0 : g)];
      acc += T::compare_data(t_end, y, d, shared, internal, rng);
    }
    refresh_output<T>(t, y, shared, internal);
    store_state<T>(v, k, y);
    store_ode<NV>(o, k, n_var, st);
    ll[k] = acc;
    if (st.err != 0) {
      rng.err = st.err;
    }
    capture_error(v.errors, v.any_error, k, rng);
  }
}

template <typename T>
class unfilter_engine : public unfilter_api {
public:
  using data_type = typename T::data_type;
  using system_type = std::conditional_t<is_continuous<T>(),
                                         continuous_system<T>,
                                         discrete_system<T>>;

  unfilter_engine(std::unique_ptr<system_type> sys, double time_start,
                  std::vector<double> times, std::vector<data_type> data,
                  int n_groups_data) :
    sys_(std::move(sys)), time_start_(time_start), times_(std::move(times)),
    n_groups_data_(n_groups_data) {
    const int G = sys_->n_groups();
    const int N = sys_->n_particles_total();
    active_.resize(G);
    ll_.resize(N);
    data_.resize(data.size());
    times_dev_.resize(times_.size());
    DUST2_CUDA(cudaMemcpy(data_.data(), data.data(),
                          data.size() * sizeof(data_type),
                          cudaMemcpyHostToDevice));
    DUST2_CUDA(cudaMemcpy(times_dev_.data(), times_.data(),
                          times_.size() * sizeof(double),
                          cudaMemcpyHostToDevice));
    if constexpr (!is_continuous<T>()) {
      double t = time_start_;
      std::vector<obs_step> sched;
      for (double ti : times_) {
        const int n = static_cast<int>(
          std::round(std::max(0.0, ti - t) / sys_->dt()));
        sched.push_back(obs_step{t, n, t + n * sys_->dt()});
        t = t + n * sys_->dt();
      }
      t_end_ = t;
      sched_.resize(sched.size());
      DUST2_CUDA(cudaMemcpy(sched_.data(), sched.data(),
                            sched.size() * sizeof(obs_step),
                            cudaMemcpyHostToDevice));
    }
  }

  system_api& sys() override {
    return *sys_;
  }
  int n_times() const override {
    return static_cast<int>(times_.size());
  }

  void update_pars(const double* pars, const int* index_group,
                   int n_index_group) override {
    sys_->update_pars(pars, index_group, n_index_group);
  }

  // unfilter.hpp:42-73 with its reset (:162-186); ll_out: one value per
  // particle of each requested group, groups in index_group order.
  void run(const double* initial, const int* index_group, int n_index_group,
           double* ll_out) override {
    auto& S = *sys_;
    const int G = S.n_groups();
    std::vector<int> active(G, index_group == nullptr ? 1 : 0);
    if (index_group != nullptr) {
      for (int i = 0; i < n_index_group; ++i) {
        active[index_group[i]] = 1;
      }
    }
    S.set_time(time_start_);
    if (initial != nullptr) {
      S.put_state(initial);
    } else {
      S.set_state_initial();
    }
    auto& base = base_of(S);
    auto s = base.stream();
    DUST2_CUDA(cudaMemcpyAsync(active_.data(), active.data(),
                               G * sizeof(int), cudaMemcpyHostToDevice, s));
    DUST2_CUDA(cudaMemsetAsync(ll_.data(), 0, ll_.size() * sizeof(double),
                               s));
    base.reset_errors();
    const auto& L = base.layout();
    if constexpr (is_continuous<T>()) {
      S.launch_unfilter(times_dev_.data(), n_times(), active_.data(),
                        data_.data(), n_groups_data_, ll_.data(),
                        k_unfilter_ode<T>);
      base.check_errors_after();
      base.set_time(times_.back());
    } else {
      k_unfilter_discrete<T><<<S.n_run_tiles(), L.tile_size, 0, s>>>(
        S.run_view(), active_.data(), sched_.data(), n_times(), S.dt(),
        data_.data(), n_groups_data_, ll_.data());
      DUST2_CUDA(cudaGetLastError());
      S.check_errors_after();
      S.set_time(t_end_);
    }
    std::vector<double> ll(ll_.size());
    DUST2_CUDA(cudaMemcpy(ll.data(), ll_.data(), ll.size() * sizeof(double),
                          cudaMemcpyDeviceToHost));
    std::size_t pos = 0;
    auto copy_group = [&](int g) {
      for (int j = 0; j < L.n_particles[g]; ++j) {
        ll_out[pos++] = ll[L.offset[g] + j];
      }
    };
    if (index_group == nullptr) {
      for (int g = 0; g < G; ++g) {
        copy_group(g);
      }
    } else {
      for (int i = 0; i < n_index_group; ++i) {
        copy_group(index_group[i]);
      }
    }
  }

private:
  static discrete_system<T>& base_of(discrete_system<T>& s) {
    return s;
  }
  static discrete_system<T>& base_of(continuous_system<T>& s) {
    return s.base();
  }

  std::unique_ptr<system_type> sys_;
  double time_start_;
  std::vector<double> times_;
  int n_groups_data_;
  double t_end_ = 0;  // time after the last data time (discrete)
  device_array<int> active_;
  device_array<double> ll_;
  device_array<data_type> data_;
  device_array<double> times_dev_;
  device_array<obs_step> sched_;
};

}  // namespace engine
}  // namespace dust2gpu
