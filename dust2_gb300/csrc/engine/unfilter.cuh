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

// What a run keeps at each data time (unfilter.hpp:60-62, 100-102,
// trajectories_.add): state entries `index` of every particle in `traj`
// ([time][entry][particle]), and the full state at the data times whose
// snap_slot is >= 0 (the snapshot's position) in `snap`
// ([snapshot][state][particle]).  Null buffers keep nothing.
struct unfilter_save {
  const int* index = nullptr;
  int n_save = 0;
  double* traj = nullptr;
  const int* snap_slot = nullptr;
  double* snap = nullptr;
};

__device__ __forceinline__ void save_data_time(const unfilter_save& sv,
                                               int i, const double* x,
                                               int n_state, long stride,
                                               int k) {
  if (sv.traj != nullptr) {
    for (int s = 0; s < sv.n_save; ++s) {
      sv.traj[(static_cast<long>(i) * sv.n_save + s) * stride + k] =
        x[sv.index[s]];
    }
  }
  if (sv.snap != nullptr) {
    const int slot = sv.snap_slot[i];
    if (slot >= 0) {
      for (int s = 0; s < n_state; ++s) {
        sv.snap[(static_cast<long>(slot) * n_state + s) * stride + k] = x[s];
      }
    }
  }
}

template <typename T>
DUST2_PARTICLE_KERNEL(T) k_unfilter_discrete(
    system_view<T> v, const int* active, const obs_step* sched,
    int n_times, double dt, const typename T::data_type* data,
    int n_groups_data, double* ll, unfilter_save sv) {
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
      save_data_time(sv, i, x, v.n_state, v.stride, k);
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
    double dt, const double* times, int n_times, const int* requires_init,
    const int* active, const typename T::data_type* data, int n_groups_data,
    double* ll, unfilter_save sv) {
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
    const int n_var = v.n_state - T::n_output - n_special<T>();
    auto rng = load_rng(v.rng, v.stride, k, v.deterministic);
    typename T::internal_state internal{};
    double y[T::n_state_max];
    load_state<T>(v, k, y);
    dopri5::state<NV> st;
    dopri5::scratch<NV> s;
    load_ode<NV>(o, k, n_var, st);
    dopri5::solver<T, NV> sol{ctl, shared, internal, n_var, k};
    sol.n_special = n_special<T>();
    if (requires_init[g]) {
      sol.initialise(time0, y, st, s);
    }
    double t = time0;
    double acc = 0;
    int update_err = 0;
    for (int i = 0; i < n_times; ++i) {
      const double t_end = times[i];
      if (st.err == 0 && update_err == 0) {
        update_err = advance<T, NV>(sol, t, t_end, dt, y, zero, st, s, rng,
                                    shared, internal);
      }
      t = t_end;
      const auto& d = data[static_cast<long>(i) * n_groups_data +
                           (n_groups_data == 1 ? 0 : g)];
      acc += T::compare_data(t_end, y, d, shared, internal, rng);
      if (sv.traj != nullptr || sv.snap != nullptr) {
        // the saved state is the system's state() at this time, with its
        // outputs recomputed (continuous/system.hpp:206-209)
        double z[T::n_state_max];
        for (int s = 0; s < v.n_state; ++s) {
          z[s] = y[s];
        }
        refresh_output<T>(t_end, z, shared, internal);
        save_data_time(sv, i, z, v.n_state, v.stride, k);
      }
    }
    refresh_output<T>(t, y, shared, internal);
    store_state<T>(v, k, y);
    store_ode<NV>(o, k, n_var, st);
    ll[k] = acc;
    if (st.err != 0 || update_err != 0) {
      rng.err = st.err != 0 ? st.err : update_err;
    }
    capture_error(v.errors, v.any_error, k, rng);
  }
}

// The adjoint run (unfilter.hpp:77-110 with the forward pass of
// discrete/system.hpp:95-117, 425-451, and compute_gradient_,
// unfilter.hpp:188-229 with :290-382 and :453-482), one thread per
// particle: the forward pass writes the state after every step to `hist`
// ([step][entry][particle]; before any zero_every reset, which acts on a
// working copy), compares each data time's saved state (at the system
// time the whole forward run ends on, as the reference's compare_data
// reads it), then walks back: adjoint_compare_data at each data time,
// adjoint_update over the steps to the previous one (zeroing the adjoint
// of zero_every entries after each step back), adjoint_initial at the
// start.  `obs_step_index[i]`: the step of data time i from the start.
template <typename T>
DUST2_PARTICLE_KERNEL(T) k_unfilter_adjoint(
    system_view<T> v, const int* active, const int* obs_step_index,
    int n_times, int n_steps_total, double time_start, double time_end,
    const double* times, double dt, const typename T::data_type* data,
    int n_groups_data, double* hist, double* ll, double* gradient,
    int n_gradient, unfilter_save sv) {
  if constexpr (has_adjoint<T>::value && has_compare_data<T>::value) {
    constexpr int NA = T::n_adjoint_max;
    const tile tl = v.tiles[blockIdx.x];
    if (static_cast<int>(threadIdx.x) >= tl.count) {
      return;
    }
    const int k = tl.start + threadIdx.x;
    const int g = group_of(v, tl, k);
    if (!active[g]) {
      return;
    }
    const auto& shared = v.shared[g];
    const zero_every_spec& zero = v.zero_every[g];
    const int ns = v.n_state;
    const long stride = v.stride;
    auto hist_at = [&](int step, int s) -> double& {
      return hist[(static_cast<long>(step) * ns + s) * stride + k];
    };
    auto rng = load_rng(v.rng, v.stride, k, v.deterministic);
    typename T::internal_state internal{};
    double x[T::n_state_max];
    double y[T::n_state_max];
    load_state<T>(v, k, x);
    for (int s = 0; s < ns; ++s) {
      hist_at(0, s) = x[s];
    }
    for (int step = 0; step < n_steps_total; ++step) {
      const double t = time_start + static_cast<double>(step) * dt;
      apply_zero_every<T>(zero, nullptr, step, t, x);
      T::update(t, dt, x, shared, internal, rng, y);
      for (int s = 0; s < ns; ++s) {
        hist_at(step + 1, s) = y[s];
        x[s] = y[s];
      }
    }
    double acc = 0;
    for (int i = 0; i < n_times; ++i) {
      for (int s = 0; s < ns; ++s) {
        y[s] = hist_at(obs_step_index[i], s);
      }
      const auto& d = data[static_cast<long>(i) * n_groups_data +
                           (n_groups_data == 1 ? 0 : g)];
      acc += T::compare_data(time_end, y, d, shared, internal, rng);
      save_data_time(sv, i, y, ns, stride, k);
    }
    double adj[NA];
    double adj_next[NA];
    for (int a = 0; a < NA; ++a) {
      adj[a] = 0;
    }
    double time = time_end;
    for (int i = n_times - 1; i >= 0; --i) {
      const double time_i = i == 0 ? time_start : times[i - 1];
      const int j = obs_step_index[i];
      for (int s = 0; s < ns; ++s) {
        y[s] = hist_at(j, s);
      }
      const auto& d = data[static_cast<long>(i) * n_groups_data +
                           (n_groups_data == 1 ? 0 : g)];
      T::adjoint_compare_data(time, y, adj, d, shared, internal, adj_next);
      for (int a = 0; a < NA; ++a) {
        adj[a] = adj_next[a];
      }
      // never more than the steps saved before this data time (rounding
      // is monotone, so this bound holds already; it keeps every read of
      // the history inside the buffer whatever the times)
      const int n_back = min(j, static_cast<int>(
        ::round(::fmax(0.0, time - time_i) / dt)));
      for (int b = 1; b <= n_back; ++b) {
        const double time_b = time - static_cast<double>(b) * dt;
        for (int s = 0; s < ns; ++s) {
          y[s] = hist_at(j - b, s);
        }
        T::adjoint_update(time_b, dt, y, adj, shared, internal, adj_next);
        for (int a = 0; a < NA; ++a) {
          adj[a] = adj_next[a];
        }
        for (int e = 0; e < zero.n; ++e) {
          if (fmod(time_b, zero.period[e]) == 0) {
            for (int s = 0; s < ns; ++s) {
              if (zero.has(e, s)) {
                adj[s] = 0;
              }
            }
          }
        }
      }
      time = time_i;
    }
    for (int s = 0; s < ns; ++s) {
      y[s] = hist_at(0, s);
    }
    T::adjoint_initial(time, y, adj, shared, internal, adj_next);
    store_state<T>(v, k, x);
    ll[k] = acc;
    for (int a = 0; a < n_gradient; ++a) {
      gradient[static_cast<long>(k) * n_gradient + a] = adj_next[ns + a];
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
    adjoint_current_ = false;
    S.set_time(time_start_);
    if (initial != nullptr) {
      S.put_state(initial);
    } else {
      S.set_state_initial();
    }
    auto& base = base_of(S);
    auto s = base.stream();
    const unfilter_save sv = prepare_save();
    DUST2_CUDA(cudaMemcpyAsync(active_.data(), active.data(),
                               G * sizeof(int), cudaMemcpyHostToDevice, s));
    DUST2_CUDA(cudaMemsetAsync(ll_.data(), 0, ll_.size() * sizeof(double),
                               s));
    base.reset_errors();
    const auto& L = base.layout();
    if constexpr (is_continuous<T>()) {
      S.launch_unfilter(times_dev_.data(), n_times(), active_.data(),
                        data_.data(), n_groups_data_, ll_.data(),
                        k_unfilter_ode<T>, sv);
      base.check_errors_after();
      base.set_time(times_.back());
    } else {
      k_unfilter_discrete<T><<<S.n_run_tiles(), L.tile_size, 0, s>>>(
        S.run_view(), active_.data(), sched_.data(), n_times(), S.dt(),
        data_.data(), n_groups_data_, ll_.data(), sv);
      DUST2_CUDA(cudaGetLastError());
      S.check_errors_after();
      S.set_time(t_end_);
    }
    copy_ll(index_group, n_index_group, ll_out);
    mark_saved(index_group, n_index_group);
  }

  int n_gradient() const override {
    if constexpr (has_adjoint<T>::value) {
      int n = 0;
      for (const auto& e : T::packing_gradient(shared0())) {
        int len = 1;
        for (int d : e.dims) {
          len *= d;
        }
        n += len;
      }
      return n;
    } else {
      return 0;
    }
  }

  // unfilter.hpp:77-110: the same log-likelihood as run(), through the
  // state history, with the gradient computed in the same kernel (the
  // reference computes it on first request, compute_gradient_,
  // :188-229).  A system without adjoint support runs as run() and has
  // no current gradient, as the reference's history-only run.
  void run_adjoint(const double* initial, const int* index_group,
                   int n_index_group, double* ll_out) override {
    if constexpr (!has_adjoint<T>::value || is_continuous<T>()) {
      run(initial, index_group, n_index_group, ll_out);
    } else {
      auto& S = *sys_;
      const int G = S.n_groups();
      std::vector<int> active(G, index_group == nullptr ? 1 : 0);
      if (index_group != nullptr) {
        for (int i = 0; i < n_index_group; ++i) {
          active[index_group[i]] = 1;
        }
      }
      adjoint_current_ = false;
      S.set_time(time_start_);
      if (initial != nullptr) {
        S.put_state(initial);
      } else {
        S.set_state_initial();
      }
      // The step of each data time from the start (adjoint_data.hpp:28-45
      // offsets); the forward pass is one run over all of them
      // (discrete/system.hpp:95-117), so step times are
      // time_start + i * dt throughout.
      const double dt = S.dt();
      std::vector<int> step_index;
      for (double ti : times_) {
        step_index.push_back(static_cast<int>(
          std::round(std::max(0.0, ti - time_start_) / dt)));
      }
      const int n_steps = static_cast<int>(
        std::round(std::max(0.0, times_.back() - time_start_) / dt));
      const double time_end = time_start_ + n_steps * dt;
      const auto& L = S.layout();
      const std::size_t need = static_cast<std::size_t>(n_steps + 1) *
        S.n_state() * L.stride;
      if (hist_.size() < need) {
        hist_.resize(need);
      }
      const int ng = n_gradient();
      if (gradient_.size() < static_cast<std::size_t>(L.n_total) * ng) {
        gradient_.resize(static_cast<std::size_t>(L.n_total) * ng);
      }
      if (step_index_.size() < step_index.size()) {
        step_index_.resize(step_index.size());
      }
      auto s = S.stream();
      const unfilter_save sv = prepare_save();
      DUST2_CUDA(cudaMemcpyAsync(step_index_.data(), step_index.data(),
                                 step_index.size() * sizeof(int),
                                 cudaMemcpyHostToDevice, s));
      DUST2_CUDA(cudaMemcpyAsync(active_.data(), active.data(),
                                 G * sizeof(int), cudaMemcpyHostToDevice, s));
      DUST2_CUDA(cudaMemsetAsync(ll_.data(), 0, ll_.size() * sizeof(double),
                                 s));
      S.reset_errors();
      k_unfilter_adjoint<T><<<S.n_run_tiles(), L.tile_size, 0, s>>>(
        S.run_view(), active_.data(), step_index_.data(), n_times(),
        n_steps, time_start_, time_end, times_dev_.data(), dt, data_.data(),
        n_groups_data_, hist_.data(), ll_.data(), gradient_.data(), ng,
        sv);
      DUST2_CUDA(cudaGetLastError());
      S.check_errors_after();
      S.set_time(time_end);
      copy_ll(index_group, n_index_group, ll_out);
      mark_saved(index_group, n_index_group);
      last_groups_.clear();
      if (index_group == nullptr) {
        for (int g = 0; g < G; ++g) {
          last_groups_.push_back(g);
        }
      } else {
        last_groups_.assign(index_group, index_group + n_index_group);
      }
      adjoint_current_ = true;
    }
  }

  // unfilter.hpp:135-142 with r/unfilter.hpp:154-180: n_gradient values
  // per particle of each group of the last adjoint run.
  void last_gradient(double* out) override {
    if (!adjoint_current_) {
      throw std::runtime_error("System was not run with 'adjoint = TRUE'");
    }
    const auto& L = base_of(*sys_).layout();
    const int ng = n_gradient();
    std::vector<double> gr(static_cast<std::size_t>(L.n_total) * ng);
    DUST2_CUDA(cudaMemcpy(gr.data(), gradient_.data(),
                          gr.size() * sizeof(double),
                          cudaMemcpyDeviceToHost));
    std::size_t pos = 0;
    for (int g : last_groups_) {
      for (int j = 0; j < L.n_particles[g]; ++j) {
        const std::size_t k = L.offset[g] + j;
        for (int a = 0; a < ng; ++a) {
          out[pos++] = gr[k * ng + a];
        }
      }
    }
  }

  int n_last_gradient_groups() const override {
    return adjoint_current_ ? static_cast<int>(last_groups_.size()) : 0;
  }

  void set_save_trajectories(bool save, const int* index_state,
                             int n_index_state) override {
    save_traj_ = save;
    traj_index_.clear();
    if (index_state == nullptr) {
      for (int s = 0; s < sys_->n_state(); ++s) {
        traj_index_.push_back(s);
      }
    } else {
      traj_index_.assign(index_state, index_state + n_index_state);
    }
  }

  void set_save_snapshots(const int* obs, int n_obs) override {
    snap_obs_.assign(obs, obs + n_obs);
  }

  bool trajectories_current() const override {
    return traj_current_;
  }
  bool snapshots_current() const override {
    return snap_current_;
  }
  int n_trajectory_state() const override {
    return traj_saved_n_;
  }
  int n_snapshots() const override {
    return snap_saved_n_;
  }
  const std::vector<int>& saved_groups() const override {
    return saved_groups_;
  }

  // r/unfilter.hpp:64-93 (export_state without reordering)
  void last_trajectories(double* out) override {
    if (!traj_current_) {
      throw std::runtime_error("Trajectories are not current");
    }
    export_saved(traj_.data(), nullptr, n_times(), traj_saved_n_, out);
  }

  // r/unfilter.hpp:95-125 (export_snapshots without reordering)
  void last_snapshots(double* out) override {
    if (!snap_current_) {
      throw std::runtime_error("Snapshots are not current");
    }
    export_saved(snap_.data(), snap_obs_dev_.data(), snap_saved_n_,
                 sys_->n_state(), out);
  }

private:
  // Buffers and device copies of the saving set-up for the next run.
  unfilter_save prepare_save() {
    traj_current_ = false;
    snap_current_ = false;
    unfilter_save sv;
    const auto& L = base_of(*sys_).layout();
    const int ns = sys_->n_state();
    if (save_traj_) {
      const std::size_t need = static_cast<std::size_t>(n_times()) *
        traj_index_.size() * L.stride;
      if (traj_.size() < need) {
        traj_.resize(need);
      }
      traj_index_dev_.resize(std::max<std::size_t>(1, traj_index_.size()));
      DUST2_CUDA(cudaMemcpy(traj_index_dev_.data(), traj_index_.data(),
                            traj_index_.size() * sizeof(int),
                            cudaMemcpyHostToDevice));
      sv.index = traj_index_dev_.data();
      sv.n_save = static_cast<int>(traj_index_.size());
      sv.traj = traj_.data();
    }
    if (!snap_obs_.empty()) {
      const std::size_t need = snap_obs_.size() * ns * L.stride;
      if (snap_.size() < need) {
        snap_.resize(need);
      }
      std::vector<int> slot(n_times(), -1);
      for (std::size_t i = 0; i < snap_obs_.size(); ++i) {
        slot[snap_obs_[i]] = static_cast<int>(i);
      }
      snap_slot_dev_.resize(slot.size());
      DUST2_CUDA(cudaMemcpy(snap_slot_dev_.data(), slot.data(),
                            slot.size() * sizeof(int),
                            cudaMemcpyHostToDevice));
      snap_obs_dev_.resize(snap_obs_.size());
      DUST2_CUDA(cudaMemcpy(snap_obs_dev_.data(), snap_obs_.data(),
                            snap_obs_.size() * sizeof(int),
                            cudaMemcpyHostToDevice));
      sv.snap_slot = snap_slot_dev_.data();
      sv.snap = snap_.data();
    }
    return sv;
  }

  void mark_saved(const int* index_group, int n_index_group) {
    saved_groups_.clear();
    if (index_group == nullptr) {
      for (int g = 0; g < sys_->n_groups(); ++g) {
        saved_groups_.push_back(g);
      }
    } else {
      saved_groups_.assign(index_group, index_group + n_index_group);
    }
    traj_current_ = save_traj_;
    traj_saved_n_ = static_cast<int>(traj_index_.size());
    snap_current_ = !snap_obs_.empty();
    snap_saved_n_ = static_cast<int>(snap_obs_.size());
  }

  // Gathers [time][entry][particle] (traj) or [snapshot][state][particle]
  // (snap, at the data times snap_obs) into [time][group][particle][entry]
  // for the saved groups.
  void export_saved(const double* src, const int* snap_obs, int n_t,
                    int n_entry, double* out) {
    const auto& L = base_of(*sys_).layout();
    const int np = L.n_particles[saved_groups_[0]];
    for (int g : saved_groups_) {
      if (L.n_particles[g] != np) {
        throw std::runtime_error(
          "Trajectories need equal particle counts in every group");
      }
    }
    const int ng = static_cast<int>(saved_groups_.size());
    device_array<int> offset(L.offset.size());
    device_array<int> groups(ng);
    device_array<double> dst(static_cast<std::size_t>(n_t) * ng * np *
                             n_entry);
    DUST2_CUDA(cudaMemcpy(offset.data(), L.offset.data(),
                          L.offset.size() * sizeof(int),
                          cudaMemcpyHostToDevice));
    DUST2_CUDA(cudaMemcpy(groups.data(), saved_groups_.data(),
                          ng * sizeof(int), cudaMemcpyHostToDevice));
    const int n_threads = ng * np;
    if (snap_obs == nullptr) {
      k_export_history<<<(n_threads + 127) / 128, 128>>>(
        src, nullptr, n_t, n_entry, L.stride, offset.data(), groups.data(),
        ng, nullptr, np, dst.data());
    } else {
      k_export_snapshots<<<(n_threads + 127) / 128, 128>>>(
        src, nullptr, n_times(), snap_obs, n_t, n_entry, L.stride,
        offset.data(), groups.data(), ng, nullptr, np, dst.data());
    }
    DUST2_CUDA(cudaGetLastError());
    DUST2_CUDA(cudaMemcpy(out, dst.data(), dst.size() * sizeof(double),
                          cudaMemcpyDeviceToHost));
  }

  void copy_ll(const int* index_group, int n_index_group, double* ll_out) {
    const auto& L = base_of(*sys_).layout();
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
      for (int g = 0; g < sys_->n_groups(); ++g) {
        copy_group(g);
      }
    } else {
      for (int i = 0; i < n_index_group; ++i) {
        copy_group(index_group[i]);
      }
    }
  }

  const typename T::shared_state& shared0() const {
    return base_of(*sys_).shared_host()[0];
  }

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
  device_array<double> hist_;
  device_array<double> gradient_;
  device_array<int> step_index_;
  std::vector<int> last_groups_;
  bool adjoint_current_ = false;
  bool save_traj_ = false;
  std::vector<int> traj_index_;
  std::vector<int> snap_obs_;
  device_array<double> traj_;
  device_array<double> snap_;
  device_array<int> traj_index_dev_;
  device_array<int> snap_slot_dev_;
  device_array<int> snap_obs_dev_;
  bool traj_current_ = false;
  bool snap_current_ = false;
  int traj_saved_n_ = 0;
  int snap_saved_n_ = 0;
  std::vector<int> saved_groups_;
};

}  // namespace engine
}  // namespace dust2gpu
