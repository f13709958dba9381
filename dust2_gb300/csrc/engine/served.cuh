// Likelihood server: continuous batching of particle-filter runs from many
// independent callers (MCMC chains) onto one device.
//
// dust2 evaluates one likelihood per call: `dust_likelihood_run` runs the
// bootstrap filter of one object (filter.hpp:42-104) to the end of its
// data, and an MCMC sampler calls it once per proposal
// (R/monty.R:90-317).  Many chains therefore mean many small, serial
// filter runs.  The server keeps every chain's filter resident in one
// device pool and advances all running requests together, one observation
// per "tick":
//
//   session   one chain's likelihood: a parameter group with its own
//             particle count, data, schedule and generator streams (the
//             stream layout of a one-group dust2 filter, r/discrete/
//             filter.hpp:63-75: 2 filter streams then the particles').
//             Its particle range, generator state and last state stay on
//             the device between requests.
//   request   one likelihood evaluation of a session at new parameters
//             (dust_likelihood_run after update_pars): initial state, then
//             every observation of the session's data.
//   tick      one observation for every running request: step+compare
//             (per-session time and data row), weights, log-sum-exp,
//             resample, reorder: the kernels of the plain filter, over the
//             tiles of all resident sessions, skipping idle ones.
//
// Requests start at the next tick after they arrive, as long as their
// session is resident and idle; sessions become resident when a slot and
// memory are free under the HBM budget given at creation (first come,
// first served; a session that does not fit waits).  Each request's
// arithmetic is that of a plain run of its session on its own, so its
// result is the same alone or in any mix.
//
// Host side: one server thread owns the device work; callers submit and
// wait through a mutex-protected queue.  At most TICKS_IN_FLIGHT ticks are
// enqueued ahead of the device; results (log-likelihood and error flag per
// slot) come back through pinned buffers per tick.
#pragma once

#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <chrono>
#include <cmath>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <stdexcept>
#include <string>
#include <thread>
#include <vector>

#include "api.hpp"
#include "device.cuh"
#include "discrete.cuh"
#include "filter.cuh"
#include "kernels_common.cuh"
#include "server_api.hpp"

namespace dust2gpu {
namespace engine {

// Static description of a resident session (device copy).
struct served_slot {
  int sched_offset;  // first row of its schedule in the schedule pool
  int data_offset;   // first row of its data in the data pool
  int n_obs;
  int pad;
  double dt;
};

// Slots starting a request at this tick (passed by value).
constexpr int SERVED_START_BATCH = 64;
struct served_start_list {
  int n;
  int slot[SERVED_START_BATCH];
};

__global__ void k_served_begin(served_start_list list, filter_view f,
                               int* active, int* obs, int* starting,
                               int* slot_error);
__global__ void k_served_advance(int* active, const served_slot* slots,
                                 int* obs, int* starting, int n_slots);
__global__ void k_reorder_active(const double* __restrict__ src,
                                 double* __restrict__ dst, int stride,
                                 int n_state, const tile* __restrict__ tiles,
                                 const int* __restrict__ active,
                                 const int* __restrict__ group_offset,
                                 const int* __restrict__ index,
                                 const int* __restrict__ group_mode);
__global__ void k_fallback_count(filter_view f, int* count);

// Initial state of the slots starting a request (filter.hpp:168-172),
// at the session's start time; clears their particle error records.
template <typename T>
DUST2_PARTICLE_KERNEL(T) k_served_initial(system_view<T> v,
                                          const int* starting,
                                 const served_slot* slots,
                                 const obs_step* sched, int* slot_error) {
  __shared__ shared_smem<T> sm;
  const tile tl = v.tiles[blockIdx.x];
  if (!starting[tl.group]) {
    return;
  }
  sm.load(v, tl.group);
  __syncthreads();
  if (static_cast<int>(threadIdx.x) >= tl.count) {
    return;
  }
  const int k = tl.start + threadIdx.x;
  const double time = sched[slots[tl.group].sched_offset].t0;
  v.errors[k] = particle_error{};
  auto rng = load_rng(v.rng, v.stride, k, v.deterministic);
  typename T::internal_state internal{};
  double x[T::n_state_max];
  load_state<T>(v, k, x);
  T::initial(time, sm.shared(), internal, rng, x);
  store_state<T>(v, k, x);
  store_rng(v.rng, v.stride, k, rng);
  capture_error(v.errors, slot_error + tl.group, k, rng);
}

// One observation of every running request: the plain filter's
// step_compare_tile with the session's own interval and data row.
template <typename T>
DUST2_PARTICLE_KERNEL(T) k_served_step_compare(system_view<T> v,
                                               filter_view f,
                                      const served_slot* slots,
                                      const int* obs, const obs_step* sched,
                                      const typename T::data_type* data,
                                      int* slot_error) {
  __shared__ shared_smem<T> sm;
  __shared__ double red[33];
  const tile tl = v.tiles[blockIdx.x];
  const int g = tl.group;
  if (!f.active[g]) {
    return;
  }
  const served_slot sl = slots[g];
  const int o = obs[g];
  const obs_step st = sched[sl.sched_offset + o];
  system_view<T> vs = v;
  vs.any_error = slot_error + g;
  step_compare_tile<T>(vs, f, tl, sm, red, st.t0, sl.dt, st.n_steps,
                       st.t_compare, data + sl.data_offset + o);
}

// First-fit allocator of [0, capacity) in units, with coalescing.
class interval_pool {
public:
  explicit interval_pool(long capacity = 0) : capacity_(capacity) {
    if (capacity > 0) {
      free_[0] = capacity;
    }
  }
  // Start of a free run of n units, or -1.
  long take(long n) {
    for (auto it = free_.begin(); it != free_.end(); ++it) {
      if (it->second >= n) {
        const long start = it->first;
        const long rest = it->second - n;
        free_.erase(it);
        if (rest > 0) {
          free_[start + n] = rest;
        }
        return start;
      }
    }
    return -1;
  }
  void give(long start, long n) {
    auto next = free_.lower_bound(start);
    if (next != free_.end() && next->first == start + n) {
      n += next->second;
      next = free_.erase(next);
    }
    if (next != free_.begin()) {
      auto prev = std::prev(next);
      if (prev->first + prev->second == start) {
        prev->second += n;
        return;
      }
    }
    free_[start] = n;
  }
  long capacity() const {
    return capacity_;
  }

private:
  long capacity_;
  std::map<long, long> free_;
};

// Staging of host -> device copies through pinned memory: each copy takes
// a region of a ring, and a region is reused only after the event recorded
// behind its copy has completed.
class pinned_ring {
public:
  pinned_ring() = default;
  pinned_ring(const pinned_ring&) = delete;
  pinned_ring& operator=(const pinned_ring&) = delete;
  ~pinned_ring() {
    for (auto& r : pending_) {
      cudaEventSynchronize(r.event);
      cudaEventDestroy(r.event);
    }
    for (auto e : spare_) {
      cudaEventDestroy(e);
    }
    if (base_ != nullptr) {
      cudaFreeHost(base_);
    }
  }
  void init(std::size_t bytes) {
    DUST2_CUDA(cudaMallocHost(reinterpret_cast<void**>(&base_), bytes));
    size_ = bytes;
  }
  // Copy n bytes from src to the device address dst on stream s.
  void upload(void* dst, const void* src, std::size_t n, cudaStream_t s) {
    if (n == 0) {
      return;
    }
    const std::size_t need = (n + 255) & ~static_cast<std::size_t>(255);
    if (need > size_) {
      // larger than the ring: copy through a temporary pinned buffer
      void* tmp = nullptr;
      DUST2_CUDA(cudaMallocHost(&tmp, n));
      std::memcpy(tmp, src, n);
      DUST2_CUDA(cudaMemcpyAsync(dst, tmp, n, cudaMemcpyHostToDevice, s));
      DUST2_CUDA(cudaStreamSynchronize(s));
      DUST2_CUDA(cudaFreeHost(tmp));
      return;
    }
    if (head_ + need > size_) {
      head_ = 0;
    }
    // wait until no pending copy overlaps [head_, head_ + need); copies
    // complete in stream order, so the oldest is waited for first
    auto overlaps = [this, need](const region& r) {
      return r.start < head_ + need && head_ < r.start + r.len;
    };
    while (std::any_of(pending_.begin(), pending_.end(), overlaps)) {
      DUST2_CUDA(cudaEventSynchronize(pending_.front().event));
      spare_.push_back(pending_.front().event);
      pending_.pop_front();
    }
    unsigned char* p = base_ + head_;
    std::memcpy(p, src, n);
    DUST2_CUDA(cudaMemcpyAsync(dst, p, n, cudaMemcpyHostToDevice, s));
    cudaEvent_t e;
    if (spare_.empty()) {
      DUST2_CUDA(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
    } else {
      e = spare_.back();
      spare_.pop_back();
    }
    DUST2_CUDA(cudaEventRecord(e, s));
    pending_.push_back(region{head_, need, e});
    head_ += need;
  }

private:
  struct region {
    std::size_t start;
    std::size_t len;
    cudaEvent_t event;
  };
  unsigned char* base_ = nullptr;
  std::size_t size_ = 0;
  std::size_t head_ = 0;
  std::deque<region> pending_;
  std::vector<cudaEvent_t> spare_;
};

template <typename T>
class served_engine : public server_api {
public:
  using shared_state = typename T::shared_state;
  using data_type = typename T::data_type;
  static constexpr int TICKS_IN_FLIGHT = 2;
  static constexpr int ALIGN = 32;  // particle ranges start on a warp

  // State storage is n_state_max wide, so sessions of systems whose
  // state length depends on parameters can share the pool.
  served_engine(double hbm_budget_bytes, int max_sessions) :
    n_state_(T::n_state_max), tile_size_(default_tile_size<T>()),
    n_slots_(max_sessions) {
    if (max_sessions < 1) {
      throw std::runtime_error("'max_sessions' must be at least 1");
    }
    if (!(hbm_budget_bytes > 0)) {
      throw std::runtime_error("The HBM budget must be positive");
    }
    DUST2_CUDA(cudaGetDevice(&device_));
    // memory plan: 1/16 of the budget for data and schedules, the rest
    // for particles
    const double per_obs = sizeof(data_type) + sizeof(obs_step);
    long n_obs_cap = static_cast<long>(hbm_budget_bytes / 16 / per_obs);
    n_obs_cap = std::max(1024L, std::min(n_obs_cap, 1L << 26));
    const double slot_bytes = static_cast<double>(n_slots_) *
      (sizeof(shared_state) + sizeof(zero_every_spec) + 256);
    double left = hbm_budget_bytes - n_obs_cap * per_obs - slot_bytes;
    long n_cap = static_cast<long>(left / bytes_per_particle());
    n_cap = std::min(n_cap, 1L << 29) / ALIGN * ALIGN;
    if (n_cap < ALIGN) {
      throw std::runtime_error("The HBM budget is too small for one session");
    }
    cap_particles_ = static_cast<int>(n_cap);
    cap_obs_ = static_cast<int>(n_obs_cap);
    particles_ = interval_pool(cap_particles_);
    obs_pool_ = interval_pool(cap_obs_);
    for (int s = n_slots_ - 1; s >= 0; --s) {
      free_slots_.push_back(s);
    }
    max_tiles_ = cap_particles_ / ALIGN + n_slots_;

    DUST2_CUDA(cudaStreamCreateWithFlags(&stream_, cudaStreamNonBlocking));
    const std::size_t P = cap_particles_;
    const std::size_t S = n_slots_;
    state_.resize(static_cast<std::size_t>(n_state_) * P);
    state_other_.resize(static_cast<std::size_t>(n_state_) * P);
    rng_.resize(4 * P);
    w_.resize(P);
    ew_.resize(P);
    pre_.resize(P);
    idx_.resize(P);
    errors_.resize(P);
    tiles_.resize(max_tiles_);
    // chunks of 32 particles: the pool's 32-aligned ranges hold at most
    // capacity / 32 of them
    chunk_sum_.resize(cap_particles_ / ALIGN + n_slots_);
    chunk_off_.resize(cap_particles_ / ALIGN + n_slots_);
    shared_dev_.resize(S);
    zero_dev_.resize(S);
    slots_dev_.resize(S);
    obs_dev_.resize(S);
    starting_.resize(S);
    slot_error_.resize(S);
    active_.resize(S);
    n_part_.resize(S);
    offset_.resize(S);
    chunk_first_.resize(S);
    chunk_count_.resize(S);
    gkey_.resize(S);
    gnz_.resize(S);
    gflag_.resize(S);
    mode_.resize(S);
    ll_.resize(S);
    gu_.resize(S);
    guu0_.resize(S);
    gdu_.resize(S);
    gtot_.resize(S);
    frng_.resize(8 * S);
    fallback_count_.resize(S);
    scalars_.resize(2);  // set_initial (unused), force_serial
    sched_.resize(cap_obs_);
    data_.resize(cap_obs_);
    auto s = stream_;
    DUST2_CUDA(cudaMemsetAsync(state_.data(), 0, state_.size() * 8, s));
    DUST2_CUDA(cudaMemsetAsync(state_other_.data(), 0,
                               state_other_.size() * 8, s));
    DUST2_CUDA(cudaMemsetAsync(errors_.data(), 0,
                               errors_.size() * sizeof(particle_error), s));
    for (auto* p : {&starting_, &slot_error_, &active_, &n_part_, &offset_,
                    &chunk_first_, &chunk_count_, &gnz_, &gflag_, &mode_,
                    &obs_dev_, &fallback_count_, &scalars_}) {
      DUST2_CUDA(cudaMemsetAsync(p->data(), 0, p->size() * sizeof(int), s));
    }
    DUST2_CUDA(cudaMemsetAsync(slots_dev_.data(), 0,
                               S * sizeof(served_slot), s));
    ring_.init(64u << 20);
    for (int i = 0; i <= TICKS_IN_FLIGHT; ++i) {
      result_slot r;
      DUST2_CUDA(cudaMallocHost(reinterpret_cast<void**>(&r.ll),
                                S * sizeof(double)));
      DUST2_CUDA(cudaMallocHost(reinterpret_cast<void**>(&r.err),
                                S * sizeof(int)));
      DUST2_CUDA(cudaEventCreateWithFlags(&r.event,
                                          cudaEventDisableTiming));
      DUST2_CUDA(cudaEventCreate(&r.step0));
      DUST2_CUDA(cudaEventCreate(&r.step1));
      results_.push_back(r);
    }
    DUST2_CUDA(cudaStreamSynchronize(s));
    slot_session_.assign(S, -1);
    thread_ = std::thread([this] { loop(); });
  }

  ~served_engine() override {
    {
      std::lock_guard<std::mutex> lock(mu_);
      stop_ = true;
    }
    cv_.notify_all();
    if (thread_.joinable()) {
      thread_.join();
    }
    cudaStreamSynchronize(stream_);
    for (auto& r : results_) {
      cudaFreeHost(r.ll);
      cudaFreeHost(r.err);
      cudaEventDestroy(r.event);
      cudaEventDestroy(r.step0);
      cudaEventDestroy(r.step1);
    }
    cudaStreamDestroy(stream_);
  }

  std::size_t bytes_per_particle() const {
    return 2 * static_cast<std::size_t>(n_state_) * sizeof(double) +
      4 * sizeof(std::uint64_t) + 3 * sizeof(double) + sizeof(int) +
      sizeof(particle_error);
  }

  int n_pars() const override {
    return parameter_length<T>();
  }
  int n_data() const override {
    return static_cast<int>(sizeof(data_type) / sizeof(double));
  }
  int n_state() const override {
    return n_state_;
  }
  void capacity(std::size_t* n_particles, std::size_t* n_sessions,
                std::size_t* n_observations) const override {
    *n_particles = cap_particles_;
    *n_sessions = n_slots_;
    *n_observations = cap_obs_;
  }

  std::int64_t open_session(const double* pars, int n_particles,
                            double time_start, const double* times,
                            int n_times, const double* data, double dt,
                            std::vector<std::uint64_t> rng_words) override {
    if (n_particles < 1) {
      throw std::runtime_error("'n_particles' must be at least 1");
    }
    const long need = round_up(n_particles);
    if (need > cap_particles_ || n_times > cap_obs_) {
      throw std::runtime_error(
        "This session needs more device memory than the server's budget");
    }
    auto ss = std::make_unique<session>();
    ss->n = n_particles;
    ss->shared = T::build_shared(pars);
    ss->dt = dt;
    ss->time_start = time_start;
    double t = time_start;
    for (int i = 0; i < n_times; ++i) {
      const int n = static_cast<int>(
        std::round(std::max(0.0, times[i] - t) / dt));
      ss->sched.push_back(obs_step{t, n, t + n * dt});
      ss->steps_per_request += n;
      t = t + n * dt;
    }
    const int nd = n_data();
    for (int i = 0; i < n_times; ++i) {
      ss->data.push_back(build_data_of<T>(
        data + static_cast<std::size_t>(i) * nd, ss->shared));
    }
    ss->rng_words = std::move(rng_words);
    std::lock_guard<std::mutex> lock(mu_);
    const std::int64_t id = next_session_++;
    ss->id = id;
    admission_.push_back(id);
    sessions_[id] = std::move(ss);
    cv_.notify_all();
    return id;
  }

  std::int64_t submit(std::int64_t session_id, const double* pars) override {
    auto r = std::make_unique<request>();
    r->t_submit = now();
    std::lock_guard<std::mutex> lock(mu_);
    auto it = sessions_.find(session_id);
    if (it == sessions_.end() || it->second->closing) {
      throw std::runtime_error("Unknown or closed session");
    }
    session& ss = *it->second;
    r->session = session_id;
    if (pars != nullptr) {
      // update_pars semantics (r/filter.hpp:101-110): constants kept
      shared_state sh = ss.has_latest ? ss.shared_latest : ss.shared;
      T::update_shared(pars, sh);
      ss.shared_latest = sh;
      ss.has_latest = true;
    }
    r->shared = ss.has_latest ? ss.shared_latest : ss.shared;
    const std::int64_t id = next_request_++;
    r->id = id;
    ss.queue.push_back(id);
    requests_[id] = std::move(r);
    cv_.notify_all();
    return id;
  }

  int wait(std::int64_t ticket, double timeout, double* ll, double* latency,
           std::string* error) override {
    std::unique_lock<std::mutex> lock(mu_);
    auto it = requests_.find(ticket);
    if (it == requests_.end()) {
      throw std::runtime_error("Unknown request");
    }
    request* r = it->second.get();
    auto done = [r] { return r->status >= REQ_DONE; };
    if (timeout < 0) {
      done_cv_.wait(lock, done);
    } else if (!done_cv_.wait_for(lock, std::chrono::duration<double>(
                                    timeout), done)) {
      return 2;
    }
    if (server_error_.size() > 0 && r->status != REQ_DONE) {
      *error = server_error_;
    }
    *ll = r->ll;
    *latency = r->t_end - r->t_submit;
    const int status = r->status == REQ_DONE ? 0 : 1;
    if (status != 0 && error->empty()) {
      *error = r->error;
    }
    requests_.erase(it);
    return status;
  }

  void close_session(std::int64_t session_id) override {
    std::lock_guard<std::mutex> lock(mu_);
    auto it = sessions_.find(session_id);
    if (it == sessions_.end()) {
      throw std::runtime_error("Unknown session");
    }
    it->second->closing = true;
    cv_.notify_all();
  }

  void session_rng_state(std::int64_t session_id,
                         std::uint64_t* out) override {
    std::unique_lock<std::mutex> lock(mu_);
    auto it = sessions_.find(session_id);
    if (it == sessions_.end()) {
      throw std::runtime_error("Unknown session");
    }
    session* ss = it->second.get();
    done_cv_.wait(lock, [ss, this] {
      return !server_error_.empty() ||
        (ss->uploaded && ss->running < 0 && ss->queue.empty());
    });
    if (!server_error_.empty()) {
      throw std::runtime_error(server_error_);
    }
    // the session is idle: nothing in flight writes its streams, and its
    // uploads are complete once the stream has drained to this point
    DUST2_CUDA(cudaStreamSynchronize(stream_));
    const std::size_t P = cap_particles_;
    std::vector<std::uint64_t> f(8);
    DUST2_CUDA(cudaMemcpy(f.data(), frng_.data() + 8 * ss->slot,
                          8 * sizeof(std::uint64_t),
                          cudaMemcpyDeviceToHost));
    std::vector<std::uint64_t> p(4 * static_cast<std::size_t>(ss->n));
    for (int w = 0; w < 4; ++w) {
      DUST2_CUDA(cudaMemcpy(p.data() + static_cast<std::size_t>(w) * ss->n,
                            rng_.data() + w * P + ss->offset,
                            ss->n * sizeof(std::uint64_t),
                            cudaMemcpyDeviceToHost));
    }
    for (int w = 0; w < 8; ++w) {
      out[w] = f[w];
    }
    for (int k = 0; k < ss->n; ++k) {
      for (int w = 0; w < 4; ++w) {
        out[8 + 4 * static_cast<std::size_t>(k) + w] =
          p[static_cast<std::size_t>(w) * ss->n + k];
      }
    }
  }

  void set_timing(bool enable) override {
    std::lock_guard<std::mutex> lock(mu_);
    timing_ = enable;
    step_ms_ = 0;
    n_timed_ = 0;
  }

  void stats(double* out, int n) override {
    std::lock_guard<std::mutex> lock(mu_);
    const double v[] = {
      static_cast<double>(ticks_.load()), particle_steps_,
      static_cast<double>(requests_done_), static_cast<double>(resident_),
      static_cast<double>(admission_.size()), static_cast<double>(queued_),
      static_cast<double>(cap_particles_), static_cast<double>(used_particles_),
      static_cast<double>(max_running_.load()), step_ms_,
      static_cast<double>(n_timed_), static_cast<double>(launches_.load())};
    for (int i = 0; i < n && i < static_cast<int>(std::size(v)); ++i) {
      out[i] = v[i];
    }
  }

private:
  enum request_status { REQ_QUEUED = 0, REQ_RUNNING = 1, REQ_DONE = 2,
                        REQ_FAILED = 3 };

  struct request {
    std::int64_t id = -1;
    std::int64_t session = -1;
    shared_state shared;
    int status = REQ_QUEUED;
    double ll = NAN;
    double t_submit = 0, t_end = 0;
    std::string error;
  };

  struct session {
    std::int64_t id = -1;
    int n = 0;
    shared_state shared;
    shared_state shared_latest;
    bool has_latest = false;
    double dt = 1;
    double time_start = 0;
    std::vector<obs_step> sched;
    std::vector<data_type> data;
    std::vector<std::uint64_t> rng_words;
    long steps_per_request = 0;
    // residency
    int slot = -1;
    long offset = -1, alloc = 0;
    long obs_offset = -1;
    bool uploaded = false;
    bool closing = false;
    std::deque<std::int64_t> queue;
    std::int64_t running = -1;
  };

  struct result_slot {
    double* ll = nullptr;
    int* err = nullptr;
    cudaEvent_t event = nullptr;
    cudaEvent_t step0 = nullptr;  // around the step kernel, when timing
    cudaEvent_t step1 = nullptr;
  };

  struct tick_record {
    int ring;
    bool timed = false;
    std::vector<std::pair<int, std::int64_t>> finishing;  // slot, request
  };

  struct start_item {
    int slot;
    std::int64_t request;
    shared_state shared;
    long remaining;
  };

  static long round_up(long n) {
    return (n + ALIGN - 1) / ALIGN * ALIGN;
  }

  static double now() {
    return std::chrono::duration<double>(
      std::chrono::steady_clock::now().time_since_epoch()).count();
  }

  filter_view fview() {
    return filter_view{tiles_.data(), active_.data(), n_part_.data(),
                       offset_.data(), chunk_first_.data(),
                       chunk_count_.data(), w_.data(), ew_.data(), pre_.data(),
                       chunk_sum_.data(), chunk_off_.data(), gkey_.data(),
                       gnz_.data(),
                       gflag_.data(), mode_.data(), ll_.data(), gu_.data(),
                       guu0_.data(), gdu_.data(), gtot_.data(), idx_.data(),
                       frng_.data(), scalars_.data(), scalars_.data() + 1};
  }

  system_view<T> sview(double* state) {
    return system_view<T>{state, rng_.data(), shared_dev_.data(),
                          zero_dev_.data(), tiles_.data(), errors_.data(),
                          slot_error_.data(), cap_particles_, n_state_,
                          false};
  }

  // -- server thread --------------------------------------------------

  void loop() {
    try {
      DUST2_CUDA(cudaSetDevice(device_));
      loop_body();
    } catch (const std::exception& e) {
      std::lock_guard<std::mutex> lock(mu_);
      server_error_ = std::string("likelihood server stopped: ") + e.what();
      for (auto& el : requests_) {
        if (el.second->status < REQ_DONE) {
          el.second->status = REQ_FAILED;
          el.second->error = server_error_;
          el.second->t_end = now();
        }
      }
      done_cv_.notify_all();
    }
  }

  void loop_body() {
    std::vector<session*> admitted;
    std::vector<start_item> starts;
    for (;;) {
      retire(false);
      bool layout_changed = false;
      admitted.clear();
      starts.clear();
      {
        std::unique_lock<std::mutex> lock(mu_);
        if (stop_) {
          fail_queued("the likelihood server was shut down");
        }
        layout_changed = release_closed() || layout_changed;
        layout_changed = admit(&admitted) || layout_changed;
        collect_starts(&starts);
        const bool idle = running_.empty() && in_flight_.empty() &&
          starts.empty() && admitted.empty() && !layout_changed;
        if (idle) {
          if (stop_) {
            return;
          }
          cv_.wait(lock);
          continue;
        }
      }
      for (auto* ss : admitted) {
        upload_session(*ss);
      }
      if (!admitted.empty()) {
        std::lock_guard<std::mutex> lock(mu_);
        for (auto* ss : admitted) {
          ss->uploaded = true;
        }
        done_cv_.notify_all();
      }
      if (layout_changed) {
        rebuild_tiles();
      }
      begin(starts);
      if (!running_.empty()) {
        if (static_cast<int>(in_flight_.size()) >= TICKS_IN_FLIGHT) {
          retire(true);
        }
        tick();
      } else if (!in_flight_.empty()) {
        retire(true);
      }
    }
  }

  // On shutdown: requests that have not started fail (lock held).
  void fail_queued(const char* why) {
    const double t = now();
    for (auto& el : sessions_) {
      for (auto rid : el.second->queue) {
        request& r = *requests_.at(rid);
        r.status = REQ_FAILED;
        r.error = why;
        r.t_end = t;
      }
      el.second->queue.clear();
    }
    admission_.clear();
    done_cv_.notify_all();
  }

  // Free the resources of closed, idle sessions (lock held).
  bool release_closed() {
    bool changed = false;
    for (auto it = sessions_.begin(); it != sessions_.end();) {
      session& ss = *it->second;
      if (ss.closing && ss.running < 0 && ss.queue.empty()) {
        if (ss.slot >= 0) {
          particles_.give(ss.offset, ss.alloc);
          obs_pool_.give(ss.obs_offset, ss.sched.size());
          free_slots_.push_back(ss.slot);
          slot_session_[ss.slot] = -1;
          used_particles_ -= ss.alloc;
          resident_--;
          changed = true;
        } else {
          admission_.erase(std::remove(admission_.begin(), admission_.end(),
                                       ss.id), admission_.end());
        }
        it = sessions_.erase(it);
      } else {
        ++it;
      }
    }
    return changed;
  }

  // Make waiting sessions resident while slots and memory allow, in
  // order of arrival (lock held).
  bool admit(std::vector<session*>* admitted) {
    bool changed = false;
    for (auto it = admission_.begin(); it != admission_.end();) {
      session& ss = *sessions_.at(*it);
      if (free_slots_.empty()) {
        break;
      }
      const long need = round_up(ss.n);
      const long start = particles_.take(need);
      if (start < 0) {
        ++it;
        continue;
      }
      const long obs_start = obs_pool_.take(ss.sched.size());
      if (obs_start < 0) {
        particles_.give(start, need);
        ++it;
        continue;
      }
      ss.slot = free_slots_.back();
      free_slots_.pop_back();
      slot_session_[ss.slot] = ss.id;
      ss.offset = start;
      ss.alloc = need;
      ss.obs_offset = obs_start;
      used_particles_ += need;
      resident_++;
      admitted->push_back(&ss);
      changed = true;
      it = admission_.erase(it);
    }
    return changed;
  }

  // Requests that can start at the next tick (lock held).
  void collect_starts(std::vector<start_item>* starts) {
    queued_ = 0;
    for (auto& el : sessions_) {
      session& ss = *el.second;
      queued_ += ss.queue.size();
      if (ss.slot < 0 || ss.running >= 0 || ss.queue.empty()) {
        continue;
      }
      const std::int64_t rid = ss.queue.front();
      ss.queue.pop_front();
      request& r = *requests_.at(rid);
      r.status = REQ_RUNNING;
      ss.running = rid;
      starts->push_back(start_item{ss.slot, rid, r.shared,
                                   static_cast<long>(ss.sched.size())});
      particle_steps_ += static_cast<double>(ss.n) * ss.steps_per_request;
    }
  }

  // Device copies of a newly resident session: schedule, data, slot
  // description, generator streams (stream order puts them after every
  // tick already enqueued).
  void upload_session(session& ss) {
    auto s = stream_;
    const std::size_t P = cap_particles_;
    ring_.upload(sched_.data() + ss.obs_offset, ss.sched.data(),
                 ss.sched.size() * sizeof(obs_step), s);
    ring_.upload(data_.data() + ss.obs_offset, ss.data.data(),
                 ss.data.size() * sizeof(data_type), s);
    served_slot sl{static_cast<int>(ss.obs_offset),
                   static_cast<int>(ss.obs_offset),
                   static_cast<int>(ss.sched.size()), 0, ss.dt};
    ring_.upload(slots_dev_.data() + ss.slot, &sl, sizeof(sl), s);
    ring_.upload(frng_.data() + 8 * ss.slot, ss.rng_words.data(),
                 8 * sizeof(std::uint64_t), s);
    std::vector<std::uint64_t> soa(static_cast<std::size_t>(ss.n));
    for (int w = 0; w < 4; ++w) {
      for (int k = 0; k < ss.n; ++k) {
        soa[k] = ss.rng_words[8 + 4 * static_cast<std::size_t>(k) + w];
      }
      ring_.upload(rng_.data() + w * P + ss.offset, soa.data(),
                   soa.size() * sizeof(std::uint64_t), s);
    }
    auto z = T::zero_every(ss.shared);
    ring_.upload(zero_dev_.data() + ss.slot, &z, sizeof(z), s);
    ring_.upload(shared_dev_.data() + ss.slot, &ss.shared,
                 sizeof(shared_state), s);
    ss.rng_words.clear();
    ss.rng_words.shrink_to_fit();
  }

  // Tiles over every resident session, grouped by slot.
  void rebuild_tiles() {
    std::vector<tile> tiles;
    std::vector<int> np(n_slots_, 0), off(n_slots_, 0), cf(n_slots_, 0),
      cc(n_slots_, 0);
    int n_chunks = 0;
    {
      std::lock_guard<std::mutex> lock(mu_);
      for (int s = 0; s < n_slots_; ++s) {
        const std::int64_t id = slot_session_[s];
        if (id < 0) {
          continue;
        }
        const session& ss = *sessions_.at(id);
        np[s] = ss.n;
        off[s] = static_cast<int>(ss.offset);
        cf[s] = n_chunks;
        cc[s] = (ss.n + 31) / 32;
        n_chunks += cc[s];
        const int nt = (ss.n + tile_size_ - 1) / tile_size_;
        for (int t = 0; t < nt; ++t) {
          const int local = t * tile_size_;
          tiles.push_back(tile{s, static_cast<int>(ss.offset) + local,
                               std::min(tile_size_, ss.n - local), local});
        }
      }
    }
    if (static_cast<int>(tiles.size()) > max_tiles_) {
      throw std::runtime_error("tile table overflow");
    }
    n_tiles_ = static_cast<int>(tiles.size());
    auto s = stream_;
    ring_.upload(tiles_.data(), tiles.data(), tiles.size() * sizeof(tile), s);
    ring_.upload(n_part_.data(), np.data(), np.size() * sizeof(int), s);
    ring_.upload(offset_.data(), off.data(), off.size() * sizeof(int), s);
    ring_.upload(chunk_first_.data(), cf.data(), cf.size() * sizeof(int), s);
    ring_.upload(chunk_count_.data(), cc.data(), cc.size() * sizeof(int), s);
  }

  // Start requests: parameters, then reset of the slot's filter state
  // and its initial particle state.
  void begin(const std::vector<start_item>& starts) {
    if (starts.empty()) {
      return;
    }
    auto s = stream_;
    filter_view f = fview();
    for (std::size_t i = 0; i < starts.size(); i += SERVED_START_BATCH) {
      served_start_list list{};
      for (std::size_t j = i; j < starts.size() &&
             j < i + SERVED_START_BATCH; ++j) {
        const auto& st = starts[j];
        ring_.upload(shared_dev_.data() + st.slot, &st.shared,
                     sizeof(shared_state), s);
        auto z = T::zero_every(st.shared);
        ring_.upload(zero_dev_.data() + st.slot, &z, sizeof(z), s);
        list.slot[list.n++] = st.slot;
        running_[st.slot] = running_entry{st.request, st.remaining};
      }
      k_served_begin<<<1, SERVED_START_BATCH, 0, s>>>(
        list, f, active_.data(), obs_dev_.data(), starting_.data(),
        slot_error_.data());
      DUST2_CUDA(cudaGetLastError());
      launches_++;
    }
    max_running_ = std::max<long>(max_running_.load(),
                                  static_cast<long>(running_.size()));
    if (n_tiles_ > 0) {
      k_served_initial<T><<<n_tiles_, tile_size_, 0, s>>>(
        sview(cur()), starting_.data(), slots_dev_.data(), sched_.data(),
        slot_error_.data());
      DUST2_CUDA(cudaGetLastError());
      launches_++;
    }
  }

  double* cur() {
    return parity_ ? state_other_.data() : state_.data();
  }
  double* other() {
    return parity_ ? state_.data() : state_other_.data();
  }

  // One observation of every running request.
  void tick() {
    auto s = stream_;
    filter_view f = fview();
    const int NT = n_tiles_;
    const int TS = tile_size_;
    const int S = n_slots_;
    if (NT == 0) {
      throw std::runtime_error("no tiles for running requests");
    }
    bool timed;
    {
      std::lock_guard<std::mutex> lock(mu_);
      timed = timing_;
    }
    result_slot& r = results_[ring_pos_];
    if (timed) {
      DUST2_CUDA(cudaEventRecord(r.step0, s));
    }
    k_served_step_compare<T><<<NT, TS, 0, s>>>(
      sview(cur()), f, slots_dev_.data(), obs_dev_.data(), sched_.data(),
      data_.data(), slot_error_.data());
    if (timed) {
      DUST2_CUDA(cudaEventRecord(r.step1, s));
    }
    k_weights<<<NT, TS, 0, s>>>(f);
    k_group<<<S, 256, 0, s>>>(f, S);
    k_resample<<<NT, TS, 0, s>>>(f);
    k_fallback_count<<<S, FALLBACK_THREADS, 0, s>>>(f,
                                                    fallback_count_.data());
    k_reorder_active<<<NT, TS, 0, s>>>(cur(), other(), cap_particles_,
                                       n_state_, tiles_.data(),
                                       active_.data(), offset_.data(),
                                       idx_.data(), mode_.data());
    k_served_advance<<<n_blocks(S, 128), 128, 0, s>>>(
      active_.data(), slots_dev_.data(), obs_dev_.data(), starting_.data(),
      S);
    DUST2_CUDA(cudaGetLastError());
    parity_ = !parity_;
    launches_ += 7;
    tick_record rec;
    rec.ring = ring_pos_;
    rec.timed = timed;
    for (auto it = running_.begin(); it != running_.end();) {
      if (--it->second.remaining == 0) {
        rec.finishing.emplace_back(it->first, it->second.request);
        it = running_.erase(it);
      } else {
        ++it;
      }
    }
    if (!rec.finishing.empty()) {
      DUST2_CUDA(cudaMemcpyAsync(r.ll, ll_.data(), S * sizeof(double),
                                 cudaMemcpyDeviceToHost, s));
      DUST2_CUDA(cudaMemcpyAsync(r.err, slot_error_.data(), S * sizeof(int),
                                 cudaMemcpyDeviceToHost, s));
    }
    DUST2_CUDA(cudaEventRecord(r.event, s));
    ring_pos_ = (ring_pos_ + 1) % static_cast<int>(results_.size());
    in_flight_.push_back(std::move(rec));
    ticks_++;
  }

  // Complete the requests of finished ticks; blocking waits for the
  // oldest tick.
  void retire(bool blocking) {
    while (!in_flight_.empty()) {
      tick_record& rec = in_flight_.front();
      result_slot& r = results_[rec.ring];
      if (blocking) {
        DUST2_CUDA(cudaEventSynchronize(r.event));
        blocking = false;
      } else {
        const cudaError_t q = cudaEventQuery(r.event);
        if (q == cudaErrorNotReady) {
          return;
        }
        DUST2_CUDA(q);
      }
      if (rec.timed) {
        float ms = 0;
        DUST2_CUDA(cudaEventElapsedTime(&ms, r.step0, r.step1));
        std::lock_guard<std::mutex> lock(mu_);
        step_ms_ += ms;
        n_timed_++;
      }
      if (!rec.finishing.empty()) {
        std::vector<std::string> messages(rec.finishing.size());
        for (std::size_t i = 0; i < rec.finishing.size(); ++i) {
          const int slot = rec.finishing[i].first;
          if (r.err[slot]) {
            messages[i] = slot_error_text(slot);
          }
        }
        const double t = now();
        std::lock_guard<std::mutex> lock(mu_);
        for (std::size_t i = 0; i < rec.finishing.size(); ++i) {
          const int slot = rec.finishing[i].first;
          auto it = requests_.find(rec.finishing[i].second);
          if (it != requests_.end()) {
            request& q = *it->second;
            q.ll = r.ll[slot];
            q.t_end = t;
            if (r.err[slot]) {
              q.status = REQ_FAILED;
              q.error = messages[i];
            } else {
              q.status = REQ_DONE;
            }
            requests_done_++;
            auto sit = sessions_.find(q.session);
            if (sit != sessions_.end()) {
              sit->second->running = -1;
            }
          }
        }
        done_cv_.notify_all();
      }
      in_flight_.pop_front();
    }
  }

  // The error summary of one slot's particles (errors.hpp:29-54).
  std::string slot_error_text(int slot) {
    std::int64_t id;
    int n, offset;
    {
      std::lock_guard<std::mutex> lock(mu_);
      id = slot_session_[slot];
      const session& ss = *sessions_.at(id);
      n = ss.n;
      offset = static_cast<int>(ss.offset);
    }
    std::vector<particle_error> e(n);
    DUST2_CUDA(cudaMemcpy(e.data(), errors_.data() + offset,
                          n * sizeof(particle_error),
                          cudaMemcpyDeviceToHost));
    return format_errors(e);
  }

  struct running_entry {
    std::int64_t request;
    long remaining;
  };

  int device_ = 0;
  int n_state_;
  int tile_size_;
  int n_slots_;
  int cap_particles_ = 0;
  int cap_obs_ = 0;
  int max_tiles_ = 0;
  int n_tiles_ = 0;
  bool parity_ = false;
  cudaStream_t stream_ = nullptr;

  // device pool
  device_array<double> state_, state_other_;
  device_array<std::uint64_t> rng_;
  device_array<double> w_, ew_, pre_;
  device_array<int> idx_;
  device_array<particle_error> errors_;
  device_array<tile> tiles_;
  device_array<double> chunk_sum_, chunk_off_;
  device_array<shared_state> shared_dev_;
  device_array<zero_every_spec> zero_dev_;
  device_array<served_slot> slots_dev_;
  device_array<int> obs_dev_, starting_, slot_error_;
  device_array<int> active_, n_part_, offset_, chunk_first_, chunk_count_;
  device_array<unsigned long long> gkey_;
  device_array<int> gnz_, gflag_, mode_;
  device_array<double> ll_, gu_, guu0_, gdu_, gtot_;
  device_array<std::uint64_t> frng_;
  device_array<int> fallback_count_;
  device_array<int> scalars_;
  device_array<obs_step> sched_;
  device_array<data_type> data_;

  pinned_ring ring_;
  std::vector<result_slot> results_;
  int ring_pos_ = 0;
  std::deque<tick_record> in_flight_;
  std::map<int, running_entry> running_;  // slot -> request (server thread)

  // shared with callers (mu_)
  std::mutex mu_;
  std::condition_variable cv_;
  std::condition_variable done_cv_;
  bool stop_ = false;
  std::string server_error_;
  std::map<std::int64_t, std::unique_ptr<session>> sessions_;
  std::map<std::int64_t, std::unique_ptr<request>> requests_;
  std::deque<std::int64_t> admission_;
  std::vector<int> free_slots_;
  std::vector<std::int64_t> slot_session_;
  interval_pool particles_;
  interval_pool obs_pool_;
  std::int64_t next_session_ = 1;
  std::int64_t next_request_ = 1;
  std::atomic<long> ticks_{0};
  double particle_steps_ = 0;
  long requests_done_ = 0;
  long resident_ = 0;
  long queued_ = 0;
  long used_particles_ = 0;
  std::atomic<long> max_running_{0};
  bool timing_ = false;
  double step_ms_ = 0;
  long n_timed_ = 0;
  std::atomic<long> launches_{0};

  std::thread thread_;
};

}  // namespace engine
}  // namespace dust2gpu
