// Type-erased interface of the likelihood server (engine/served.cuh).
#pragma once

#include <cstddef>
#include <cstdint>
#include <string>
#include <vector>

namespace dust2gpu {
namespace engine {

class server_api {
public:
  virtual ~server_api() = default;
  virtual int n_pars() const = 0;
  virtual int n_data() const = 0;
  virtual int n_state() const = 0;
  virtual void capacity(std::size_t* n_particles, std::size_t* n_sessions,
                        std::size_t* n_observations) const = 0;
  // A session: one parameter group (pars, one row of the parameter
  // table), its particle count, data schedule (times, data rows of
  // n_data values) and the stream block of a one-group filter.
  virtual std::int64_t open_session(const double* pars, int n_particles,
                                    double time_start, const double* times,
                                    int n_times, const double* data,
                                    double dt,
                                    std::vector<std::uint64_t> rng_words) = 0;
  // Queue one likelihood evaluation; pars (one row, NaN = keep) update
  // the session's parameters first, as update_pars does; nullptr keeps
  // them.
  virtual std::int64_t submit(std::int64_t session, const double* pars) = 0;
  // 0: done (ll, latency set); 1: the request failed (error set);
  // 2: still pending after `timeout` seconds (negative: wait forever).
  virtual int wait(std::int64_t ticket, double timeout, double* ll,
                   double* latency, std::string* error) = 0;
  // Release the session once its queued requests have run.
  virtual void close_session(std::int64_t session) = 0;
  // Generator state of an idle session, in the layout of a one-group
  // filter (2 filter streams, then the particles').
  virtual void session_rng_state(std::int64_t session,
                                 std::uint64_t* out) = 0;
  // Record device time of every tick's step+compare kernel.
  virtual void set_timing(bool enable) = 0;
  virtual void stats(double* out, int n) = 0;
};

}  // namespace engine
}  // namespace dust2gpu
