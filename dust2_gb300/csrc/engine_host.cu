// Host-side helpers of the engine that do not depend on a system type:
// error message formatting and stream seeding.
#include <algorithm>
#include <cstdio>
#include <sstream>
#include <string>
#include <thread>
#include <vector>

#include "dust2gpu/random.hpp"
#include "engine/api.hpp"
#include "engine/error_text.hpp"
#include "engine/seeding.hpp"

namespace dust2gpu {
namespace engine {

std::string describe_error(const particle_error& e) {
  return error_text(e);
}

// inst/include/dust2/errors.hpp:29-54: "<count> particles reported
// errors." followed by the first n_max, 1-based, and a tail count.
std::string format_errors(const std::vector<particle_error>& errors,
                          const char* title, std::size_t n_max) {
  std::size_t count = 0;
  for (const auto& e : errors) {
    if (e.code != 0) {
      ++count;
    }
  }
  std::stringstream msg;
  msg << count << " " << title << " reported errors.";
  const std::size_t n_report = std::min(n_max, count);
  for (std::size_t i = 0, j = 0; i < errors.size() && j < n_report; ++i) {
    if (errors[i].code != 0) {
      msg << std::endl << "  - " << i + 1 << ": " << describe_error(errors[i]);
      ++j;
    }
  }
  if (n_report < count) {
    msg << std::endl << "  - (and " << (count - n_report) << " more)";
  }
  return msg.str();
}

// Streams 0 .. n-1 of a seed: stream 0 is the seed state (or its
// SplitMix64 expansion), stream k+1 = jump(stream k).  Blocks of streams
// are filled in parallel, each block starting from a GF(2) skip-ahead.
std::vector<std::uint64_t> make_streams(const std::uint64_t* first_state,
                                        std::size_t n_streams) {
  std::vector<std::uint64_t> out(4 * n_streams);
  if (n_streams == 0) {
    return out;
  }
  const std::size_t block = 4096;
  const std::size_t n_blocks_total = (n_streams + block - 1) / block;
  std::vector<random::gf2_matrix> powers;
  if (n_blocks_total > 1) {
    int n_pow = 1;
    while ((static_cast<std::size_t>(1) << n_pow) < n_streams) {
      ++n_pow;
    }
    powers = random::jump_powers(n_pow + 1);
  }
  auto fill_block = [&](std::size_t b) {
    std::uint64_t s[4] = {first_state[0], first_state[1], first_state[2],
                          first_state[3]};
    const std::size_t start = b * block;
    if (start > 0) {
      random::jump_n(powers, start, s);
    }
    const std::size_t end = std::min(n_streams, start + block);
    for (std::size_t k = start; k < end; ++k) {
      if (k > start) {
        random::jump(s);
      }
      for (int w = 0; w < 4; ++w) {
        out[4 * k + w] = s[w];
      }
    }
  };
  const std::size_t n_threads = std::min<std::size_t>(
    n_blocks_total, std::max(1u, std::thread::hardware_concurrency()));
  if (n_threads <= 1) {
    for (std::size_t b = 0; b < n_blocks_total; ++b) {
      fill_block(b);
    }
  } else {
    std::vector<std::thread> pool;
    for (std::size_t t = 0; t < n_threads; ++t) {
      pool.emplace_back([&, t]() {
        for (std::size_t b = t; b < n_blocks_total; b += n_threads) {
          fill_block(b);
        }
      });
    }
    for (auto& th : pool) {
      th.join();
    }
  }
  return out;
}

std::vector<std::uint64_t> make_streams_from_seed(std::uint64_t seed,
                                                  std::size_t n_streams) {
  std::uint64_t s[4];
  random::seed_state(seed, s);
  return make_streams(s, n_streams);
}

}  // namespace engine
}  // namespace dust2gpu
