// TEST INFRASTRUCTURE (oracle).  A stand-in for the `monty` package's
// random-number header, which dust2's engine headers include
// (inst/include/dust2/discrete/system.hpp:16, filter.hpp:6,
// continuous/system.hpp:20) but which is not part of the reference tree
// (DESCRIPTION: Imports/LinkingTo monty >= 0.3.11, not vendored).
//
// It supplies exactly what those headers use -- monty::random::prng (a
// vector of per-particle generators with state(k), export_state(),
// import_state()) and random_real() -- on top of the project's own
// generator (dust2_gb300/csrc/dust2gpu/random.hpp), so that the reference
// engine compiled against this shim draws the same streams as the GPU
// kernels.  Streams follow the documented monty layout: 4 uint64 words per
// stream, stream k+1 = jump(stream k).
#pragma once

#include <cstdint>
#include <stdexcept>
#include <vector>

#include "dust2gpu/distributions.hpp"
#include "dust2gpu/random.hpp"

namespace monty {
namespace random {

template <typename real_type>
using generator = dust2gpu::random::rng_state;

template <typename T>
class prng {
public:
  using int_type = typename T::int_type;

  // seed: 1 word (integer seed), 4 words (first stream) or 4 * n words
  // (all streams).
  prng(std::size_t n_streams, const std::vector<int_type>& seed,
       bool deterministic) : state_(n_streams) {
    std::uint64_t s[4];
    if (seed.size() == 4 * n_streams && n_streams > 0) {
      for (std::size_t i = 0; i < n_streams; ++i) {
        for (int w = 0; w < 4; ++w) {
          state_[i].state[w] = seed[4 * i + w];
        }
      }
    } else {
      if (seed.size() == 1) {
        dust2gpu::random::seed_state(seed[0], s);
      } else if (seed.size() >= 4) {
        for (int w = 0; w < 4; ++w) {
          s[w] = seed[w];
        }
      } else {
        throw std::runtime_error("invalid seed");
      }
      for (std::size_t i = 0; i < n_streams; ++i) {
        if (i > 0) {
          dust2gpu::random::jump(s);
        }
        for (int w = 0; w < 4; ++w) {
          state_[i].state[w] = s[w];
        }
      }
    }
    for (auto& el : state_) {
      el.deterministic = deterministic;
      el.err = 0;
      el.err_v0 = 0;
      el.err_v1 = 0;
    }
  }

  T& state(std::size_t i) {
    return state_[i];
  }

  std::size_t size() const {
    return state_.size();
  }

  std::vector<int_type> export_state() const {
    std::vector<int_type> ret;
    ret.reserve(4 * state_.size());
    for (const auto& el : state_) {
      for (int w = 0; w < 4; ++w) {
        ret.push_back(el.state[w]);
      }
    }
    return ret;
  }

  void import_state(const std::vector<int_type>& s) {
    if (s.size() != 4 * state_.size()) {
      throw std::runtime_error("invalid rng state length");
    }
    for (std::size_t i = 0; i < state_.size(); ++i) {
      for (int w = 0; w < 4; ++w) {
        state_[i].state[w] = s[4 * i + w];
      }
    }
  }

private:
  std::vector<T> state_;
};

template <typename real_type, typename T>
real_type random_real(T& state) {
  return dust2gpu::random::random_real(state);
}

}  // namespace random
}  // namespace monty
