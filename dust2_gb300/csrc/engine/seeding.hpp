// Stream seeding for systems and filters (see dust2gpu/random.hpp for the
// stream contract).
#pragma once

#include <cstdint>
#include <vector>

namespace dust2gpu {
namespace engine {

// n_streams streams starting from a given first-stream state.
std::vector<std::uint64_t> make_streams(const std::uint64_t* first_state,
                                        std::size_t n_streams);

// n_streams streams from an integer seed (SplitMix64 expansion).
std::vector<std::uint64_t> make_streams_from_seed(std::uint64_t seed,
                                                  std::size_t n_streams);

}  // namespace engine
}  // namespace dust2gpu
