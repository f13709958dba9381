// Integer pieces of the exact parallel running sum used by the serial
// resampling fallback (engine kernel `exact_running_sums`): the reference
// accumulates the weights as s_j = fl(s_{j-1} + w_j)
// (inst/include/dust2/filter_details.hpp:45-74), and these functions let
// a block reproduce that sequence bit for bit with integer prefix sums.
//
// While the running sum s stays in one binade [2^e, 2^(e+1)) (or among
// the subnormals and the first normal binade, which share a grid), every
// sum it takes is rounded to the same grid of multiples of 2^(e-52).  So
// fl(s + w) = s + 2^(e-52) * round(w / 2^(e-52)), where the integer does
// not depend on s, except when w / 2^(e-52) lies exactly halfway between
// two integers (round-half-even then looks at s).  Within a binade the
// running sum is therefore a prefix sum of integers, which is associative.
// Written once for host and device.
#pragma once

#include <cstdint>

#include "common.hpp"
#include "math.hpp"

namespace dust2gpu {
namespace exact_sum {

// Grid counts saturate here: anything this large leaves the binade.
constexpr std::uint64_t CAP = 1ull << 62;
// A running sum whose grid count reaches this has left its binade.
constexpr std::uint64_t TOP = 1ull << 53;

// Sum of two counts <= CAP, saturated at CAP (associative for such
// non-negative values, so a parallel scan may use it).
DUST2_HD std::uint64_t sat_add(std::uint64_t a, std::uint64_t b) {
  const std::uint64_t c = a + b;  // both <= 2^62: no wrap
  return c > CAP ? CAP : c;
}

// A running sum s written as base + count on its binade's grid:
// bits(s) = base + count, s = count * 2^e_grid; `ok` is false for Inf,
// NaN and negative sums, which the caller continues one add at a time.
struct grid {
  std::uint64_t base;
  std::uint64_t count;
  int e_grid;
  bool ok;
};

DUST2_HD grid grid_of(double s) {
  const std::uint64_t sb = math::bits_of(s);
  const int be = static_cast<int>(sb >> 52);  // includes the sign bit
  grid gr{0, 0, 0, be < 2047};
  const int bep = be < 1 ? 1 : be;  // subnormals share binade 1's grid
  gr.e_grid = bep - 1075;
  gr.base = static_cast<std::uint64_t>(bep - 1) << 52;
  gr.count = gr.ok ? sb - gr.base : 0;
  return gr;
}

// The value with `count` units (< TOP) on the grid of `gr`; exact.
DUST2_HD double grid_value(const grid& gr, std::uint64_t count) {
  return math::from_bits(gr.base + count);
}

// round(w / 2^e_grid) for w >= 0, saturated at CAP; *tie when
// w / 2^e_grid is exactly halfway between two integers.  A negative w
// (outside the weights' contract) saturates, so its step is taken with a
// real add.
DUST2_HD std::uint64_t grid_units(double w, int e_grid, bool* tie) {
  const std::uint64_t wb = math::bits_of(w);
  const int be = static_cast<int>(wb >> 52);
  std::uint64_t m = wb & ((1ull << 52) - 1);
  int e_w = -1074;
  if (be != 0) {
    m |= 1ull << 52;
    e_w = be - 1075;
  }
  *tie = false;
  if (m == 0) {
    return 0;  // +0 (or -0)
  }
  const int d = e_w - e_grid;
  if (d >= 0) {
    if (d >= 62 || (m >> (62 - d)) != 0) {
      return CAP;
    }
    return m << d;
  }
  const int sh = -d;
  if (sh > 54) {
    return 0;  // below half a unit (m < 2^53)
  }
  std::uint64_t q = m >> sh;
  const std::uint64_t rem = m & ((1ull << sh) - 1);
  const std::uint64_t half = 1ull << (sh - 1);
  if (rem > half) {
    q += 1;
  } else if (rem == half) {
    *tie = true;
  }
  return q;
}

// Whether the step that brings the grid count to `count` (after its
// units) must be taken with a real add: it leaves the binade or is a tie.
DUST2_HD bool is_break(std::uint64_t count, bool tie) {
  return tie || count >= TOP;
}

}  // namespace exact_sum
}  // namespace dust2gpu
