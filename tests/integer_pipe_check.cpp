// Checks the integer-pipe replacements of FP64 operations in the
// samplers.  random::centered_uniform against the FP64 subtractions it
// replaces (u = U - 1/2, us = 1/2 - |u| for U = random_real), bit for
// bit, on the edge values of the 53-bit integer behind U and on 5 million
// random ones; math::floor_bits against std::floor on special values,
// values near integers and powers of two, and random bit patterns;
// and math::twice_normal against 2 x.
// Prints "cases N bad B".
#include <cmath>
#include <cstdio>
#include <cstring>
#include <random>

#include "dust2gpu/random.hpp"

using namespace dust2gpu;

int main() {
  std::mt19937_64 g(1);
  long cases = 0, bad = 0;
  auto check = [&](unsigned long long m) {
    // a stream whose next output is m << 11 (xoshiro256+ returns s0 + s3)
    random::rng_state a{};
    a.state[0] = m << 11;
    a.state[1] = 12345;
    a.state[2] = 678;
    a.state[3] = 0;
    random::rng_state b = a;
    const double u1 = random::random_real(a) - 0.5;
    const double us1 = 0.5 - math::abs_bits(u1);
    double u2, us2;
    random::centered_uniform(b, &u2, &us2);
    ++cases;
    if (math::bits_of(u1) != math::bits_of(u2) ||
        math::bits_of(us1) != math::bits_of(us2) ||
        a.state[0] != b.state[0] || a.state[3] != b.state[3]) {
      ++bad;
    }
  };
  const unsigned long long half = 1ull << 52;
  for (unsigned long long m : {0ull, 1ull, 2ull, half - 2, half - 1, half,
                               half + 1, half + 2, (1ull << 53) - 1}) {
    check(m);
  }
  for (int i = 0; i < 5000000; ++i) {
    check(g() >> 11);
  }
  auto check_floor = [&](double x) {
    ++cases;
    if (math::bits_of(math::floor_bits(x)) != math::bits_of(std::floor(x))) {
      ++bad;
    }
  };
  for (double x : {0.0, -0.0, 0.5, -0.5, 1.0, -1.0, 1.5, -1.5, 2.0, -2.0,
                   0x1p52, -0x1p52, 0x1p52 + 1, 0x1.fffffffffffffp51,
                   -0x1.fffffffffffffp51, 0x1.fffffffffffffp-1,
                   -0x1.fffffffffffffp-1, 0x1p-1074, -0x1p-1074,
                   1e300, -1e300, HUGE_VAL, -HUGE_VAL}) {
    check_floor(x);
  }
  for (int k = -60; k <= 60; ++k) {
    const double p2 = std::ldexp(1.0, k);
    for (double d : {-1.0, 0.0, 1.0}) {
      const double x = p2 + d * std::ldexp(1.0, k - 52);
      check_floor(x);
      check_floor(-x);
      check_floor(std::nextafter(x, 0.0));
      check_floor(-std::nextafter(x, 0.0));
    }
  }
  std::uniform_real_distribution<double> wide(-1e6, 1e6);
  for (int i = 0; i < 2000000; ++i) {
    check_floor(wide(g));
    check_floor(std::round(wide(g)));
    unsigned long long b = g();
    double x;
    std::memcpy(&x, &b, 8);
    if (!std::isnan(x)) {
      check_floor(x);
    }
  }
  // the exact doubling used for BTRS's and PTRS's 2a
  for (int i = 0; i < 1000000; ++i) {
    const double x = std::ldexp(1.0 + (g() >> 12) * 0x1p-52,
                                static_cast<int>(g() % 2000) - 1000);
    ++cases;
    if (math::bits_of(math::twice_normal(x)) != math::bits_of(2.0 * x)) {
      ++bad;
    }
  }
  const double nan = std::nan("");
  ++cases;
  if (!std::isnan(math::floor_bits(nan))) {
    ++bad;
  }
  std::printf("cases %ld bad %ld\n", cases, bad);
  return bad != 0;
}
