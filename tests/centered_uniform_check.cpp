// Checks random::centered_uniform against the FP64 subtractions it
// replaces (u = U - 1/2, us = 1/2 - |u| for U = random_real), bit for
// bit, on the edge values of the 53-bit integer behind U and on 5 million
// random ones.  Prints "cases N bad B".
#include <cstdio>
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
  std::printf("cases %ld bad %ld\n", cases, bad);
  return bad != 0;
}
