// Per-particle random number streams: xoshiro256+ (Blackman & Vigna,
// "Scrambled linear pseudorandom number generators", ACM TOMS 2021).
//
// dust2 takes its generator from monty (monty::random::prng /
// monty::random::generator<double>, used at
// inst/include/dust2/discrete/system.hpp:401 and filter.hpp:148).  The
// contract kept here is the one dust2's tests rely on:
//   * one stream is 4 x uint64 = 32 bytes of raw state
//     (tests/testthat/test-filter.R:130, test-sir.R:14);
//   * stream i+1 is stream i advanced by jump(), i.e. 2^128 draws;
//   * an integer seed is expanded into the first stream with SplitMix64
//     (Steele, Lea & Flood 2014), the seeding the xoshiro authors
//     recommend;
//   * random_real() maps the top 53 bits of a draw onto [0, 1).
// monty's own bit patterns cannot be checked in this build (monty is not
// vendored), so equality is defined against this header, which the CPU
// oracle and the CUDA kernels share.
#pragma once

#include <cstdint>
#include <vector>

#include "common.hpp"
#include "math.hpp"

namespace dust2gpu {
namespace random {

// The per-particle generator: the 4-word xoshiro state, the
// deterministic flag (draws return their expectation, as dust2's
// `deterministic = TRUE` systems expect, test-walk.R:59-66) and an error
// slot filled by samplers that receive invalid arguments.
struct rng_state {
  using int_type = std::uint64_t;
  static constexpr std::size_t size() {
    return 4;
  }
  std::uint64_t state[4];
  bool deterministic;
  int err;
  double err_v0;
  double err_v1;

  DUST2_HD std::uint64_t& operator[](int i) {
    return state[i];
  }
  DUST2_HD const std::uint64_t& operator[](int i) const {
    return state[i];
  }
};

DUST2_HD void set_error(rng_state& s, int code, double v0, double v1) {
  if (s.err == 0) {
    s.err = code;
    s.err_v0 = v0;
    s.err_v1 = v1;
  }
}

DUST2_HD std::uint64_t rotl(std::uint64_t x, int k) {
  return (x << k) | (x >> (64 - k));
}

// xoshiro256+: returns s0 + s3, then advances the linear engine.
DUST2_HD std::uint64_t next(std::uint64_t* s) {
  const std::uint64_t result = s[0] + s[3];
  const std::uint64_t t = s[1] << 17;
  s[2] ^= s[0];
  s[3] ^= s[1];
  s[1] ^= s[2];
  s[0] ^= s[3];
  s[2] ^= t;
  s[3] = rotl(s[3], 45);
  return result;
}

DUST2_HD std::uint64_t next(rng_state& s) {
  return next(s.state);
}

// Uniform on [0, 1) with 53 random bits.
DUST2_HD double random_real(rng_state& s) {
  if (s.deterministic) {
    return 0.5;
  }
  // same value as static_cast<double>(next(s) >> 11) * 2^-53, built on
  // the integer pipe
  return math::u53_to_unit(next(s) >> 11);
}

// For the next uniform U of random_real (U = m 2^-53): u = U - 1/2 and
// us = 1/2 - |u|.  Both are multiples of 2^-53 smaller than 1, so the
// FP64 subtractions are exact; here they are assembled from the integer
// m - 2^52 on the integer pipe, with the same values and signs (U = 1/2
// gives u = +0; U = 0 gives us = +0).
DUST2_HD void centered_uniform(rng_state& s, double* u, double* us) {
  if (s.deterministic) {
    *u = 0.0;
    *us = 0.5;
    return;
  }
  const std::uint64_t m = next(s) >> 11;
  constexpr std::uint64_t half = static_cast<std::uint64_t>(1) << 52;
  const bool neg = m < half;
  const std::uint64_t ad = neg ? half - m : m - half;
  const double mag = math::u53_to_unit(ad);
  *u = neg ? math::from_bits(math::bits_of(mag) | 0x8000000000000000ull) :
    mag;
  *us = math::u53_to_unit(half - ad);
}

// Advance a stream by 2^128 draws.  The characteristic-polynomial
// coefficients are the published jump constants for xoshiro256.
DUST2_HD void jump(std::uint64_t* s) {
  constexpr std::uint64_t JUMP[4] = {
    0x180ec6d33cfd0abaull, 0xd5a61266f0c9392cull,
    0xa9582618e03fc9aaull, 0x39abdc4529b1661cull};
  std::uint64_t s0 = 0, s1 = 0, s2 = 0, s3 = 0;
  for (int i = 0; i < 4; ++i) {
    for (int b = 0; b < 64; ++b) {
      if (JUMP[i] & (static_cast<std::uint64_t>(1) << b)) {
        s0 ^= s[0];
        s1 ^= s[1];
        s2 ^= s[2];
        s3 ^= s[3];
      }
      next(s);
    }
  }
  s[0] = s0;
  s[1] = s1;
  s[2] = s2;
  s[3] = s3;
}

// Advance a stream by 2^192 draws (published long-jump constants).
DUST2_HD void long_jump(std::uint64_t* s) {
  constexpr std::uint64_t LONG_JUMP[4] = {
    0x76e15d3efefdcbbfull, 0xc5004e441c522fb3ull,
    0x77710069854ee241ull, 0x39109bb02acbe635ull};
  std::uint64_t s0 = 0, s1 = 0, s2 = 0, s3 = 0;
  for (int i = 0; i < 4; ++i) {
    for (int b = 0; b < 64; ++b) {
      if (LONG_JUMP[i] & (static_cast<std::uint64_t>(1) << b)) {
        s0 ^= s[0];
        s1 ^= s[1];
        s2 ^= s[2];
        s3 ^= s[3];
      }
      next(s);
    }
  }
  s[0] = s0;
  s[1] = s1;
  s[2] = s2;
  s[3] = s3;
}

// SplitMix64 step, used to expand an integer seed into a full state.
inline std::uint64_t splitmix64(std::uint64_t& x) {
  std::uint64_t z = (x += 0x9e3779b97f4a7c15ull);
  z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
  z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
  return z ^ (z >> 31);
}

// The first stream for an integer seed.
inline void seed_state(std::uint64_t seed, std::uint64_t* s) {
  for (int i = 0; i < 4; ++i) {
    s[i] = splitmix64(seed);
  }
}

// ---------------------------------------------------------------------
// Skip-ahead over many jumps.  The state transition of xoshiro256 is
// linear over GF(2), so jump() is a 256x256 bit matrix J.  Stream k of a
// seed is J^k s0; computing J^(2^b) by repeated squaring lets any stream
// be reached in at most 64 matrix-vector products, so stream blocks can
// be filled in parallel and still equal the sequential jump() chain.
struct gf2_matrix {
  // column c (0..255) is the image of basis vector e_c: 4 words each
  std::uint64_t col[256][4];
};

inline void gf2_apply(const gf2_matrix& m, const std::uint64_t* v,
                      std::uint64_t* out) {
  std::uint64_t r[4] = {0, 0, 0, 0};
  for (int w = 0; w < 4; ++w) {
    std::uint64_t word = v[w];
    while (word) {
      const int b = __builtin_ctzll(word);
      const auto& c = m.col[w * 64 + b];
      r[0] ^= c[0];
      r[1] ^= c[1];
      r[2] ^= c[2];
      r[3] ^= c[3];
      word &= word - 1;
    }
  }
  out[0] = r[0];
  out[1] = r[1];
  out[2] = r[2];
  out[3] = r[3];
}

inline void gf2_multiply(const gf2_matrix& a, const gf2_matrix& b,
                         gf2_matrix& out) {
  for (int c = 0; c < 256; ++c) {
    gf2_apply(a, b.col[c], out.col[c]);
  }
}

inline void jump_matrix(gf2_matrix& m) {
  for (int c = 0; c < 256; ++c) {
    std::uint64_t s[4] = {0, 0, 0, 0};
    s[c / 64] = static_cast<std::uint64_t>(1) << (c % 64);
    jump(s);
    for (int w = 0; w < 4; ++w) {
      m.col[c][w] = s[w];
    }
  }
}

// J^(2^b) for b = 0 .. n_pow-1.
inline std::vector<gf2_matrix> jump_powers(int n_pow) {
  std::vector<gf2_matrix> pw(n_pow);
  jump_matrix(pw[0]);
  for (int b = 1; b < n_pow; ++b) {
    gf2_multiply(pw[b - 1], pw[b - 1], pw[b]);
  }
  return pw;
}

// s <- J^k s
inline void jump_n(const std::vector<gf2_matrix>& pw, std::uint64_t k,
                   std::uint64_t* s) {
  for (std::size_t b = 0; k != 0; ++b, k >>= 1) {
    if (k & 1) {
      gf2_apply(pw[b], s, s);
    }
  }
}

}  // namespace random
}  // namespace dust2gpu
