// Project-owned FP64 elementary functions, identical on host and device.
//
// dust2 draws its random variates through monty (an external package that
// is not available here), and monty's samplers evaluate exp/log/lgamma.
// Platform libm implementations (glibc, CUDA) differ in the last bit, so
// the particle trajectories of a CPU run and a GPU run would drift apart
// after the first differently-rounded draw.  Everything here is therefore
// written from textbook methods using only correctly rounded IEEE
// operations, so that the host oracle and the kernels produce identical
// bits.  GB300 executes FP64 at 1/64 of its FP32 rate, so the methods are
// chosen to need few FP64 operations and no FP64 division:
//
//   exp    table-driven (Tang 1989): x = (128 k + j) ln2/128 + r,
//          |r| <= ln2/256, exp(x) = 2^k 2^(j/128) (1 + expm1(r)), expm1 by
//          its Taylor polynomial through r^6.  Evaluated in integer fixed
//          point (exp_fixed, below) for |x| < 704; near overflow and
//          underflow in FP64 (exp_slow, Taylor through r^5, a double-double
//          table and a two-part ln2/128).
//   log    table-driven (Tang 1990): x = 2^e m, m in [sqrt(2)/2, sqrt(2)),
//          F = j/256 nearest to m, r = (m - F)/F, then
//          log(x) = e ln2 + log(F) + log1p(r), log1p by its Taylor
//          polynomial through r^7; evaluated in integer fixed point
//          (log_fixed, below).
//   rcp    1/y from the correctly rounded FP32 reciprocal of (float)y
//          (cheap on this GPU) refined by two Newton steps in FP64 FMA.
//   lgamma for x > 0: exact table of log(k!) for integer arguments below
//          30; otherwise the argument is shifted up to >= 10 with the
//          recurrence Gamma(x+1) = x Gamma(x) and the Stirling series
//          with Bernoulli coefficients B_2k / (2k (2k-1)), k = 1..7.  On
//          the device, integer arguments up to 2^20 + 1 are read from a
//          table that the device filled with these same values.
//   cos_2pi / sin_2pi (argument in turns) for the Box-Muller transform:
//          quadrant reduction on the turn count (exact), then Taylor
//          series of cos and sin on |x| <= pi/4.
//
// Range checks, rounding to an integer, scaling by powers of two and the
// FP64 <-> FP32 conversions are done on the bit patterns where that is
// exact: every FP64 instruction, comparisons and conversions included,
// occupies the one slow FP64 pipe of this GPU.
//
// All constants below and in tables.hpp (make_tables.py) are the correctly
// rounded doubles of the stated exact rationals or mathematical constants.
#pragma once

#include <cmath>
#include <cstdint>
#include <cstring>
#include <limits>

#include "common.hpp"
#include "tables.hpp"

namespace dust2gpu {
namespace math {

// Functions compiled once per kernel and called rather than expanded at
// every call site: the fixed-point exp/log cores, the reciprocal and the
// rarely taken slow paths.  Expanded, they would raise the register
// pressure of the large sampler kernels and, above all, their code size:
// making the reciprocal alone a called function took the SIR filter from
// 1.51G to 1.75G particle-steps/s and the SEIR filter from 80M to 101M,
// by relieving instruction-fetch stalls.
#if defined(__CUDACC__)
#define DUST2_MATH_CORE inline __host__ __device__ __noinline__
#else
#define DUST2_MATH_CORE inline
#endif

DUST2_HD std::uint64_t bits_of(double x) {
#if defined(__CUDA_ARCH__)
  return static_cast<std::uint64_t>(__double_as_longlong(x));
#else
  std::uint64_t u;
  std::memcpy(&u, &x, sizeof(u));
  return u;
#endif
}

DUST2_HD double from_bits(std::uint64_t u) {
#if defined(__CUDA_ARCH__)
  return __longlong_as_double(static_cast<long long>(u));
#else
  double x;
  std::memcpy(&x, &u, sizeof(x));
  return x;
#endif
}

DUST2_HD double infinity() {
  return from_bits(0x7ff0000000000000ull);
}

DUST2_HD double quiet_nan() {
  return from_bits(0x7ff8000000000000ull);
}

DUST2_HD bool is_nan(double x) {
  return x != x;
}

DUST2_HD bool is_finite(double x) {
  return (bits_of(x) & 0x7ff0000000000000ull) != 0x7ff0000000000000ull;
}

// 2^k as a double, for k in the normal range [-1022, 1023].
DUST2_HD double pow2i(int k) {
  return from_bits(static_cast<std::uint64_t>(k + 1023) << 52);
}

// p * 2^k for p in [0.5, 2) and k in [-1080, 1025], rounding once.
DUST2_HD double scale2(double p, int k) {
  if (k > 1023) {
    return p * pow2i(1023) * pow2i(k - 1023);
  }
  if (k < -1021) {
    // p * 2^(k+54) is exact (normal), then one rounding into the
    // subnormal range.
    return (p * pow2i(k + 54)) * pow2i(-54);
  }
  return p * pow2i(k);
}

// ln(2) split so that k * LN2_HI is exact for |k| < 2^11.
constexpr double LN2_HI = 0x1.62e42fefa3800p-1;
constexpr double LN2_LO = 0x1.ef35793c76730p-45;
constexpr double LOG2E = 0x1.71547652b82fep+0;
constexpr double SQRT2 = 0x1.6a09e667f3bcdp+0;
constexpr double HALF_LOG_2PI = 0x1.d67f1c864beb5p-1;  // log(2 pi) / 2

// Overflow / underflow thresholds of exp: exp(x) > DBL_MAX above
// 709.782712893384 and rounds to zero below -745.1332191019412.
constexpr double EXP_OVERFLOW = 0x1.62e42fefa39efp+9;
constexpr double EXP_UNDERFLOW = -0x1.74910d52d3051p+9;

// Paired constant tables: device code reads global memory (lanes index
// different entries, which constant memory would serialise), host code a
// plain array with the same values.
#if defined(__CUDACC__)
#define DUST2_TABLE(name, n, values)                                      \
  __device__ const double name##_dev[n] = {values};                      \
  inline const double name##_host[n] = {values};
#else
#define DUST2_TABLE(name, n, values)                                      \
  inline const double name##_host[n] = {values};
#endif
#if defined(__CUDA_ARCH__)
#define DUST2_TAB(name, i) (name##_dev[i])
#else
#define DUST2_TAB(name, i) (name##_host[i])
#endif

DUST2_TABLE(exp2_hi, 128, DUST2_EXP2_HI)
DUST2_TABLE(exp2_lo, 128, DUST2_EXP2_LO)
DUST2_TABLE(recip_int, 129, DUST2_RECIP_INT)

#if defined(__CUDACC__)
#define DUST2_TABLE_U64(name, n, values)                                  \
  __device__ const std::uint64_t name##_dev[n] = {values};               \
  inline const std::uint64_t name##_host[n] = {values};
#define DUST2_TABLE_I64(name, n, values)                                  \
  __device__ const std::int64_t name##_dev[n] = {values};                \
  inline const std::int64_t name##_host[n] = {values};
#else
#define DUST2_TABLE_U64(name, n, values)                                  \
  inline const std::uint64_t name##_host[n] = {values};
#define DUST2_TABLE_I64(name, n, values)                                  \
  inline const std::int64_t name##_host[n] = {values};
#endif

// Integer-pipe helpers.  On this GPU every FP64 instruction (arithmetic,
// comparison, rounding, conversion) shares one slow pipe, so decisions
// that can be taken on the bit patterns are taken there, exactly.

// a > b for doubles a >= +0 and b not NaN (b may be negative or -0; a
// and b must not both be zeros of different sign with a = +0, b = -0).
DUST2_HD bool gt_nonneg(double a, double b) {
  return static_cast<std::int64_t>(bits_of(a)) >
    static_cast<std::int64_t>(bits_of(b));
}

// a <= b for doubles a, b >= +0 (neither NaN nor -0).
DUST2_HD bool le_nonneg(double a, double b) {
  return bits_of(a) <= bits_of(b);
}

// floor(x) on the integer pipe, the same value as std::floor for every
// x (including -0, infinities and NaN): the fraction bits are cleared,
// and a negative x with a fraction moves one unit further from zero (a
// carry out of the mantissa lands in the exponent, as it should).
DUST2_HD double floor_bits(double x) {
  const std::uint64_t u = bits_of(x);
  const int e = static_cast<int>((u >> 52) & 0x7ff);
  const bool neg = (u >> 63) != 0;
  if (e >= 1075) {  // |x| >= 2^52, infinite or NaN: already integral
    return x;
  }
  if (e < 1023) {  // |x| < 1
    if ((u << 1) == 0 || !neg) {
      return from_bits(u & 0x8000000000000000ull);  // +-0
    }
    return -1.0;
  }
  const std::uint64_t unit = static_cast<std::uint64_t>(1) << (1075 - e);
  const std::uint64_t frac = u & (unit - 1);
  if (frac == 0) {
    return x;
  }
  const std::uint64_t t = u - frac;  // toward zero
  return from_bits(neg ? t + unit : t);
}

// 2 x for a normal x whose double is also normal (an exponent
// increment: the same value as the exact FP64 product).
DUST2_HD double twice_normal(double x) {
  return from_bits(bits_of(x) + (static_cast<std::uint64_t>(1) << 52));
}

// |x| by clearing the sign bit.
DUST2_HD double abs_bits(double x) {
  return from_bits(bits_of(x) & 0x7fffffffffffffffull);
}

// m * 2^-53 for an integer 0 <= m < 2^53, assembled from its bits (the
// value is exact, the same as static_cast<double>(m) * 2^-53).
DUST2_HD double u53_to_unit(std::uint64_t m) {
  if (m == 0) {
    return 0.0;
  }
#if defined(__CUDA_ARCH__)
  const int lz = __clzll(static_cast<long long>(m)) - 11;
#else
  const int lz = __builtin_clzll(m) - 11;
#endif
  // m has 53 - lz significant bits; the leading one moves to bit 52
  const std::uint64_t mant = (m << lz) & 0x000fffffffffffffull;
  const std::uint64_t expo = static_cast<std::uint64_t>(1023 - 1 - lz);
  return from_bits((expo << 52) | mant);
}

// |x| below this (704) takes the fast path of exp: the result is normal
// and the scaling by 2^e is an exponent add.
constexpr std::uint64_t EXP_FAST_BITS = 0x4086000000000000ull;
// 1.5 * 2^52: adding it to |v| < 2^51 rounds v to an integer (ties to
// even, the same as rint) in the low mantissa bits.
constexpr double ROUND_SHIFTER = 0x1.8p52;

DUST2_MATH_CORE double exp_slow(double x) {
  if (is_nan(x)) {
    return x;
  }
  if (x > EXP_OVERFLOW) {
    return infinity();
  }
  if (x < EXP_UNDERFLOW) {
    return 0.0;
  }
  const double kf = std::rint(x * DUST2_INV_LN2_128);
  const int k = static_cast<int>(kf);
  double r = std::fma(-kf, DUST2_LN2_128_HI, x);
  r = std::fma(-kf, DUST2_LN2_128_LO, r);
  const int j = k & 127;
  const int e = (k - j) / 128;
  double p = std::fma(r, 0x1.1111111111111p-7, 0x1.5555555555555p-5);
  p = std::fma(p, r, 0x1.5555555555555p-3);
  p = std::fma(p, r, 0.5);
  const double pm1 = std::fma(r * r, p, r);
  const double t_hi = DUST2_TAB(exp2_hi, j);
  const double t_lo = DUST2_TAB(exp2_lo, j);
  return scale2(t_hi + std::fma(t_hi, pm1, t_lo), e);
}

// ---- integer-arithmetic exp and log --------------------------------------
//
// The same methods in fixed point: every operation is an integer
// instruction, so the evaluation runs on the integer pipes, which this GPU
// has in far greater width than its FP64 pipe (one FP64 warp instruction
// holds an SM partition's FP64 unit for 64 cycles; a 64 x 64 -> 128-bit
// product costs about a third of that on the integer pipe, and overlaps
// with FP64 work).  Host and device run the same integer arithmetic, so
// results are identical.  Relative error before the final rounding is
// below 2^-60: the result is the correctly rounded value except within
// ~2^-8 ulp of a rounding midpoint, where it may be the other neighbour.

using u128 = unsigned __int128;
using i128 = __int128;


DUST2_TABLE_U64(exp2_q63, 128, DUST2_EXP2_Q63)
DUST2_TABLE_U64(log_inv_q62, DUST2_LOG_N, DUST2_LOG_INV_Q62)
DUST2_TABLE_I64(log_f96_hi, DUST2_LOG_N, DUST2_LOG_F96_HI)
DUST2_TABLE_U64(log_f96_lo, DUST2_LOG_N, DUST2_LOG_F96_LO)

// (a * b) >> s for signed a, b (arithmetic shift; floor).
DUST2_HD std::int64_t mul_shift(std::int64_t a, std::int64_t b, int s) {
  return static_cast<std::int64_t>((static_cast<i128>(a) *
                                    static_cast<i128>(b)) >> s);
}

#if defined(__CUDA_ARCH__)
DUST2_HD int clz64(std::uint64_t v) {
  return __clzll(static_cast<long long>(v));
}
#else
DUST2_HD int clz64(std::uint64_t v) {
  return v == 0 ? 64 : __builtin_clzll(v);
}
#endif

// v * 2^-scale for a non-zero unsigned 128-bit v, rounded to 53 bits
// (ties away from zero) with the given sign; the result must be normal.
DUST2_HD double u128_to_double(u128 v, int scale, bool negative) {
  const std::uint64_t hi = static_cast<std::uint64_t>(v >> 64);
  const int p = hi != 0 ? 127 - clz64(hi) :
    63 - clz64(static_cast<std::uint64_t>(v));  // position of the top bit
  std::uint64_t m;
  int top = p;
  if (p >= 53) {
    const int sh = p - 52;
    m = static_cast<std::uint64_t>((v + (static_cast<u128>(1) << (sh - 1)))
                                   >> sh);
    if (m >> 53) {
      m >>= 1;
      top += 1;
    }
  } else {
    m = static_cast<std::uint64_t>(v) << (52 - p);
  }
  const std::uint64_t e = static_cast<std::uint64_t>(top - scale + 1023);
  return from_bits((negative ? 0x8000000000000000ull : 0ull) | (e << 52) |
                   (m & 0x000fffffffffffffull));
}

// exp(x) for 2^-54 <= |x| < 704 (the caller handles the rest).
//   t = |x| 128/ln2 in fixed point with 64 fraction bits, from the 53-bit
//       significand times a 128-bit 128/ln2 (error < 2^-64);
//   k = rint(+-t), f = +-t - k in [-1/2, 1/2]; r = f ln2/128, held as
//       r 2^71;
//   expm1(r) = r + r^2 P(r), P = 1/2 + r/6 + r^2/24 + r^3/120 + r^4/720
//       (Taylor; the next term is below 2^-72), Horner in Q63;
//   2^(k/128) = 2^(k >> 7) 2^(j/128), j = k & 127, 2^(j/128) in Q63.
DUST2_MATH_CORE double exp_fixed(std::uint64_t u) {
  const std::uint64_t a = u & 0x7fffffffffffffffull;
  const int be = static_cast<int>(a >> 52);
  const std::uint64_t mant = (a & 0x000fffffffffffffull) |
    0x0010000000000000ull;
  const u128 p_lo = static_cast<u128>(mant) * DUST2_EXP_C120_LO;
  const u128 p_hi = static_cast<u128>(mant) * DUST2_EXP_C120_HI;
  const u128 w = p_hi + (p_lo >> 64);  // floor(mant * C / 2^64)
  const u128 t = w >> (1067 - be);     // |x| 128/ln2 2^64, be in [969, 1032]
  const u128 tr = t + (static_cast<u128>(1) << 63);
  const std::int64_t n = static_cast<std::int64_t>(tr >> 64);
  std::int64_t f = static_cast<std::int64_t>(
    static_cast<std::uint64_t>(tr) - 0x8000000000000000ull);
  std::int64_t k = n;
  if (u >> 63) {
    k = -n;
    f = f == INT64_MIN ? INT64_MAX : -f;
  }
  // r 2^71 = f ln2 (f in units of 2^-64)
  const std::int64_t r = static_cast<std::int64_t>(
    (static_cast<i128>(f) * static_cast<i128>(DUST2_LN2_Q64)) >> 64);
  std::int64_t pq = 0x002d82d82d82d82ell;          // 1/720 in Q63
  pq = 0x0111111111111111ll + mul_shift(r, pq, 71);  // 1/120
  pq = 0x0555555555555555ll + mul_shift(r, pq, 71);  // 1/24
  pq = 0x1555555555555555ll + mul_shift(r, pq, 71);  // 1/6
  pq = 0x4000000000000000ll + mul_shift(r, pq, 71);  // 1/2
  const std::int64_t rp = mul_shift(r, pq, 71);      // r P, Q63
  const std::int64_t em1 = r + mul_shift(r, rp, 63);  // expm1(r) 2^71
  const int j = static_cast<int>(k & 127);
  const int e = static_cast<int>(k >> 7);
  const std::uint64_t tj = DUST2_TAB(exp2_q63, j);
  const std::uint64_t v = static_cast<std::uint64_t>(
    static_cast<i128>(tj) + ((static_cast<i128>(tj) *
                              static_cast<i128>(em1)) >> 71));
  // v = 2^(j/128) exp(r) in Q63, in [2^63 - 2^55, 2^64)
  std::uint64_t m;
  int ee = e;
  if (v >> 63) {
    m = (v >> 11) + ((v >> 10) & 1);
  } else {
    m = (v >> 10) + ((v >> 9) & 1);
    ee -= 1;
  }
  if (m >> 53) {
    m >>= 1;
    ee += 1;
  }
  return from_bits((static_cast<std::uint64_t>(ee + 1023) << 52) |
                   (m & 0x000fffffffffffffull));
}

// log(x) for x positive, normal and finite: the method of log() below
// (x = 2^e m, m in [sqrt(2)/2, sqrt(2)), F = j/256 nearest m,
// r = (m - F)/F, log x = e ln2 + log F + log1p(r)) in fixed point:
// r 2^71 from (m - F) and 256/j in Q62; log1p(r) = r Q(r),
// Q = 1 - r/2 + r^2/3 - ... + r^6/7 in Q62 (the next term of log1p is
// below 2^-71); the sum at 2^-96, or, for m rounding to F = 1 with e = 0,
// r Q alone, which keeps full relative precision for x near 1.
DUST2_MATH_CORE double log_fixed(std::uint64_t u, int e_adj) {
  const std::uint64_t mant = u & 0x000fffffffffffffull;
  int e = static_cast<int>(u >> 52) - 1023 + e_adj;
  const bool half = mant > (0x3ff6a09e667f3bcdull & 0x000fffffffffffffull);
  const int s = half ? 45 : 44;
  const std::uint64_t q =
    (mant + (1ull << (s - 1)) - 1 + ((mant >> s) & 1)) >> s;
  const std::int64_t m2 = static_cast<std::int64_t>(mant |
                                                    0x0010000000000000ull);
  int j;
  std::int64_t fi;  // m - F in units of 2^-52 (2^-53 when half)
  if (half) {
    e += 1;
    j = 128 + static_cast<int>(q);
    fi = m2 - (static_cast<std::int64_t>(j) << 45);
  } else {
    j = 256 + static_cast<int>(q);
    fi = m2 - (static_cast<std::int64_t>(j) << 44);
  }
  const int i = j - DUST2_LOG_J0;
  const std::int64_t inv = static_cast<std::int64_t>(
    DUST2_TAB(log_inv_q62, i));
  const std::int64_t r = mul_shift(fi, inv, half ? 44 : 43);  // r 2^71
  std::int64_t pq = 0x0924924924924925ll;               // 1/7 in Q62
  pq = -0x0aaaaaaaaaaaaaabll + mul_shift(r, pq, 71);    // -1/6
  pq = 0x0ccccccccccccccdll + mul_shift(r, pq, 71);     // 1/5
  pq = -0x1000000000000000ll + mul_shift(r, pq, 71);    // -1/4
  pq = 0x1555555555555555ll + mul_shift(r, pq, 71);     // 1/3
  pq = -0x2000000000000000ll + mul_shift(r, pq, 71);    // -1/2
  pq = 0x4000000000000000ll + mul_shift(r, pq, 71);     // Q, Q62
  const i128 rq = static_cast<i128>(r) * static_cast<i128>(pq);  // 2^-133
  if (e == 0 && j == 256) {
    if (rq == 0) {
      return 0.0;
    }
    return rq < 0 ? u128_to_double(static_cast<u128>(-rq), 133, true) :
      u128_to_double(static_cast<u128>(rq), 133, false);
  }
  const i128 ln2 = (static_cast<i128>(DUST2_LN2_96_HI) << 64) |
    static_cast<i128>(DUST2_LN2_96_LO);
  const i128 lf = static_cast<i128>(static_cast<u128>(
    static_cast<std::uint64_t>(DUST2_TAB(log_f96_hi, i))) << 64) |
    static_cast<i128>(DUST2_TAB(log_f96_lo, i));
  const i128 sum = static_cast<i128>(e) * ln2 + lf + (rq >> 37);
  return sum < 0 ? u128_to_double(static_cast<u128>(-sum), 96, true) :
    u128_to_double(static_cast<u128>(sum), 96, false);
}

DUST2_HD double exp(double x) {
#if defined(DUST2_HOST_LIBM) && !defined(__CUDA_ARCH__)
  // the timing build of the CPU oracle: the host's libm, as dust2 calls it
  return std::exp(x);
#endif
  const std::uint64_t u = bits_of(x);
  const std::uint64_t a = u & 0x7fffffffffffffffull;
  if (a >= EXP_FAST_BITS) {
    return exp_slow(x);  // NaN, infinities, |x| >= 704
  }
  if (a < 0x3c90000000000000ull) {
    return 1.0;  // |x| < 2^-54: 1 + x rounds to 1
  }
  return exp_fixed(u);
}

DUST2_HD double log(double x) {
#if defined(DUST2_HOST_LIBM) && !defined(__CUDA_ARCH__)
  return std::log(x);
#endif
  std::uint64_t u = bits_of(x);
  int e_adj = 0;
  // positive normal finite numbers have u in [2^52, 0x7ff0...)
  if (u - 0x0010000000000000ull >= 0x7fe0000000000000ull) {
    if (is_nan(x) || x < 0) {
      return quiet_nan();
    }
    if (x == 0) {
      return -infinity();
    }
    if (!is_finite(x)) {
      return x;
    }
    // subnormal: renormalise exactly
    u = bits_of(x * 0x1p54);
    e_adj = -54;
  }
  return log_fixed(u, e_adj);
}

DUST2_HD float float_from_bits(std::uint32_t u) {
#if defined(__CUDA_ARCH__)
  return __uint_as_float(u);
#else
  float x;
  std::memcpy(&x, &u, sizeof(x));
  return x;
#endif
}

DUST2_HD std::uint32_t float_bits_of(float x) {
#if defined(__CUDA_ARCH__)
  return __float_as_uint(x);
#else
  std::uint32_t u;
  std::memcpy(&u, &x, sizeof(u));
  return u;
#endif
}

// 1/y for finite y with |y| in [1e-30, 1e30] (within 1 ulp; not
// correctly rounded).  The seed is the correctly rounded FP32 reciprocal
// of (float)y; both conversions between FP64 and FP32 are done on the
// bits (round to nearest even, as the conversion instruction would).
DUST2_MATH_CORE double rcp(double y) {
  const std::uint64_t u = bits_of(y);
  const std::uint64_t fe = ((u >> 52) & 0x7ff) - 1023 + 127;
  if (fe - 1 >= 252) {
    // (float)y or its reciprocal is not a normal float (or y is 0, inf,
    // NaN): convert with the instructions
    const double r0 = static_cast<double>(1.0f / static_cast<float>(y));
    double e = std::fma(-y, r0, 1.0);
    double r = std::fma(r0, e, r0);
    e = std::fma(-y, r, 1.0);
    return std::fma(r, e, r);
  }
  std::uint32_t t = static_cast<std::uint32_t>(
    (fe << 23) | ((u >> 29) & 0x7fffffu));
  const std::uint32_t rem = static_cast<std::uint32_t>(u & 0x1fffffffu);
  t += (rem > 0x10000000u || (rem == 0x10000000u && (t & 1))) ? 1 : 0;
  const float yf =
    float_from_bits(t | static_cast<std::uint32_t>((u >> 32) & 0x80000000u));
  const std::uint32_t rb = float_bits_of(1.0f / yf);
  const double r0 = from_bits(
    (static_cast<std::uint64_t>(rb & 0x80000000u) << 32) |
    ((static_cast<std::uint64_t>((rb >> 23) & 0xff) - 127 + 1023) << 52) |
    (static_cast<std::uint64_t>(rb & 0x7fffffu) << 29));
  double e = std::fma(-y, r0, 1.0);
  double r = std::fma(r0, e, r0);
  e = std::fma(-y, r, 1.0);
  return std::fma(r, e, r);
}

// 1/x for integer x in [1, 128] (correctly rounded, from a table).
DUST2_HD double recip_int(int x) {
  return DUST2_TAB(recip_int, x);
}

// log(k!) for k = 0..29, correctly rounded.  One copy per side: device
// code reads global memory (the index differs between threads, so
// constant memory would serialise).
#define DUST2_LOG_FACTORIAL_TABLE                                          \
  0.0, 0.0,                                                                \
  0x1.62e42fefa39efp-1, 0x1.cab0bfa2a2002p+0, 0x1.96ca77c922cf9p+1,        \
  0x1.326643c4479c9p+2, 0x1.a51273acf01cap+2, 0x1.10ce1f32dcc30p+3,        \
  0x1.5358e82fcb70dp+3, 0x1.99a8921a7f7cfp+3, 0x1.e357590954d15p+3,        \
  0x1.180973f3a8d74p+4, 0x1.3fcba16d50143p+4, 0x1.68d5a9c3b32cep+4,        \
  0x1.930f3df162a42p+4, 0x1.be636a63fd346p+4, 0x1.eabff061f1a84p+4,        \
  0x1.0c0a63f2f353ap+5, 0x1.2329df2d5ee52p+5, 0x1.3ab8153363985p+5,        \
  0x1.52af57aed77bep+5, 0x1.6b0a8643472a9p+5, 0x1.83c4faba84f06p+5,        \
  0x1.9cda78b856a45p+5, 0x1.b6472034e8d14p+5, 0x1.d007622cd65e7p+5,        \
  0x1.ea17f717c6794p+5, 0x1.023aeb67e4fefp+6, 0x1.0f8f18d330240p+6,        \
  0x1.1d07353917231p+6

#if defined(__CUDACC__)
__device__ const double log_factorial_table_dev[30] = {
  DUST2_LOG_FACTORIAL_TABLE};
#endif
inline const double log_factorial_table_host[30] = {
  DUST2_LOG_FACTORIAL_TABLE};

DUST2_HD double log_factorial_table(int k) {
#if defined(__CUDA_ARCH__)
  return log_factorial_table_dev[k];
#else
  return log_factorial_table_host[k];
#endif
}

// Stirling series for log Gamma(y), y >= 10.
DUST2_HD double lgamma_stirling(double y) {
  const double t = rcp(y);
  const double t2 = t * t;
  // B_2k / (2k (2k-1)), k = 7 .. 1
  double s = 0x1.a41a41a41a41ap-8;
  s = std::fma(s, t2, -0x1.f6ab0d9993c7dp-10);
  s = std::fma(s, t2, 0x1.b951e2b18ff23p-11);
  s = std::fma(s, t2, -0x1.3813813813814p-11);
  s = std::fma(s, t2, 0x1.a01a01a01a01ap-11);
  s = std::fma(s, t2, -0x1.6c16c16c16c17p-9);
  s = std::fma(s, t2, 0x1.5555555555555p-4);
  s = s * t;
  return ((y - 0.5) * log(y) - y) + (HALF_LOG_2PI + s);
}

// log Gamma(x) for x > 0 (returns +inf at 0 and NaN for x < 0 or NaN),
// computed.
DUST2_MATH_CORE double lgamma_nontable(double x) {
  if (is_nan(x) || x < 0) {
    return quiet_nan();
  }
  if (x == 0 || !is_finite(x)) {
    return infinity();
  }
  if (x < 31 && x == std::floor(x)) {
    return log_factorial_table(static_cast<int>(x) - 1);
  }
  if (x >= 10) {
    return lgamma_stirling(x);
  }
  // Shift up: Gamma(x) = Gamma(x + n) / (x (x+1) ... (x+n-1))
  double prod = x;
  double y = x + 1.0;
  while (y < 10) {
    prod = prod * y;
    y = y + 1.0;
  }
  return lgamma_stirling(y) - log(prod);
}

// log(k!) for k = 0 .. LF_TABLE_MAX in device memory (8 MiB), filled once
// per device with lgamma_nontable(k + 1) by the same code, so reading the
// table returns exactly what computing would.  Each translation unit
// holds its own pointer (no relocatable device code); it stays null, and
// lgamma computes, until the host binds it.
constexpr int LF_TABLE_MAX = 1 << 20;
#if defined(__CUDACC__)
static __constant__ const double* lf_table_ptr = nullptr;
#endif

// x as an int if x is an integer in [1, 2^21), else -1 (on the bits).
DUST2_HD int small_integer(double x) {
  const std::uint64_t u = bits_of(x);
  const int e = static_cast<int>(u >> 52) - 1023;  // sign set: e > 1023
  if (e < 0 || e > 20) {
    return -1;
  }
  const std::uint64_t m = (u & 0x000fffffffffffffull) | 0x0010000000000000ull;
  const int sh = 52 - e;
  if (m & ((1ull << sh) - 1)) {
    return -1;
  }
  return static_cast<int>(m >> sh);
}

// log Gamma(x), as lgamma_nontable; on the device integer arguments up to
// LF_TABLE_MAX + 1 are read from the table.
DUST2_HD double lgamma(double x) {
#if defined(__CUDA_ARCH__)
  const double* t = lf_table_ptr;
  if (t != nullptr) {
    const int k = small_integer(x);
    if (k >= 1 && k <= LF_TABLE_MAX + 1) {
      return t[k - 1];
    }
  }
#endif
  return lgamma_nontable(x);
}

// log(k!) for an integer-valued k >= 0.
DUST2_HD double log_factorial(double k) {
  return lgamma(k + 1.0);
}

// cos(2 pi t) and sin(2 pi t) for a turn count t.
DUST2_HD void sincos_2pi(double t, double* s_out, double* c_out) {
  // Reduce to the nearest quarter turn; t - q/4 is exact for |t| < 2^50.
  const double q = std::rint(4.0 * t);
  const double r = t - 0.25 * q;                   // |r| <= 1/8 turn
  const double x = r * 0x1.921fb54442d18p+2;       // 2 pi r, |x| <= pi/4
  const double x2 = x * x;
  // sin x = x (1 - x^2/3! + x^4/5! - ...) up to x^15
  double sp = -0x1.ae7f3e733b81fp-41;              // -1/15!
  sp = std::fma(sp, x2, 0x1.6124613a86d09p-33);    //  1/13!
  sp = std::fma(sp, x2, -0x1.ae64567f544e4p-26);   // -1/11!
  sp = std::fma(sp, x2, 0x1.71de3a556c734p-19);    //  1/9!
  sp = std::fma(sp, x2, -0x1.a01a01a01a01ap-13);   // -1/7!
  sp = std::fma(sp, x2, 0x1.1111111111111p-7);     //  1/5!
  sp = std::fma(sp, x2, -0x1.5555555555555p-3);    // -1/3!
  const double sn = std::fma(sp * x2, x, x);
  // cos x = 1 - x^2/2! + x^4/4! - ... up to x^16
  double cp = 0x1.ae7f3e733b81fp-45;               //  1/16!
  cp = std::fma(cp, x2, -0x1.93974a8c07c9dp-37);   // -1/14!
  cp = std::fma(cp, x2, 0x1.1eed8eff8d898p-29);    //  1/12!
  cp = std::fma(cp, x2, -0x1.27e4fb7789f5cp-22);   // -1/10!
  cp = std::fma(cp, x2, 0x1.a01a01a01a01ap-16);    //  1/8!
  cp = std::fma(cp, x2, -0x1.6c16c16c16c17p-10);   // -1/6!
  cp = std::fma(cp, x2, 0x1.5555555555555p-5);     //  1/4!
  cp = std::fma(cp, x2, -0.5);                     // -1/2!
  const double cs = std::fma(cp, x2, 1.0);
  const int quadrant = static_cast<int>(q - 4.0 * std::floor(0.25 * q));
  switch (quadrant) {
  case 0: *s_out = sn; *c_out = cs; break;
  case 1: *s_out = cs; *c_out = -sn; break;
  case 2: *s_out = -sn; *c_out = -cs; break;
  default: *s_out = -cs; *c_out = sn; break;
  }
}

}  // namespace math
}  // namespace dust2gpu
