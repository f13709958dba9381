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
//   exp    table-driven (Tang 1989): x = (128 k + j) ln2/128 + r with a
//          two-part ln2/128 (exact k * hi), |r| <= ln2/256, then
//          2^(j/128) (double-double table) * (1 + expm1(r)), expm1 by its
//          Taylor polynomial through r^5, scaled by 2^k.
//   log    table-driven (Tang 1990): x = 2^e m, m in [sqrt(2)/2, sqrt(2)),
//          F = j/256 nearest to m, r = (m - F) * (1/F) (m - F exact), then
//          log(x) = e ln2 + log(F) (double-double table) + log1p(r) by its
//          Taylor polynomial through r^7.
//   rcp    1/y from the correctly rounded FP32 reciprocal of (float)y
//          (cheap on this GPU) refined by two Newton steps in FP64 FMA.
//   lgamma for x > 0: exact table of log(k!) for integer arguments below
//          30; otherwise the argument is shifted up to >= 10 with the
//          recurrence Gamma(x+1) = x Gamma(x) and the Stirling series
//          with Bernoulli coefficients B_2k / (2k (2k-1)), k = 1..7.
//   cos_2pi / sin_2pi (argument in turns) for the Box-Muller transform:
//          quadrant reduction on the turn count (exact), then Taylor
//          series of cos and sin on |x| <= pi/4.
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
DUST2_TABLE(log_inv, DUST2_LOG_N, DUST2_LOG_INV)
DUST2_TABLE(log_hi, DUST2_LOG_N, DUST2_LOG_HI)
DUST2_TABLE(log_lo, DUST2_LOG_N, DUST2_LOG_LO)
DUST2_TABLE(recip_int, 129, DUST2_RECIP_INT)

DUST2_HD double exp(double x) {
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
  // expm1(r) = r + r^2 (1/2 + r (1/6 + r (1/24 + r / 120)))
  double p = std::fma(r, 0x1.1111111111111p-7, 0x1.5555555555555p-5);
  p = std::fma(p, r, 0x1.5555555555555p-3);
  p = std::fma(p, r, 0.5);
  const double pm1 = std::fma(r * r, p, r);
  const double t_hi = DUST2_TAB(exp2_hi, j);
  const double t_lo = DUST2_TAB(exp2_lo, j);
  return scale2(t_hi + std::fma(t_hi, pm1, t_lo), e);
}

DUST2_HD double log(double x) {
  if (is_nan(x) || x < 0) {
    return quiet_nan();
  }
  if (x == 0) {
    return -infinity();
  }
  if (!is_finite(x)) {
    return x;
  }
  std::uint64_t u = bits_of(x);
  int e = static_cast<int>(u >> 52) - 1023;
  if (e == -1023) {
    // subnormal: renormalise exactly
    u = bits_of(x * 0x1p54);
    e = static_cast<int>(u >> 52) - 1023 - 54;
  }
  double m = from_bits((u & 0x000fffffffffffffull) | 0x3ff0000000000000ull);
  if (m > SQRT2) {
    m = from_bits((bits_of(m) & 0x000fffffffffffffull) | 0x3fe0000000000000ull);
    e += 1;
  }
  const int j = static_cast<int>(std::rint(m * 256.0));
  const double f = m - static_cast<double>(j) * 0x1p-8;  // exact
  const int i = j - DUST2_LOG_J0;
  const double r = f * DUST2_TAB(log_inv, i);
  // log1p(r) = r + r^2 (-1/2 + r (1/3 + r (-1/4 + r (1/5 + r (-1/6 + r/7)))))
  double p = std::fma(r, 0x1.2492492492492p-3, -0x1.5555555555555p-3);
  p = std::fma(p, r, 0x1.999999999999ap-3);
  p = std::fma(p, r, -0.25);
  p = std::fma(p, r, 0x1.5555555555555p-2);
  p = std::fma(p, r, -0.5);
  const double lp = std::fma(r * r, p, r);
  const double ef = static_cast<double>(e);
  const double hi = std::fma(ef, LN2_HI, DUST2_TAB(log_hi, i));
  const double lo = std::fma(ef, LN2_LO, DUST2_TAB(log_lo, i)) + lp;
  return hi + lo;
}

// 1/y for finite y with |y| in [1e-30, 1e30] (within 1 ulp; not
// correctly rounded).
DUST2_HD double rcp(double y) {
  const double r0 =
    static_cast<double>(1.0f / static_cast<float>(y));
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

// log Gamma(x) for x > 0 (returns +inf at 0 and NaN for x < 0 or NaN).
DUST2_HD double lgamma(double x) {
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
