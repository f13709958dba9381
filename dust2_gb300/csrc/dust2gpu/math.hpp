// Project-owned FP64 elementary functions, identical on host and device.
//
// dust2 draws its random variates through monty (an external package that
// is not available here), and monty's samplers evaluate exp/log/lgamma.
// Platform libm implementations (glibc, CUDA) differ in the last bit, so
// the particle trajectories of a CPU run and a GPU run would drift apart
// after the first differently-rounded draw.  Everything here is therefore
// written from textbook methods using only correctly rounded IEEE
// operations, so that the host oracle and the kernels produce identical
// bits:
//
//   exp    Cody & Waite (1980) additive range reduction x = k ln2 + r,
//          |r| <= ln2/2, then the Taylor series of e^r to degree 13 in
//          Horner form (truncation < 5e-18 relative), scaled by 2^k.
//   log    x = 2^e m with m in [sqrt(2)/2, sqrt(2)), then
//          log(m) = 2 atanh(s), s = (m-1)/(m+1), summed as the odd series
//          2 s^(2k+1)/(2k+1) in s^2 (11 terms), recombined in the
//          "f - (hf^2/2 - s (hf^2/2 + R))" form that keeps the leading
//          term exact.
//   lgamma for x > 0: exact table of log(k!) for integer arguments below
//          30; otherwise the argument is shifted up to >= 10 with the
//          recurrence Gamma(x+1) = x Gamma(x) and the Stirling series
//          with Bernoulli coefficients B_2k / (2k (2k-1)), k = 1..7.
//   cos_2pi / sin_2pi (argument in turns) for the Box-Muller transform:
//          quadrant reduction on the turn count (exact), then Taylor
//          series of cos and sin on |x| <= pi/4.
//
// All constants below are the correctly rounded doubles of the stated
// exact rationals or mathematical constants.
#pragma once

#include <cmath>
#include <cstdint>
#include <cstring>
#include <limits>

#include "common.hpp"

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
  const double kf = std::rint(x * LOG2E);
  const int k = static_cast<int>(kf);
  double r = std::fma(-kf, LN2_HI, x);
  r = std::fma(-kf, LN2_LO, r);
  // Taylor coefficients 1/j!, j = 13 .. 0
  double p = 0x1.6124613a86d09p-33;
  p = std::fma(p, r, 0x1.1eed8eff8d898p-29);
  p = std::fma(p, r, 0x1.ae64567f544e4p-26);
  p = std::fma(p, r, 0x1.27e4fb7789f5cp-22);
  p = std::fma(p, r, 0x1.71de3a556c734p-19);
  p = std::fma(p, r, 0x1.a01a01a01a01ap-16);
  p = std::fma(p, r, 0x1.a01a01a01a01ap-13);
  p = std::fma(p, r, 0x1.6c16c16c16c17p-10);
  p = std::fma(p, r, 0x1.1111111111111p-7);
  p = std::fma(p, r, 0x1.5555555555555p-5);
  p = std::fma(p, r, 0x1.5555555555555p-3);
  p = std::fma(p, r, 0x1.0000000000000p-1);
  p = std::fma(p, r, 1.0);
  p = std::fma(p, r, 1.0);
  return scale2(p, k);
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
  const double f = m - 1.0;  // exact (Sterbenz)
  const double s = f / (2.0 + f);
  const double z = s * s;
  // R = sum_{k>=1} 2 z^k / (2k+1), k = 1..11
  double R = 0x1.642c8590b2164p-4;
  R = std::fma(R, z, 0x1.8618618618618p-4);
  R = std::fma(R, z, 0x1.af286bca1af28p-4);
  R = std::fma(R, z, 0x1.e1e1e1e1e1e1ep-4);
  R = std::fma(R, z, 0x1.1111111111111p-3);
  R = std::fma(R, z, 0x1.3b13b13b13b14p-3);
  R = std::fma(R, z, 0x1.745d1745d1746p-3);
  R = std::fma(R, z, 0x1.c71c71c71c71cp-3);
  R = std::fma(R, z, 0x1.2492492492492p-2);
  R = std::fma(R, z, 0x1.999999999999ap-2);
  R = std::fma(R, z, 0x1.5555555555555p-1);
  R = R * z;
  const double hfsq = 0.5 * f * f;
  const double logm = f - (hfsq - s * (hfsq + R));
  const double ef = static_cast<double>(e);
  return std::fma(ef, LN2_HI, std::fma(ef, LN2_LO, logm));
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
  const double t = 1.0 / y;
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
