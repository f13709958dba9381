// Random variates drawn from a per-particle stream, identical on host and
// device.
//
// dust2 calls these through monty (monty::random::binomial, poisson,
// exponential_rate, normal; call sites inst/examples/sir.cpp:63-66,116,
// walk.cpp:58,75).  monty is not available in this build, so the
// samplers are restated here from the published algorithms monty
// documents:
//   binomial  inversion (Kachitvichyanukul & Schmeiser 1988, "BINV") when
//             n * min(p, 1-p) < 10, otherwise BTRS, the transformed
//             rejection method with squeeze of Hormann (1993), "The
//             generation of binomial random variates", J. Stat. Comput.
//             Simul. 46:101-110.  p > 1/2 is handled by symmetry.
//   poisson   multiplication of uniforms (Knuth, TAOCP vol 2) when
//             lambda < 10, otherwise PTRS, Hormann (1993), "The
//             transformed rejection method for generating Poisson random
//             variables", Insurance: Math. Econ. 12:39-45.
//   exponential  inversion, -log(1 - U) / rate.
//   normal    Box & Muller (1958), one variate per pair of uniforms.
//
// The constant-heavy setup of the rejection samplers (the log-factorial
// terms of BTRS, the log terms of PTRS) only feeds the final acceptance
// test, so it is evaluated lazily, the first time a candidate falls
// outside the squeeze; this changes no result.
//
// Invalid arguments do not throw (device code cannot): the sampler
// records the first error in the generator's error slot and returns NaN.
// Every rejection loop is bounded so that no input can make a kernel spin.
#pragma once

#include <cmath>

#include "common.hpp"
#include "math.hpp"
#include "random.hpp"

namespace dust2gpu {
namespace random {

// The two sampler cores are compiled once per kernel and called rather
// than inlined at every draw site: a system drawing many binomials per
// step (one per age class and transition) otherwise outgrows the
// instruction cache, and the call costs only integer-pipe instructions on
// an FP64-bound kernel.
#if defined(__CUDACC__)
#define DUST2_SAMPLER inline __host__ __device__ __noinline__
#else
#define DUST2_SAMPLER inline
#endif

// Bound on candidate draws in a rejection loop; with valid arguments the
// acceptance rate is above 0.8, so reaching this means corrupt input.
constexpr int MAX_REJECTION_ATTEMPTS = 100000;
// BINV restarts when the search passes this count (the published cap).
constexpr int BINV_MAX_X = 110;

// Comparisons whose operands are known to be non-negative (uniforms,
// probabilities, the inversion remainder) are taken on the bit patterns
// (math::gt_nonneg / le_nonneg); they decide exactly as the FP64
// comparison would.

// The recurrence f(x) = f(x-1) ((n+1) s / x - s), s = p/q, uses 1/x from
// a table, and s from a reciprocal, so the loop has no FP64 division.
// u stays >= 0 (it only loses a smaller r), so `u > r` is a bit compare.
// The terms that depend on p only (q = 1 - p, s = p * rcp(q), log q) are
// arguments, so that a prepared probability can supply them.
DUST2_SAMPLER double binomial_inversion(rng_state& rng, double n, double p,
                                   double q, double s, double logq) {
  const double a = (n + 1.0) * s;
  const double r0 = math::exp(n * logq);  // q^n
  for (int attempt = 0; attempt < MAX_REJECTION_ATTEMPTS; ++attempt) {
    double r = r0;
    double u = random_real(rng);
    int x = 0;
    while (math::gt_nonneg(u, r)) {
      u = u - r;
      x = x + 1;
      r = r * std::fma(a, math::recip_int(x), -s);
      if (x > BINV_MAX_X) {
        break;
      }
    }
    if (x <= BINV_MAX_X) {
      return static_cast<double>(x);
    }
  }
  set_error(rng, ERR_BINOMIAL_INVALID, n, p);
  return math::quiet_nan();
}

// Divisions by b, us, q and the hat denominator are multiplications by
// reciprocals (math::rcp); us = 0 (u = -1/2 exactly) is rejected.  Here
// n p >= 10 and q >= 1/2, so b > 6.8 and v_r > 0.3.  log(p / q) of the
// acceptance test is given by a prepared probability (lpq_given, always
// finite there), or, when lpq_given is NaN, computed the first time a
// candidate needs that test; one body serves both, so a kernel holds one
// copy of the sampler.
DUST2_SAMPLER double binomial_btrs(rng_state& rng, double n, double p, double q,
                                   double lpq_given) {
  const double spq = std::sqrt(n * p * q);
  const double b = std::fma(2.53, spq, 1.15);
  const double a = std::fma(0.01, p, std::fma(0.0248, b, -0.0873));
  const double a2 = math::twice_normal(a);  // a > 0.08
  const double c = std::fma(n, p, 0.5);
  const double inv_b = math::rcp(b);
  const double v_r = std::fma(-4.2, inv_b, 0.92);
  const std::int64_t n_bits = static_cast<std::int64_t>(math::bits_of(n));
  bool have_setup = false;
  double alpha = 0, lpq = 0, m = 0, h = 0;
  for (int attempt = 0; attempt < MAX_REJECTION_ATTEMPTS; ++attempt) {
    double u, us;  // U - 1/2 and 1/2 - |U - 1/2|, us >= +0
    centered_uniform(rng, &u, &us);
    double v = random_real(rng);
    if (math::bits_of(us) == 0) {
      continue;
    }
    const double inv_us = math::rcp(us);
    const double k = math::floor_bits(std::fma(std::fma(a2, inv_us, b), u, c));
    if (math::le_nonneg(0.07, us) && math::le_nonneg(v, v_r)) {
      return k;
    }
    // k < 0 || k > n (k is never -0: the floored sum is >= -0.5 + c > 0
    // or an exact negative integer)
    const std::int64_t k_bits = static_cast<std::int64_t>(math::bits_of(k));
    if (k_bits < 0 || k_bits > n_bits) {
      continue;
    }
    if (!have_setup) {
      alpha = std::fma(5.1, inv_b, 2.83) * spq;
      lpq = math::is_nan(lpq_given) ? math::log(p * math::rcp(q)) :
        lpq_given;
      m = math::floor_bits((n + 1.0) * p);
      h = math::log_factorial(m) + math::log_factorial(n - m);
      have_setup = true;
    }
    v = math::log(v * alpha * math::rcp(std::fma(a * inv_us, inv_us, b)));
    if (v <= std::fma(k - m, lpq, h - math::log_factorial(k) -
                      math::log_factorial(n - k))) {
      return k;
    }
  }
  set_error(rng, ERR_BINOMIAL_INVALID, n, p);
  return math::quiet_nan();
}

constexpr std::uint64_t BITS_MINUS_ZERO = 0x8000000000000000ull;
constexpr std::uint64_t BITS_ONE = 0x3ff0000000000000ull;
constexpr std::uint64_t BITS_HALF = 0x3fe0000000000000ull;
constexpr std::uint64_t BITS_TEN = 0x4024000000000000ull;

// n >= 0 and finite (-0 included), on the bits.
DUST2_HD bool binomial_n_ok(std::uint64_t nb) {
  return nb < 0x7ff0000000000000ull || nb == BITS_MINUS_ZERO;
}

// Binomial(n, p) for integer-valued n >= 0 and p in [0, 1].  The argument
// checks are taken on the bit patterns, with the FP64 semantics of
// !(n >= 0) || !finite(n) || !(p >= 0) || !(p <= 1) (so -0 is valid).
DUST2_HD double binomial(rng_state& rng, double n, double p) {
  const std::uint64_t nb = math::bits_of(n);
  const std::uint64_t pb = math::bits_of(p);
  const bool p_ok = pb <= BITS_ONE || pb == BITS_MINUS_ZERO;
  if (!binomial_n_ok(nb) || !p_ok) {
    set_error(rng, ERR_BINOMIAL_INVALID, n, p);
    return math::quiet_nan();
  }
  if (rng.deterministic) {
    return n * p;
  }
  if ((nb << 1) == 0 || (pb << 1) == 0) {  // n == 0 || p == 0
    return 0;
  }
  if (pb == BITS_ONE) {  // p == 1
    return n;
  }
  const bool flip = pb > BITS_HALF;  // p > 1/2
  const double pp = flip ? 1.0 - p : p;
  const double q = 1.0 - pp;
  // n * pp < 10 (n * pp is positive and finite)
  double x;
  if (math::bits_of(n * pp) < BITS_TEN) {
    const double s = pp * math::rcp(q);
    x = binomial_inversion(rng, n, pp, q, s, math::log(q));
  } else {
    x = binomial_btrs(rng, n, pp, q, math::quiet_nan());
  }
  return flip ? n - x : x;
}

// A probability prepared for many Binomial draws (the same p for several
// counts, as a system drawing one transition per age class does): the
// terms of both samplers that depend on p alone, evaluated once by the
// expressions binomial() uses, so binomial(rng, n, binomial_prepare(p))
// returns exactly binomial(rng, n, p) and consumes the same draws.
struct binomial_prob {
  double p;     // as given
  double pp;    // min(p, 1 - p)
  double q;     // 1 - pp
  double s;     // pp * rcp(q)
  double logq;  // log(q)
  double lpq;   // log(s)
  std::uint64_t bits;
  bool valid;
  bool flip;
};

DUST2_HD binomial_prob binomial_prepare(double p) {
  binomial_prob b{};
  b.p = p;
  b.bits = math::bits_of(p);
  b.valid = b.bits <= BITS_ONE || b.bits == BITS_MINUS_ZERO;
  b.flip = b.valid && b.bits > BITS_HALF;
  b.pp = b.flip ? 1.0 - p : p;
  if (b.valid && (b.bits << 1) != 0 && b.bits != BITS_ONE) {
    b.q = 1.0 - b.pp;
    b.s = b.pp * math::rcp(b.q);
    b.logq = math::log(b.q);
    b.lpq = math::log(b.s);
  }
  return b;
}

DUST2_HD double binomial(rng_state& rng, double n, const binomial_prob& b) {
  const std::uint64_t nb = math::bits_of(n);
  if (!binomial_n_ok(nb) || !b.valid) {
    set_error(rng, ERR_BINOMIAL_INVALID, n, b.p);
    return math::quiet_nan();
  }
  if (rng.deterministic) {
    return n * b.p;
  }
  if ((nb << 1) == 0 || (b.bits << 1) == 0) {
    return 0;
  }
  if (b.bits == BITS_ONE) {
    return n;
  }
  double x;
  if (math::bits_of(n * b.pp) < BITS_TEN) {
    x = binomial_inversion(rng, n, b.pp, b.q, b.s, b.logq);
  } else {
    x = binomial_btrs(rng, n, b.pp, b.q, b.lpq);
  }
  return b.flip ? n - x : x;
}

DUST2_HD double poisson_knuth(rng_state& rng, double lambda) {
  const double enlam = math::exp(-lambda);  // > 0 for lambda < 10
  double prod = 1.0;
  for (int x = 0; x < MAX_REJECTION_ATTEMPTS; ++x) {
    prod = prod * random_real(rng);
    if (math::le_nonneg(prod, enlam)) {
      return x;
    }
  }
  set_error(rng, ERR_POISSON_INVALID, lambda, 0);
  return math::quiet_nan();
}

// lambda >= 10, so b > 8.9 and vr > 0.4.
DUST2_HD double poisson_ptrs(rng_state& rng, double lambda) {
  const double slam = std::sqrt(lambda);
  const double b = std::fma(2.53, slam, 0.931);
  const double a = std::fma(0.02483, b, -0.059);
  const double a2 = math::twice_normal(a);  // a > 0.16
  const double c = lambda + 0.43;
  const double vr = std::fma(-3.6224, math::rcp(b - 2.0), 0.9277);
  bool have_setup = false;
  double log_invalpha = 0, loglam = 0;
  for (int attempt = 0; attempt < MAX_REJECTION_ATTEMPTS; ++attempt) {
    double u, us;  // U - 1/2 and 1/2 - |U - 1/2|, us >= +0
    centered_uniform(rng, &u, &us);
    const double v = random_real(rng);
    if (math::bits_of(us) == 0) {
      continue;
    }
    const double inv_us = math::rcp(us);
    const double k = math::floor_bits(std::fma(std::fma(a2, inv_us, b), u, c));
    if (math::le_nonneg(0.07, us) && math::le_nonneg(v, vr)) {
      return k;
    }
    // k < 0 || (us < 0.013 && v > us); k is never -0
    if (static_cast<std::int64_t>(math::bits_of(k)) < 0 ||
        (!math::le_nonneg(0.013, us) && !math::le_nonneg(v, us))) {
      continue;
    }
    if (!have_setup) {
      log_invalpha = math::log(std::fma(1.1328, math::rcp(b - 3.4), 1.1239));
      loglam = math::log(lambda);
      have_setup = true;
    }
    if (math::log(v) + log_invalpha -
        math::log(std::fma(a * inv_us, inv_us, b)) <=
        std::fma(k, loglam, -lambda) - math::log_factorial(k)) {
      return k;
    }
  }
  set_error(rng, ERR_POISSON_INVALID, lambda, 0);
  return math::quiet_nan();
}

// Poisson(lambda) for lambda >= 0 (checks on the bits, with the FP64
// semantics of !(lambda >= 0) || !finite(lambda)).
DUST2_HD double poisson(rng_state& rng, double lambda) {
  const std::uint64_t lb = math::bits_of(lambda);
  if (!(lb < 0x7ff0000000000000ull || lb == 0x8000000000000000ull)) {
    set_error(rng, ERR_POISSON_INVALID, lambda, 0);
    return math::quiet_nan();
  }
  if (rng.deterministic) {
    return lambda;
  }
  if ((lb << 1) == 0) {
    return 0;
  }
  return lb < BITS_TEN ? poisson_knuth(rng, lambda) :
    poisson_ptrs(rng, lambda);
}

DUST2_HD double exponential_rate(rng_state& rng, double rate) {
  if (rng.deterministic) {
    return 1.0 / rate;
  }
  return -math::log(1.0 - random_real(rng)) / rate;
}

DUST2_HD double uniform(rng_state& rng, double min, double max) {
  if (rng.deterministic) {
    return 0.5 * (min + max);
  }
  return min + (max - min) * random_real(rng);
}

DUST2_HD double normal(rng_state& rng, double mean, double sd) {
  if (rng.deterministic) {
    return mean;
  }
  const double u1 = 1.0 - random_real(rng);  // (0, 1]
  const double u2 = random_real(rng);
  double s, c;
  math::sincos_2pi(u2, &s, &c);
  const double z = std::sqrt(-2.0 * math::log(u1)) * c;
  return mean + sd * z;
}

}  // namespace random

namespace density {

// log Poisson(x | lambda), with 0 log 0 = 0.
DUST2_HD double poisson(double x, double lambda, bool log) {
  double ret;
  if (x == 0 && lambda == 0) {
    ret = 0;
  } else {
    ret = x * math::log(lambda) - lambda - math::lgamma(x + 1.0);
  }
  return log ? ret : math::exp(ret);
}

// log NegBinomial(x | size, mu), mean/size parameterisation.
DUST2_HD double negative_binomial_mu(double x, double size, double mu,
                                     bool log) {
  double ret;
  if (x == 0 && mu == 0) {
    ret = 0;
  } else {
    const double lsm = math::log(size + mu);
    ret = math::lgamma(x + size) - math::lgamma(size) -
      math::lgamma(x + 1.0) + size * (math::log(size) - lsm) +
      x * (math::log(mu) - lsm);
  }
  return log ? ret : math::exp(ret);
}

// x log y with 0 log 0 = 0.
DUST2_HD double x_log_y(double x, double y) {
  return (x == 0 && y == 0) ? 0 : x * math::log(y);
}

// log Binomial(x | size, prob): log C(size, x) + x log p
// + (size - x) log(1 - p), with 0 log 0 = 0 (so p = 0 or 1 give 0 or -Inf
// without special cases).
DUST2_HD double binomial(double x, double size, double prob, bool log) {
  double ret;
  if (x == 0 && size == 0) {
    ret = 0;
  } else {
    ret = math::lgamma(size + 1.0) - math::lgamma(x + 1.0) -
      math::lgamma(size - x + 1.0) + x_log_y(x, prob) +
      x_log_y(size - x, 1 - prob);
  }
  return log ? ret : math::exp(ret);
}

DUST2_HD double normal(double x, double mu, double sd, bool log) {
  const double z = (x - mu) / sd;
  const double ret = -0.5 * z * z - math::log(sd) - math::HALF_LOG_2PI;
  return log ? ret : math::exp(ret);
}

}  // namespace density
}  // namespace dust2gpu
