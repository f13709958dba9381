// TEST INFRASTRUCTURE (oracle): algorithmic FP64 operation counts of the
// step + compare work of the discrete filter, per particle-step.
//
// The update and compare of the SIR (sir_cases) and age-structured SEIR
// (seir_age) systems and the binomial sampler they call (BINV inversion
// and Hormann's BTRS, with the prepared-probability form) are restated
// here over `counted`, a real type that counts every floating-point
// operation it performs: +, -, *, / and sqrt count one flop each, a
// fused multiply-add two; comparisons, floors and the elementary
// functions (exp, log, log k!, lgamma) are counted separately as calls.
// The expressions are the engine's own formulation (a reciprocal counts
// as one division, 2a as one multiplication), and every value is
// computed with the engine's functions (dust2_gb300/csrc/dust2gpu), so
// the counted run draws exactly what the engine and the oracle port
// draw: opcount_filter returns the filter's log-likelihoods, and the
// caller checks them against the port's bit for bit before trusting the
// counts.
//
// The filter around the counted work (dust2's filter.hpp:42-104:
// run_to_time with zero_every, compare, scale_log_weights,
// resample_weight, reorder) is plain double arithmetic and not counted.
// References: the samplers follow monty's published algorithms as
// restated in dust2gpu/distributions.hpp; the systems follow
// inst/examples/sir.cpp:38-120 in structure.
//
// Build: g++ -std=c++17 -O2 -ffp-contract=off (oracle/build.py).
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <limits>
#include <string>
#include <vector>

#include "systems/seir_age.hpp"
#include "systems/sir_cases.hpp"
#include "systems/sirode.hpp"

namespace {

namespace m = dust2gpu::math;
namespace rnd = dust2gpu::random;
using rng_t = rnd::rng_state;

// operation counters: [add, mul, div, fma, sqrt, cmp, floor, exp, log,
// log_factorial, lgamma, pow]
enum { ADD, MUL, DIV, FMA, SQRT, CMP, FLOOR, EXP, LOG, LFACT, LGAMMA, POW,
       NOPS };
std::uint64_t g_ops[NOPS];

struct counted {
  double v;
  counted() = default;
  constexpr counted(double x) : v(x) {}  // NOLINT: literals and inputs
};

counted operator+(counted a, counted b) { ++g_ops[ADD]; return a.v + b.v; }
counted operator-(counted a, counted b) { ++g_ops[ADD]; return a.v - b.v; }
counted operator-(counted a) { return -a.v; }  // a sign flip
counted operator*(counted a, counted b) { ++g_ops[MUL]; return a.v * b.v; }
counted operator/(counted a, counted b) { ++g_ops[DIV]; return a.v / b.v; }
bool operator<=(counted a, counted b) { ++g_ops[CMP]; return a.v <= b.v; }
bool operator<(counted a, counted b) { ++g_ops[CMP]; return a.v < b.v; }
bool operator>(counted a, counted b) { ++g_ops[CMP]; return a.v > b.v; }
bool operator==(counted a, counted b) { ++g_ops[CMP]; return a.v == b.v; }
counted fma(counted a, counted b, counted c) {
  ++g_ops[FMA];
  return std::fma(a.v, b.v, c.v);
}
counted sqrt(counted a) { ++g_ops[SQRT]; return std::sqrt(a.v); }
counted rcp(counted a) { ++g_ops[DIV]; return m::rcp(a.v); }
counted recip_int(int x) { ++g_ops[DIV]; return m::recip_int(x); }
counted twice(counted a) { ++g_ops[MUL]; return m::twice_normal(a.v); }
counted floor(counted a) { ++g_ops[FLOOR]; return m::floor_bits(a.v); }
counted exp(counted a) { ++g_ops[EXP]; return m::exp(a.v); }
counted log(counted a) { ++g_ops[LOG]; return m::log(a.v); }
counted log_factorial(counted a) {
  ++g_ops[LFACT];
  return m::log_factorial(a.v);
}
counted lgamma(counted a) { ++g_ops[LGAMMA]; return m::lgamma(a.v); }
counted pow(counted a, counted b) { ++g_ops[POW]; return std::pow(a.v, b.v); }
counted max(counted a, counted b) { ++g_ops[CMP]; return std::max(a.v, b.v); }
counted min(counted a, counted b) { ++g_ops[CMP]; return std::min(a.v, b.v); }
counted abs(counted a) { return std::abs(a.v); }  // a sign clear

// The uniform's centred forms U - 1/2 and 1/2 - |U - 1/2|: two additions.
void centered(rng_t& rng, counted* u, counted* us) {
  double a, b;
  rnd::centered_uniform(rng, &a, &b);
  g_ops[ADD] += 2;
  *u = a;
  *us = b;
}

constexpr int MAX_ATTEMPTS = 100000;
constexpr int BINV_MAX_X = 110;

// BINV (dust2gpu/distributions.hpp binomial_inversion)
counted binomial_inversion(rng_t& rng, counted n, counted s, counted logq) {
  const counted a = (n + 1.0) * s;
  const counted r0 = exp(n * logq);
  for (int attempt = 0; attempt < MAX_ATTEMPTS; ++attempt) {
    counted r = r0;
    counted u = rnd::random_real(rng);
    int x = 0;
    while (u > r) {
      u = u - r;
      x = x + 1;
      r = r * fma(a, recip_int(x), -s);
      if (x > BINV_MAX_X) {
        break;
      }
    }
    if (x <= BINV_MAX_X) {
      return static_cast<double>(x);
    }
  }
  return std::numeric_limits<double>::quiet_NaN();
}

// BTRS (dust2gpu/distributions.hpp binomial_btrs); log(p / q) comes from
// a prepared probability when lpq_ready, else it is computed the first
// time a candidate needs the full acceptance test.
counted binomial_btrs(rng_t& rng, counted n, counted p, counted q,
                      bool lpq_ready, counted lpq_given) {
  const counted spq = sqrt(n * p * q);
  const counted b = fma(2.53, spq, 1.15);
  const counted a = fma(0.01, p, fma(0.0248, b, -0.0873));
  const counted a2 = twice(a);
  const counted c = fma(n, p, 0.5);
  const counted inv_b = rcp(b);
  const counted v_r = fma(-4.2, inv_b, 0.92);
  bool have_setup = false;
  counted alpha = 0, lpq = 0, mm = 0, h = 0;
  for (int attempt = 0; attempt < MAX_ATTEMPTS; ++attempt) {
    counted u, us;
    centered(rng, &u, &us);
    counted v = rnd::random_real(rng);
    if (us == 0.0) {
      continue;
    }
    const counted inv_us = rcp(us);
    const counted k = floor(fma(fma(a2, inv_us, b), u, c));
    if (counted(0.07) <= us && v <= v_r) {
      return k;
    }
    if (k < 0.0 || k > n) {
      continue;
    }
    if (!have_setup) {
      alpha = fma(5.1, inv_b, 2.83) * spq;
      lpq = lpq_ready ? lpq_given : log(p * rcp(q));
      mm = floor((n + 1.0) * p);
      h = log_factorial(mm) + log_factorial(n - mm);
      have_setup = true;
    }
    v = log(v * alpha * rcp(fma(a * inv_us, inv_us, b)));
    if (v <= fma(k - mm, lpq, h - log_factorial(k) - log_factorial(n - k))) {
      return k;
    }
  }
  return std::numeric_limits<double>::quiet_NaN();
}

// The prepared probability (binomial_prepare): the p-only terms.
struct prob {
  counted p, pp, q, s, logq, lpq;
  bool trivial, flip;
};

prob prepare(counted p) {
  prob b{};
  b.p = p;
  b.trivial = p.v == 0 || p.v == 1;
  b.flip = p.v > 0.5;
  ++g_ops[CMP];
  b.pp = b.flip ? 1.0 - p : p;
  if (!b.trivial) {
    b.q = 1.0 - b.pp;
    b.s = b.pp * rcp(b.q);
    b.logq = log(b.q);
    b.lpq = log(b.s);
  }
  return b;
}

// binomial(rng, n, prepared p): the argument checks and the n == 0 / p
// == 0 / p == 1 shortcuts are integer work on the bit patterns.
counted binomial(rng_t& rng, counted n, const prob& b) {
  if (n.v == 0 || b.trivial) {
    return b.p.v == 1 ? n : counted(0.0);
  }
  counted x;
  if (n * b.pp < 10.0) {
    x = binomial_inversion(rng, n, b.s, b.logq);
  } else {
    x = binomial_btrs(rng, n, b.pp, b.q, true, b.lpq);
  }
  return b.flip ? n - x : x;
}

// binomial(rng, n, p) with its own set-up (distributions.hpp binomial)
counted binomial(rng_t& rng, counted n, counted p) {
  if (n.v == 0 || p.v == 0) {
    return 0.0;
  }
  if (p.v == 1) {
    return n;
  }
  const bool flip = p.v > 0.5;
  ++g_ops[CMP];
  const counted pp = flip ? 1.0 - p : p;
  const counted q = 1.0 - pp;
  counted x;
  if (n * pp < 10.0) {
    const counted s = pp * rcp(q);
    x = binomial_inversion(rng, n, s, log(q));
  } else {
    x = binomial_btrs(rng, n, pp, q, false, 0.0);
  }
  return flip ? n - x : x;
}

// ---- systems (dust2gpu/systems/sir_cases.hpp, seir_age.hpp) ----

struct sir_counted {
  using sys = dust2gpu::systems::sir_cases;
  static constexpr int n_state = 4;
  struct internal {
    bool ready = false;
    prob b_IR;
  };
  static void update(double dt, const counted* state,
                     const sys::shared_state& shared, internal& in,
                     rng_t& rng, counted* next) {
    const counted S = state[0], I = state[1], R = state[2], inc = state[3];
    const counted p_SI =
      1.0 - exp(-counted(shared.beta) * I / counted(shared.N) * dt);
    if (!in.ready) {  // the engine prepares it once per particle
      in.b_IR = prepare(1.0 - exp(-counted(shared.gamma) * dt));
      in.ready = true;
    }
    const counted n_SI = binomial(rng, S, p_SI);
    const counted n_IR = binomial(rng, I, in.b_IR);
    next[0] = S - n_SI;
    next[1] = I + n_SI - n_IR;
    next[2] = R + n_IR;
    next[3] = inc + n_SI;
  }
  static counted compare(const counted* state, double obs,
                         const sys::shared_state&) {
    if (std::isnan(obs)) {
      return 0.0;
    }
    const counted lambda = state[3] + 1e-6;
    const counted x = obs;
    if (x.v == 0 && lambda.v == 0) {
      return 0.0;
    }
    return x * log(lambda) - lambda - lgamma(x + 1.0);
  }
};

struct seir_counted {
  using sys = dust2gpu::systems::seir_age;
  static constexpr int A = sys::n_age;
  static constexpr int n_state = 6 * A;
  struct internal {};
  static void update(double dt, const counted* state,
                     const sys::shared_state& sh, internal&, rng_t& rng,
                     counted* next) {
    const counted* S = state;
    const counted* E = state + A;
    const counted* I = state + 2 * A;
    const counted* R = state + 3 * A;
    const counted* cum = state + 4 * A;
    const counted* inc = state + 5 * A;
    counted x[A];
    for (int b = 0; b < A; ++b) {
      x[b] = I[b] * sh.inv_N[b];
    }
    const counted p_EI = 1.0 - exp(-counted(sh.sigma) * dt);
    const counted p_IR = 1.0 - exp(-counted(sh.gamma) * dt);
    const prob b_EI = prepare(p_EI);
    const prob b_IR = prepare(p_IR);
    for (int a = 0; a < A; ++a) {
      counted acc = 0.0;
      for (int b = 0; b < A; ++b) {
        acc = fma(sh.contact[a][b], x[b], acc);
      }
      const counted lambda = counted(sh.beta) * acc;
      const counted p_SE = 1.0 - exp(-lambda * dt);
      const counted n_SE = binomial(rng, S[a], p_SE);
      const counted n_EI = binomial(rng, E[a], b_EI);
      const counted n_IR = binomial(rng, I[a], b_IR);
      next[a] = S[a] - n_SE;
      next[A + a] = E[a] + n_SE - n_EI;
      next[2 * A + a] = I[a] + n_EI - n_IR;
      next[3 * A + a] = R[a] + n_IR;
      next[4 * A + a] = cum[a] + n_EI;
      next[5 * A + a] = inc[a] + n_EI;
    }
  }
  static counted compare(const counted* state, double obs,
                         const sys::shared_state& sh) {
    if (std::isnan(obs)) {
      return 0.0;
    }
    counted mu = 0.0;
    for (int a = 0; a < A; ++a) {
      mu = mu + state[5 * A + a];
    }
    mu = mu + 1e-6;
    const counted x = obs, size = sh.size;
    if (x.v == 0 && mu.v == 0) {
      return 0.0;
    }
    const counted lsm = log(size + mu);
    return lgamma(x + size) - lgamma(size) - lgamma(x + 1.0) +
      size * (log(size) - lsm) + x * (log(mu) - lsm);
  }
};

// ---- the filter around the counted work (dust2 filter.hpp:42-104) ----

double scale_log_weights(size_t n, double* w) {  // filter_details.hpp:11-39
  if (n == 1) {
    return *w;
  }
  const double ninf = -std::numeric_limits<double>::infinity();
  double max_w = ninf;
  for (size_t i = 0; i < n; ++i) {
    if (std::isnan(w[i])) {
      w[i] = ninf;
    } else {
      max_w = std::max(max_w, w[i]);
    }
  }
  if (max_w == ninf) {
    return max_w;
  }
  double tot = 0.0;
  for (size_t i = 0; i < n; ++i) {
    w[i] = std::exp(w[i] - max_w);
    tot += w[i];
  }
  return std::log(tot / n) + max_w;
}

void resample_weight(size_t n, const double* w, double u,
                     size_t* idx) {  // filter_details.hpp:45-74
  double tot = 0.0;
  for (size_t i = 0; i < n; ++i) {
    tot += w[i];
  }
  const double uu0 = tot * u / n;
  const double du = tot / n;
  double ww = 0.0;
  size_t j = 0;
  for (size_t i = 0; i < n; ++i) {
    const double uu = uu0 + i * du;
    while (ww < uu && j < n) {
      ww += w[j];
      ++j;
    }
    idx[i] = j == 0 ? 0 : j - 1;
  }
}

rng_t make_rng(const std::uint64_t* w) {
  rng_t r{};
  for (int i = 0; i < 4; ++i) {
    r.state[i] = w[i];
  }
  r.deterministic = false;
  return r;
}

// One group: initial conditions at time_start, then for each data time
// its steps (zero_every: the daily incidence entries are cleared at whole
// times), compare, and resampling.  Only update and compare are counted.
template <typename C, typename SYS>
double filter_group(const typename SYS::shared_state& sh, int n, double dt,
                    const double* times, int n_times, const double* data,
                    int data_stride, const std::uint64_t* words,
                    std::uint64_t* step_ops, std::uint64_t* compare_ops) {
  const int ns = C::n_state;
  rng_t frng = make_rng(words);
  std::vector<rng_t> rng(n);
  for (int j = 0; j < n; ++j) {
    rng[j] = make_rng(words + 4 * (2 + j));
  }
  std::vector<counted> state(static_cast<size_t>(n) * ns),
    next(static_cast<size_t>(n) * ns);
  std::vector<typename C::internal> internal(n);
  {
    std::vector<double> init(ns);
    typename SYS::internal_state is{};
    for (int j = 0; j < n; ++j) {
      SYS::initial(0.0, sh, is, rng[j], init.data());
      for (int s = 0; s < ns; ++s) {
        state[static_cast<size_t>(j) * ns + s] = init[s];
      }
    }
  }
  const auto zero = SYS::zero_every(sh);
  double time = 0.0, ll = 0.0;
  std::vector<double> w(n);
  std::vector<size_t> idx(n);
  for (int it = 0; it < n_times; ++it) {
    const double t = times[it];
    const size_t n_steps = static_cast<size_t>(std::round((t - time) / dt));
    std::uint64_t before[NOPS];
    std::memcpy(before, g_ops, sizeof(before));
    for (int j = 0; j < n; ++j) {
      counted* y = state.data() + static_cast<size_t>(j) * ns;
      counted* yn = next.data() + static_cast<size_t>(j) * ns;
      for (size_t i = 0; i < n_steps; ++i) {
        const double time_i = time + i * dt;
        for (int z = 0; z < zero.n; ++z) {
          if (std::fmod(time_i, zero.period[z]) == 0) {
            for (int s = 0; s < ns; ++s) {
              if (zero.has(z, s)) {
                y[s] = 0.0;
              }
            }
          }
        }
        C::update(dt, y, sh, internal[j], rng[j], yn);
        std::copy(yn, yn + ns, y);
      }
    }
    for (int k = 0; k < NOPS; ++k) {
      step_ops[k] += g_ops[k] - before[k];
    }
    time += n_steps * dt;
    std::memcpy(before, g_ops, sizeof(before));
    for (int j = 0; j < n; ++j) {
      w[j] = C::compare(state.data() + static_cast<size_t>(j) * ns,
                        data[static_cast<size_t>(it) * data_stride], sh).v;
    }
    for (int k = 0; k < NOPS; ++k) {
      compare_ops[k] += g_ops[k] - before[k];
    }
    if (std::any_of(w.begin(), w.end(), [](double v) { return v != 0; })) {
      ll += scale_log_weights(n, w.data());
      const double u = rnd::random_real(frng);
      resample_weight(n, w.data(), u, idx.data());
      for (int j = 0; j < n; ++j) {
        std::copy_n(state.data() + idx[j] * ns, ns,
                    next.data() + static_cast<size_t>(j) * ns);
      }
      state.swap(next);
    }
  }
  return ll;
}

// ---- dopri5 (dust2's continuous/solver.hpp, as the oracle port) ----

// sirode's right-hand side (dust2gpu/systems/sirode.hpp)
void sirode_rhs(const dust2gpu::systems::sirode::shared_state& sh,
                const counted* y, counted* dy) {
  const counted S = y[0], I = y[1];
  const counted rate_SI = counted(sh.beta) * S * I / counted(sh.N);
  const counted rate_IR = counted(sh.gamma) * I;
  dy[0] = -rate_SI;
  dy[1] = rate_SI - rate_IR;
  dy[2] = rate_IR;
  dy[3] = rate_SI;
  dy[4] = rate_SI;
}

// One sirode instance integrated from 0 through `times` with the
// reference's unfused arithmetic (solver.hpp:96-324, 437-492; controls
// of control.hpp:11-27 with rtol = atol = 1e-6, step_size_min = DBL_EPSILON,
// no maximum step), writing the state at each time; returns the number of
// attempted steps.
struct dopri5_counted {
  static constexpr int n = 5;
  const dust2gpu::systems::sirode::shared_state& sh;
  counted atol = 1e-6, rtol = 1e-6, factor_safe = 0.9, beta = 0.04,
    constant = 0.2 - 0.04 * 0.75;
  double facc1 = 1 / 0.2, facc2 = 1 / 10.0;
  double step_size_min = std::numeric_limits<double>::epsilon();
  counted y_next[n], y_stiff[n], k2[n], k3[n], k4[n], k5[n], k6[n];
  counted dydt[n], c1[n], c2[n], c3[n], c4[n], c5[n];
  counted t0 = 0.0, h_last = 0.0, step_size = 0.0, error = 0.0;
  long n_steps = 0, n_accepted = 0;

  static constexpr double C2 = 0.2, C3 = 0.3, C4 = 0.8, C5 = 8.0 / 9.0;
  static constexpr double A21 = 0.2, A31 = 3.0 / 40.0, A32 = 9.0 / 40.0;
  static constexpr double A41 = 44.0 / 45.0, A42 = -56.0 / 15.0,
    A43 = 32.0 / 9.0;
  static constexpr double A51 = 19372.0 / 6561.0, A52 = -25360.0 / 2187.0,
    A53 = 64448.0 / 6561.0, A54 = -212.0 / 729.0;
  static constexpr double A61 = 9017.0 / 3168.0, A62 = -355.0 / 33.0,
    A63 = 46732.0 / 5247.0, A64 = 49.0 / 176.0, A65 = -5103.0 / 18656.0;
  static constexpr double A71 = 35.0 / 384.0, A73 = 500.0 / 1113.0,
    A74 = 125.0 / 192.0, A75 = -2187.0 / 6784.0, A76 = 11.0 / 84.0;
  static constexpr double E1 = 71.0 / 57600.0, E3 = -71.0 / 16695.0,
    E4 = 71.0 / 1920.0, E5 = -17253.0 / 339200.0, E6 = 22.0 / 525.0,
    E7 = -1.0 / 40.0;
  static constexpr double D1 = -12715105075.0 / 11282082432.0,
    D3 = 87487479700.0 / 32700410799.0, D4 = -10690763975.0 / 1880347072.0,
    D5 = 701980252875.0 / 199316789632.0, D6 = -1453857185.0 / 822651844.0,
    D7 = 69997945.0 / 29380423.0;

  explicit dopri5_counted(const dust2gpu::systems::sirode::shared_state& s)
    : sh(s) {}

  counted try_step(counted t, counted h, const counted* y) {
    const counted t_next = t + h;
    const counted* k1 = dydt;
    for (int i = 0; i < n; ++i) y_next[i] = y[i] + h * A21 * k1[i];
    sirode_rhs(sh, y_next, k2);
    for (int i = 0; i < n; ++i)
      y_next[i] = y[i] + h * (A31 * k1[i] + A32 * k2[i]);
    sirode_rhs(sh, y_next, k3);
    for (int i = 0; i < n; ++i)
      y_next[i] = y[i] + h * (A41 * k1[i] + A42 * k2[i] + A43 * k3[i]);
    sirode_rhs(sh, y_next, k4);
    for (int i = 0; i < n; ++i)
      y_next[i] = y[i] + h * (A51 * k1[i] + A52 * k2[i] + A53 * k3[i] +
                              A54 * k4[i]);
    sirode_rhs(sh, y_next, k5);
    for (int i = 0; i < n; ++i)
      y_stiff[i] = y[i] + h * (A61 * k1[i] + A62 * k2[i] + A63 * k3[i] +
                               A64 * k4[i] + A65 * k5[i]);
    sirode_rhs(sh, y_stiff, k6);
    for (int i = 0; i < n; ++i)
      y_next[i] = y[i] + h * (A71 * k1[i] + A73 * k3[i] + A74 * k4[i] +
                              A75 * k5[i] + A76 * k6[i]);
    sirode_rhs(sh, y_next, k2);
    (void)t_next;
    for (int i = 0; i < n; ++i)
      c5[i] = h * (D1 * k1[i] + D3 * k3[i] + D4 * k4[i] + D5 * k5[i] +
                   D6 * k6[i] + D7 * k2[i]);
    for (int i = 0; i < n; ++i)
      k4[i] = h * (E1 * k1[i] + E3 * k3[i] + E4 * k4[i] + E5 * k5[i] +
                   E6 * k6[i] + E7 * k2[i]);
    counted err = 0.0;
    for (int i = 0; i < n; ++i) {
      const counted sk = k4[i] / (atol + rtol * max(abs(y[i]),
                                                    abs(y_next[i])));
      err = err + sk * sk;
    }
    return sqrt(err / counted(n));
  }

  counted step(counted t, counted t_end, counted* y) {
    bool success = false, reject = false, truncated = false;
    counted h = step_size;
    while (!success) {
      if (h.v < step_size_min || n_steps > 10000) {
        return std::numeric_limits<double>::quiet_NaN();
      }
      truncated = t + h > t_end;
      if (truncated) {
        h = t_end - t;
      }
      const counted err = try_step(t, h, y);
      n_steps++;
      const counted fac11 = pow(err, constant);
      if (err <= 1.0) {
        success = true;
        t0 = t;
        h_last = h;
        for (int i = 0; i < n; ++i) {
          const counted ydiff = y_next[i] - y[i];
          const counted bspl = h * dydt[i] - ydiff;
          c1[i] = y[i];
          c2[i] = ydiff;
          c3[i] = bspl;
          c4[i] = -h * k2[i] + ydiff - bspl;
        }
        std::copy(k2, k2 + n, dydt);
        std::copy(y_next, y_next + n, y);
        n_accepted++;
        if (!truncated) {
          const counted fac_old = max(error, 1e-4);
          counted fac = fac11 / pow(fac_old, beta);
          fac = max(min(fac / factor_safe, facc1), facc2);
          const counted h_max =
            reject ? h : counted(std::numeric_limits<double>::infinity());
          step_size = min(h / fac, h_max);
          error = err;
        }
      } else {
        reject = true;
        h = h / min(facc1, fac11 / factor_safe);
      }
    }
    return truncated ? t_end : t + h;
  }

  // zero_every of cases_inc (entry 4) every whole time: the reset by
  // dense-output interpolation (solver.hpp:437-492)
  void reset_inc(counted t_reset, counted* y) {
    const counted u = (t_reset - t0) / h_last;
    const counted v = 1.0 - u;
    const counted val = c1[4] + u * (c2[4] + v * (c3[4] + u * (c4[4] +
                                                              v * c5[4])));
    c4[0] = val;
    y[4] = y[4] - val;
  }

  void apply_zero_every(counted t, counted* y) {
    if (h_last.v == 0) {
      return;
    }
    const counted period = 1.0;
    const counted nn = floor(t / period);
    const counted mm = floor(t0 / period);
    if (nn > mm) {
      const counted t_reset = nn * period;
      if (t_reset == t) {
        y[4] = 0.0;
      } else {
        reset_inc(t_reset, y);
      }
    }
  }

  void apply_zero_every_final(counted t, counted* y) {
    if (h_last.v == 0 || !(h_last.v > 1.0)) {
      return;
    }
    const int nn = static_cast<int>(std::ceil(t.v));
    const int mm = static_cast<int>(std::ceil(t0.v));
    if (nn > mm) {
      reset_inc(static_cast<double>(nn - 1), y);
    }
  }

  void initialise(counted t, const counted* y) {
    counted* f0 = dydt;
    counted* f1 = k3;
    counted* y1 = y_next;
    sirode_rhs(sh, y, f0);
    counted norm_f = 0.0, norm_y = 0.0;
    for (int i = 0; i < n; ++i) {
      const counted sk = atol + rtol * abs(y[i]);
      norm_f = norm_f + (f0[i] / sk) * (f0[i] / sk);
      norm_y = norm_y + (y[i] / sk) * (y[i] / sk);
    }
    counted h = (norm_f <= 1e-10 || norm_y <= 1e-10) ?
      counted(1e-6) : sqrt(norm_y / norm_f) * 0.01;
    for (int i = 0; i < n; ++i) {
      y1[i] = y[i] + h * f0[i];
    }
    sirode_rhs(sh, y1, f1);
    counted der2 = 0.0;
    for (int i = 0; i < n; ++i) {
      const counted sk = atol + rtol * abs(y[i]);
      der2 = der2 + ((f1[i] - f0[i]) / sk) * ((f1[i] - f0[i]) / sk);
    }
    der2 = sqrt(der2) / h;
    const counted der12 = max(abs(der2), sqrt(norm_f));
    const counted h1 = (der12 <= 1e-15) ?
      max(1e-6, abs(h) * 1e-3) : pow(0.01 / der12, 1.0 / 5.0);
    h = min(100.0 * abs(h), h1);
    h = max(h, step_size_min * 100);
    step_size = h;
    error = 0.0;
  }

  void run(counted t, counted t_end, counted* y) {
    while (t < t_end) {
      apply_zero_every(t, y);
      t = step(t, t_end, y);
      if (std::isnan(t.v)) {
        return;
      }
    }
    apply_zero_every_final(t, y);
  }
};

}  // namespace

extern "C" {

int opcount_n_ops() {
  return NOPS;
}

// Filter runs of groups 0..n_groups-1 of a workload.  pars: the packed
// parameter rows (n_pars doubles per group); n_particles per group; data
// [time][group]; words: the raw generator words of every group's stream
// block [2 filter streams | n_g particle streams], 4 words each.
// Outputs: ll per group; step_ops and compare_ops: NOPS counters each,
// summed over the run.  Returns 0, or -1 for an unknown system.
int opcount_filter(const char* name, const double* pars, int n_pars,
                   int n_groups, const int* n_particles, double dt,
                   const double* times, int n_times, const double* data,
                   const std::uint64_t* words, double* ll,
                   std::uint64_t* step_ops, std::uint64_t* compare_ops) {
  const std::string sys_name(name);
  std::fill(step_ops, step_ops + NOPS, 0);
  std::fill(compare_ops, compare_ops + NOPS, 0);
  size_t pos = 0;
  for (int g = 0; g < n_groups; ++g) {
    const double* row = pars + static_cast<size_t>(g) * n_pars;
    const int n = n_particles[g];
    if (sys_name == "sir_cases") {
      using S = dust2gpu::systems::sir_cases;
      ll[g] = filter_group<sir_counted, S>(
        S::build_shared(row), n, dt, times, n_times, data + g, n_groups,
        words + pos, step_ops, compare_ops);
    } else if (sys_name == "seir_age") {
      using S = dust2gpu::systems::seir_age;
      ll[g] = filter_group<seir_counted, S>(
        S::build_shared(row), n, dt, times, n_times, data + g, n_groups,
        words + pos, step_ops, compare_ops);
    } else {
      return -1;
    }
    pos += 4 * static_cast<size_t>(2 + n);
  }
  return 0;
}

// sirode instances (packed rows of n_pars doubles), each integrated from 0
// through `times`; out [time][instance][5]; steps: attempted steps per
// instance; ops: NOPS counters summed over the integration (initialisation
// included).
int opcount_dopri5_sirode(const double* pars, int n_pars, int n,
                          const double* times, int n_times, double* out,
                          std::int64_t* steps, std::uint64_t* ops) {
  std::fill(g_ops, g_ops + NOPS, 0);
  using S = dust2gpu::systems::sirode;
  for (int k = 0; k < n; ++k) {
    const auto sh = S::build_shared(pars + static_cast<size_t>(k) * n_pars);
    typename S::internal_state in{};
    rnd::rng_state r{};
    double y0[5];
    S::initial(0.0, sh, in, r, y0);
    counted y[5];
    for (int i = 0; i < 5; ++i) y[i] = y0[i];
    dopri5_counted sol(sh);
    sol.initialise(0.0, y);
    counted t = 0.0;
    for (int i = 0; i < n_times; ++i) {
      sol.run(t, times[i], y);
      t = times[i];
      for (int q = 0; q < 5; ++q) {
        out[(static_cast<size_t>(i) * n + k) * 5 + q] = y[q].v;
      }
    }
    steps[k] = sol.n_steps;
  }
  std::copy(g_ops, g_ops + NOPS, ops);
  return 0;
}

}  // extern "C"
