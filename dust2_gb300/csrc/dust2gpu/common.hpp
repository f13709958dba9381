// Portability macros shared by host (g++) and device (nvcc) builds.
//
// Every arithmetic routine in dust2gpu/ is written once and compiled for
// both sides.  Bit-identical results between the CPU oracle and the GPU
// kernels rely on three rules, enforced by the build flags:
//   * g++ uses -ffp-contract=off and nvcc uses -fmad=false, so a*b+c is
//     never silently fused;
//   * fused multiply-adds are written explicitly as fma(), which is
//     correctly rounded on both sides;
//   * only IEEE-754 correctly rounded operations are used (+ - * / sqrt,
//     fma, conversions, floor/rint/fmod); transcendental functions come
//     from dust2gpu/math.hpp, never from the platform libm.
#pragma once

#include <cstddef>
#include <cstdint>

#if defined(__CUDACC__)
#define DUST2_HD __host__ __device__ __forceinline__
#define DUST2_HOST_DEVICE __host__ __device__
#else
#define DUST2_HD inline
#define DUST2_HOST_DEVICE
#endif

namespace dust2gpu {

// Per-particle error codes written by device code (there are no
// exceptions on the GPU).  The host turns these into the same summary
// message the reference builds from its captured exceptions
// (inst/include/dust2/errors.hpp:29-54).
enum error_code : int {
  ERR_NONE = 0,
  ERR_BINOMIAL_INVALID = 1,     // n < 0, p < 0 or p > 1 (or non-finite)
  ERR_POISSON_INVALID = 2,      // lambda < 0 or non-finite
  ERR_ODE_TOO_MANY_STEPS = 3,   // continuous/solver.hpp:163-167
  ERR_ODE_STEP_TOO_SMALL = 4,   // continuous/solver.hpp:168-170
  ERR_ODE_STEP_VANISHED = 5,    // continuous/solver.hpp:171-173
  ERR_ODE_INITIAL_STEP = 6,     // continuous/solver.hpp:318-320
  ERR_NEGBIN_INVALID = 7
};

// A particle's error slot: first error wins, values keep the offending
// arguments so the host can format a message.
struct particle_error {
  int code;
  double v0;
  double v1;
};

}  // namespace dust2gpu
