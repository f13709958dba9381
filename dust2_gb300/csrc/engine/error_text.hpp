// Text of a per-particle error, shared by the engine's error summary and
// the oracle builds so that messages match word for word.
#pragma once

#include <cstdio>
#include <string>

#include "../dust2gpu/common.hpp"

namespace dust2gpu {

inline std::string error_text(const particle_error& e) {
  char buf[256];
  switch (e.code) {
  case ERR_BINOMIAL_INVALID:
    std::snprintf(buf, sizeof(buf),
                  "Invalid call to binomial with n = %.17g, p = %.17g",
                  e.v0, e.v1);
    return buf;
  case ERR_POISSON_INVALID:
    std::snprintf(buf, sizeof(buf),
                  "Invalid call to Poisson with lambda = %.17g", e.v0);
    return buf;
  case ERR_ODE_TOO_MANY_STEPS:
    return "too many steps";
  case ERR_ODE_STEP_TOO_SMALL:
    return "step too small";
  case ERR_ODE_STEP_VANISHED:
    return "step size vanished";
  case ERR_ODE_INITIAL_STEP:
    return "Initial step size was not finite";
  case ERR_NEGBIN_INVALID:
    return "Invalid call to negative binomial";
  default:
    std::snprintf(buf, sizeof(buf), "unknown error code %d", e.code);
    return buf;
  }
}

}  // namespace dust2gpu
