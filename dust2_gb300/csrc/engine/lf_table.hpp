// The device table of log(k!) read by math::lgamma (dust2gpu/math.hpp).
#pragma once

#include <cuda_runtime.h>

#include <mutex>

#include "../dust2gpu/math.hpp"
#include "device.cuh"

namespace dust2gpu {
namespace engine {

// Address of the current device's table, filled on first use (once per
// device; later calls return at once).  Defined in lf_table.cu.
const double* lf_table_device();

// Point this translation unit's copy of math::lf_table_ptr at the
// current device's table.  Each translation unit that launches kernels
// using the samplers or densities calls this before its first launch on
// a device; until then its kernels compute lgamma instead, with the same
// results.
static inline void bind_lf_table() {
  constexpr int MAX_DEVICES = 64;
  static std::mutex mutex;
  static bool bound[MAX_DEVICES] = {};
  int dev = 0;
  DUST2_CUDA(cudaGetDevice(&dev));
  if (dev < 0 || dev >= MAX_DEVICES) {
    return;
  }
  std::lock_guard<std::mutex> lock(mutex);
  if (!bound[dev]) {
    const double* p = lf_table_device();
    DUST2_CUDA(cudaMemcpyToSymbol(math::lf_table_ptr, &p, sizeof(p)));
    bound[dev] = true;
  }
}

}  // namespace engine
}  // namespace dust2gpu
