// Kernels shared by the discrete-time and continuous-time engines: block
// loads of per-group data into shared memory, generator load/store, error
// capture, and the state gather/scatter used by the state export, import
// and reorder verbs.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <type_traits>

#include "../dust2gpu/common.hpp"
#include "../dust2gpu/random.hpp"
#include "../dust2gpu/system.hpp"
#include "device.cuh"
#include "layout.hpp"

namespace dust2gpu {
namespace engine {

// Copy a trivially copyable object from global to shared memory with the
// whole block.
template <typename S>
__device__ __forceinline__ void block_load(S* dst, const S* src) {
  constexpr int n_bytes = static_cast<int>(sizeof(S));
  if constexpr (n_bytes % 8 == 0 && alignof(S) >= 8) {
    const auto* s = reinterpret_cast<const unsigned long long*>(src);
    auto* d = reinterpret_cast<unsigned long long*>(dst);
    for (int i = threadIdx.x; i < n_bytes / 8; i += blockDim.x) {
      d[i] = s[i];
    }
  } else {
    const auto* s = reinterpret_cast<const unsigned char*>(src);
    auto* d = reinterpret_cast<unsigned char*>(dst);
    for (int i = threadIdx.x; i < n_bytes; i += blockDim.x) {
      d[i] = s[i];
    }
  }
}

__device__ __forceinline__ random::rng_state load_rng(
    const std::uint64_t* rng, int stride, int k, bool deterministic) {
  random::rng_state r;
  r.state[0] = rng[k];
  r.state[1] = rng[stride + k];
  r.state[2] = rng[2 * stride + k];
  r.state[3] = rng[3 * stride + k];
  r.deterministic = deterministic;
  r.err = 0;
  r.err_v0 = 0;
  r.err_v1 = 0;
  return r;
}

__device__ __forceinline__ void store_rng(std::uint64_t* rng, int stride,
                                          int k,
                                          const random::rng_state& r) {
  rng[k] = r.state[0];
  rng[stride + k] = r.state[1];
  rng[2 * stride + k] = r.state[2];
  rng[3 * stride + k] = r.state[3];
}

__device__ __forceinline__ void capture_error(particle_error* errors,
                                              int* any_error, int k,
                                              const random::rng_state& r) {
  if (r.err != 0) {
    if (errors[k].code == 0) {
      errors[k].code = r.err;
      errors[k].v0 = r.err_v0;
      errors[k].v1 = r.err_v1;
    }
    atomicOr(any_error, 1);
  }
}

// out[k * n_out + i] = state[index[i] * stride + k]  (index may be null:
// identity over n_out entries).  Writes dust2's particle-major order.
static __global__ void k_gather_state(const double* __restrict__ state, int stride,
                               int n_total, const int* __restrict__ index,
                               int n_out, double* __restrict__ out) {
  const long i = static_cast<long>(blockIdx.x) * blockDim.x + threadIdx.x;
  const long n = static_cast<long>(n_total) * n_out;
  if (i >= n) {
    return;
  }
  const int k = static_cast<int>(i / n_out);
  const int j = static_cast<int>(i % n_out);
  const int s = index == nullptr ? j : index[j];
  out[i] = state[static_cast<long>(s) * stride + k];
}

// Inverse of k_gather_state for the full state.
static __global__ void k_scatter_state(const double* __restrict__ in, int stride,
                                int n_total, int n_state,
                                double* __restrict__ state) {
  const long i = static_cast<long>(blockIdx.x) * blockDim.x + threadIdx.x;
  const long n = static_cast<long>(n_total) * n_state;
  if (i >= n) {
    return;
  }
  const int k = static_cast<int>(i / n_state);
  const int s = static_cast<int>(i % n_state);
  state[static_cast<long>(s) * stride + k] = in[i];
}

// dst[s][k] = src[s][offset(group(k)) + index[k]] for every particle of
// tile blockIdx.x; index is group-local.  Particles of groups whose mode
// is not "resampled" (mode == nullptr means all are) are copied as is.
static __global__ void k_reorder(const double* __restrict__ src,
                          double* __restrict__ dst, int stride, int n_state,
                          const tile* __restrict__ tiles,
                          const int* __restrict__ group_offset,
                          const int* __restrict__ index,
                          const int* __restrict__ group_mode) {
  const tile tl = tiles[blockIdx.x];
  if (static_cast<int>(threadIdx.x) >= tl.count) {
    return;
  }
  const int k = tl.start + threadIdx.x;
  const bool move = group_mode == nullptr || group_mode[tl.group] != 0;
  const int from = move ? group_offset[tl.group] + index[k] : k;
  for (int s = 0; s < n_state; ++s) {
    dst[static_cast<long>(s) * stride + k] =
      src[static_cast<long>(s) * stride + from];
  }
}

// k_reorder for one row of integers (solver step counters).
static __global__ void k_reorder_int(const int* __restrict__ src,
                                     int* __restrict__ dst, int stride,
                                     const tile* __restrict__ tiles,
                                     const int* __restrict__ group_offset,
                                     const int* __restrict__ index,
                                     const int* __restrict__ group_mode) {
  const tile tl = tiles[blockIdx.x];
  if (static_cast<int>(threadIdx.x) >= tl.count) {
    return;
  }
  const int k = tl.start + threadIdx.x;
  const bool move = group_mode == nullptr || group_mode[tl.group] != 0;
  dst[k] = src[move ? group_offset[tl.group] + index[k] : k];
  (void)stride;
}

inline int n_blocks(long n, int block) {
  return static_cast<int>((n + block - 1) / block);
}

}  // namespace engine
}  // namespace dust2gpu
