// Device-side building blocks shared by the engine kernels: CUDA error
// checking, structure-of-arrays access, warp/block reductions and scans
// in FP64, and an order-preserving integer key for atomic max of doubles.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <stdexcept>
#include <string>

#include "../dust2gpu/common.hpp"

namespace dust2gpu {

inline void cuda_check(cudaError_t err, const char* what) {
  if (err != cudaSuccess) {
    throw std::runtime_error(std::string("CUDA error in ") + what + ": " +
                             cudaGetErrorString(err));
  }
}

#define DUST2_CUDA(expr) ::dust2gpu::cuda_check((expr), #expr)

// Owning device buffer (cudaMalloc / cudaFree).
template <typename T>
class device_array {
public:
  device_array() : ptr_(nullptr), size_(0) {}
  explicit device_array(std::size_t n) : ptr_(nullptr), size_(0) {
    resize(n);
  }
  ~device_array() {
    release();
  }
  device_array(const device_array&) = delete;
  device_array& operator=(const device_array&) = delete;
  device_array(device_array&& o) noexcept : ptr_(o.ptr_), size_(o.size_) {
    o.ptr_ = nullptr;
    o.size_ = 0;
  }
  device_array& operator=(device_array&& o) noexcept {
    if (this != &o) {
      release();
      ptr_ = o.ptr_;
      size_ = o.size_;
      o.ptr_ = nullptr;
      o.size_ = 0;
    }
    return *this;
  }
  void resize(std::size_t n) {
    release();
    if (n > 0) {
      DUST2_CUDA(cudaMalloc(reinterpret_cast<void**>(&ptr_), n * sizeof(T)));
    }
    size_ = n;
  }
  void release() {
    if (ptr_ != nullptr) {
      cudaFree(ptr_);
    }
    ptr_ = nullptr;
    size_ = 0;
  }
  T* data() {
    return ptr_;
  }
  const T* data() const {
    return ptr_;
  }
  std::size_t size() const {
    return size_;
  }

private:
  T* ptr_;
  std::size_t size_;
};

#if defined(__CUDACC__)

__device__ __forceinline__ unsigned long long ordered_key(double d) {
  const unsigned long long u = static_cast<unsigned long long>(
    __double_as_longlong(d));
  return (u >> 63) ? ~u : (u | 0x8000000000000000ull);
}

__device__ __forceinline__ double ordered_value(unsigned long long k) {
  const unsigned long long u =
    (k >> 63) ? (k & 0x7fffffffffffffffull) : ~k;
  return __longlong_as_double(static_cast<long long>(u));
}

__device__ __forceinline__ double warp_max(double v) {
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) {
    v = fmax(v, __shfl_xor_sync(0xffffffffu, v, off));
  }
  return v;
}

__device__ __forceinline__ int warp_or(int v) {
  return __any_sync(0xffffffffu, v != 0) ? 1 : 0;
}

// Inclusive scan within a warp (Kogge-Stone); the addition order is fixed
// by lane index, so results are reproducible run to run.
__device__ __forceinline__ double warp_inclusive_scan(double v) {
  const int lane = threadIdx.x & 31;
#pragma unroll
  for (int off = 1; off < 32; off <<= 1) {
    const double t = __shfl_up_sync(0xffffffffu, v, off);
    if (lane >= off) {
      v = v + t;
    }
  }
  return v;
}

// Inclusive scan over the whole block (blockDim.x a multiple of 32, at
// most 1024).  `smem` needs 32 doubles.  Returns the thread's inclusive
// prefix; the block total is written to *total.
__device__ __forceinline__ double block_inclusive_scan(double v, double* smem,
                                                       double* total) {
  const int lane = threadIdx.x & 31;
  const int warp = threadIdx.x >> 5;
  const int n_warps = blockDim.x >> 5;
  v = warp_inclusive_scan(v);
  if (lane == 31) {
    smem[warp] = v;
  }
  __syncthreads();
  if (warp == 0) {
    double w = lane < n_warps ? smem[lane] : 0.0;
    w = warp_inclusive_scan(w);
    smem[lane] = w;
  }
  __syncthreads();
  if (warp > 0) {
    v = v + smem[warp - 1];
  }
  *total = smem[n_warps - 1];
  __syncthreads();
  return v;
}

__device__ __forceinline__ double block_max(double v, double* smem) {
  const int lane = threadIdx.x & 31;
  const int warp = threadIdx.x >> 5;
  const int n_warps = blockDim.x >> 5;
  v = warp_max(v);
  if (lane == 0) {
    smem[warp] = v;
  }
  __syncthreads();
  if (warp == 0) {
    double w = lane < n_warps ? smem[lane] : -INFINITY;
    w = warp_max(w);
    if (lane == 0) {
      smem[32] = w;
    }
  }
  __syncthreads();
  const double r = smem[32];
  __syncthreads();
  return r;
}

#endif

}  // namespace dust2gpu
