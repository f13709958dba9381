// The device table of log(k!), k = 0 .. math::LF_TABLE_MAX, behind
// math::lgamma.  It lives in one statically allocated device array (8 MiB,
// part of this module) and is filled by a kernel that evaluates
// math::lgamma_nontable, the function the host oracle calls, so that a
// table read and a computation agree to the bit.
#include <cuda_runtime.h>

#include <mutex>

#include "dust2gpu/math.hpp"
#include "engine/device.cuh"
#include "engine/lf_table.hpp"

namespace dust2gpu {
namespace engine {

static __device__ double lf_table_storage[math::LF_TABLE_MAX + 1];

static __global__ void k_fill_lf_table(double* t, int n) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k < n) {
    t[k] = math::lgamma_nontable(static_cast<double>(k) + 1.0);
  }
}

const double* lf_table_device() {
  constexpr int MAX_DEVICES = 64;
  static std::mutex mutex;
  static const double* table[MAX_DEVICES] = {};
  int dev = 0;
  DUST2_CUDA(cudaGetDevice(&dev));
  if (dev < 0 || dev >= MAX_DEVICES) {
    throw std::runtime_error("device ordinal out of range");
  }
  std::lock_guard<std::mutex> lock(mutex);
  if (table[dev] == nullptr) {
    void* p = nullptr;
    DUST2_CUDA(cudaGetSymbolAddress(&p, lf_table_storage));
    const int n = math::LF_TABLE_MAX + 1;
    cudaStream_t stream;
    DUST2_CUDA(cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking));
    k_fill_lf_table<<<(n + 255) / 256, 256, 0, stream>>>(
      static_cast<double*>(p), n);
    const cudaError_t launch = cudaGetLastError();
    const cudaError_t done = cudaStreamSynchronize(stream);
    cudaStreamDestroy(stream);
    DUST2_CUDA(launch);
    DUST2_CUDA(done);
    table[dev] = static_cast<const double*>(p);
  }
  return table[dev];
}

}  // namespace engine
}  // namespace dust2gpu
