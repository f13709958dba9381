// FP64 pipe peak: independent DFMA chains on every SM, timed with CUDA
// events.  The roofline of the FP64-bound kernels is reported against
// this measured rate.  The loop is bounded and every thread writes one
// element of an array sized for the grid.
#include <cuda_runtime.h>

#include <vector>

#include "../../include/dust2_gb300.h"
#include "engine/device.cuh"

namespace {

__global__ void k_dfma_chains(double* out, int iters, double a, double b) {
  double x0 = threadIdx.x * 1e-3, x1 = x0 + 1, x2 = x0 + 2, x3 = x0 + 3;
  double x4 = x0 + 4, x5 = x0 + 5, x6 = x0 + 6, x7 = x0 + 7;
  for (int i = 0; i < iters; ++i) {
    x0 = fma(x0, a, b);
    x1 = fma(x1, a, b);
    x2 = fma(x2, a, b);
    x3 = fma(x3, a, b);
    x4 = fma(x4, a, b);
    x5 = fma(x5, a, b);
    x6 = fma(x6, a, b);
    x7 = fma(x7, a, b);
  }
  out[blockIdx.x * blockDim.x + threadIdx.x] =
    x0 + x1 + x2 + x3 + x4 + x5 + x6 + x7;
}

}  // namespace

extern "C" int dust2_gb300_fp64_peak(double* tflops) {
  try {
    int dev = 0;
    DUST2_CUDA(cudaGetDevice(&dev));
    cudaDeviceProp p;
    DUST2_CUDA(cudaGetDeviceProperties(&p, dev));
    const int blocks = p.multiProcessorCount * 8;
    const int threads = 256;
    const int iters = 4096;
    dust2gpu::device_array<double> out(static_cast<std::size_t>(blocks) *
                                       threads);
    cudaEvent_t e0, e1;
    DUST2_CUDA(cudaEventCreate(&e0));
    DUST2_CUDA(cudaEventCreate(&e1));
    double best = 0;
    for (int rep = 0; rep < 4; ++rep) {
      DUST2_CUDA(cudaEventRecord(e0));
      k_dfma_chains<<<blocks, threads>>>(out.data(), iters, 0.999999, 1e-7);
      DUST2_CUDA(cudaEventRecord(e1));
      DUST2_CUDA(cudaEventSynchronize(e1));
      float ms = 0;
      DUST2_CUDA(cudaEventElapsedTime(&ms, e0, e1));
      const double flops = 2.0 * 8 * iters * static_cast<double>(blocks) *
        threads;
      if (rep > 0) {
        best = std::max(best, flops / (ms * 1e-3) / 1e12);
      }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    *tflops = best;
    return DUST2_GB300_OK;
  } catch (...) {
    return DUST2_GB300_ERROR;
  }
}
