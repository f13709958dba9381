// Systematic resampling without any device allocation.
//
// dust2_gb300_resample_weight allocates its working arrays with cudaMalloc
// on every call.  Some callers cannot allow that: an application whose
// GPU memory is owned by another allocator (a framework's caching pool or
// a host runtime that enforces its own device-memory budget) may have no
// free device memory outside that pool, and a latency-critical loop cannot
// afford the device-wide synchronisation that cudaFree implies.  This
// variant runs the same kernels on scratch space that lives in a
// file-scope __device__ array, reserved once when the library is loaded
// onto a device and kept until the process exits.
//
// Limits and sharing:
//   * the array takes 2 MiB on every device that loads this library; a
//     call uses at most about 1.9 MB of it (NOALLOC_MAX_N = 65536
//     weights per call);
//   * every call uses the same array, which keeps the previous call's
//     contents; everything that must start at zero is cleared per call;
//   * calls that overlap on the GPU race on that array (for example, two
//     host threads calling at once): serialise them;
//   * the work runs on the calling thread's per-thread default stream
//     (cudaStreamPerThread), which needs nothing created and does not
//     wait for the caller's other streams;
//   * the first call on a device looks up the array's device address
//     (cudaGetSymbolAddress) with that device current, and later calls
//     reuse it; make that first call before any stream capture on the
//     device, and do not call the entry point on a device after
//     cudaDeviceReset in the same process (the library's module may then
//     be loaded at another address).
#include <cuda_runtime.h>

#include <algorithm>
#include <mutex>
#include <stdexcept>
#include <string>

#include "../../include/dust2_gb300.h"
#include "engine/api.hpp"
#include "engine/device.cuh"
#include "engine/filter.cuh"
#include "engine/layout.hpp"
#include "resample_hooks.cuh"

namespace {

constexpr std::size_t NOALLOC_MAX_N = 65536;
constexpr int NOALLOC_TILE = 256;
constexpr int NOALLOC_MAX_TILES =
  static_cast<int>(NOALLOC_MAX_N / NOALLOC_TILE);
constexpr std::size_t NOALLOC_SCRATCH_BYTES = 2u * 1024u * 1024u;

// The scratch space.  In host code this name is only a stand-in for the
// device object: its device address comes from cudaGetSymbolAddress.
static __device__ __align__(256) char noalloc_scratch[NOALLOC_SCRATCH_BYTES];

constexpr int MAX_DEVICES = 64;
std::mutex setup_mutex;
char* scratch_address[MAX_DEVICES] = {};

// Device address of the scratch array on the current device (looked up
// once per device, with that device current).
char* scratch_on_current_device() {
  int dev = 0;
  DUST2_CUDA(cudaGetDevice(&dev));
  if (dev < 0 || dev >= MAX_DEVICES) {
    throw std::runtime_error("device index out of range");
  }
  std::lock_guard<std::mutex> lock(setup_mutex);
  if (scratch_address[dev] == nullptr) {
    void* ptr = nullptr;
    const cudaError_t err = cudaGetSymbolAddress(&ptr, noalloc_scratch);
    if (err != cudaSuccess || ptr == nullptr) {
      throw std::runtime_error(
        std::string("cudaGetSymbolAddress failed for the resampling "
                    "scratch array: ") + cudaGetErrorString(err));
    }
    scratch_address[dev] = static_cast<char*>(ptr);
  }
  return scratch_address[dev];
}

// idx (int, group-local) -> size_t for the caller's output array.
__global__ void k_widen_index(const int* idx, int n, unsigned long long* out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) {
    out[i] = static_cast<unsigned long long>(idx[i]);
  }
}

}  // namespace

extern "C" int dust2_gb300_resample_weight_noalloc(const double* w, size_t n,
                                                   double u, size_t* idx) {
  using namespace dust2gpu::engine;
  try {
    if (n < 1) {
      throw std::runtime_error("'n' must be at least 1");
    }
    if (n > NOALLOC_MAX_N) {
      throw std::runtime_error(
        "'n' is " + std::to_string(n) + ", above the limit of " +
        std::to_string(NOALLOC_MAX_N) + " weights for "
        "dust2_gb300_resample_weight_noalloc; use "
        "dust2_gb300_resample_weight for larger inputs");
    }
    static_assert(sizeof(size_t) == sizeof(unsigned long long),
                  "size_t must be 64-bit");
    // tiles of one group, without heap allocation
    tile tiles[NOALLOC_MAX_TILES];
    const int nt = static_cast<int>((n + NOALLOC_TILE - 1) / NOALLOC_TILE);
    for (int t = 0; t < nt; ++t) {
      const int local = t * NOALLOC_TILE;
      tiles[t] = tile{0, local,
                      std::min(NOALLOC_TILE, static_cast<int>(n) - local),
                      local};
    }
    const std::size_t need = hook_scratch_bytes(n, NOALLOC_TILE) +
      sizeof(int) + 256;
    if (need > NOALLOC_SCRATCH_BYTES) {
      throw std::runtime_error("resampling scratch array too small");
    }
    char* base = scratch_on_current_device();
    // the calling thread's default stream: nothing is created, and it
    // does not wait for the caller's other (blocking) streams
    const cudaStream_t s = cudaStreamPerThread;
    int* fallback_count = reinterpret_cast<int*>(base);
    hook_buffers hb;
    hook_layout(base + 256, n, tiles, nt, hb, s);
    DUST2_CUDA(cudaMemsetAsync(fallback_count, 0, sizeof(int), s));
    DUST2_CUDA(cudaMemcpyAsync(hb.f.w, w, n * sizeof(double),
                               cudaMemcpyHostToDevice, s));
    hook_resample(hb, u, NOALLOC_TILE, 0, fallback_count, s);
    // the prefix-sum array is free once the indices exist
    auto* wide = reinterpret_cast<unsigned long long*>(hb.f.pre);
    k_widen_index<<<(static_cast<int>(n) + 255) / 256, 256, 0, s>>>(
      hb.f.idx, static_cast<int>(n), wide);
    DUST2_CUDA(cudaGetLastError());
    DUST2_CUDA(cudaMemcpyAsync(idx, wide, n * sizeof(size_t),
                               cudaMemcpyDeviceToHost, s));
    DUST2_CUDA(cudaStreamSynchronize(s));
    return DUST2_GB300_OK;
  } catch (const std::exception& e) {
    set_last_error(e.what());
    return DUST2_GB300_ERROR;
  }
}
