// The filter's log-weight scaling and systematic resampling on a single
// group of weights, as standalone entry points.  dust2 exposes the same
// two helpers to its R tests (src/test.cpp:10-23, test_resample_weight and
// test_scale_log_weights, pinned by tests/testthat/test-filter-details.R);
// here they run the GPU kernels of the particle filter (k_weights,
// k_resample, k_fallback_count) on device buffers allocated per call.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <stdexcept>
#include <string>
#include <vector>

#include "../../include/dust2_gb300.h"
#include "dust2gpu/math.hpp"
#include "engine/device.cuh"
#include "engine/filter.cuh"
#include "engine/layout.hpp"
#include "resample_hooks.cuh"

namespace dust2gpu {
namespace engine {

// Chunk scans of raw (already exponentiated) weights: ew = w.
__global__ void k_weights_raw(filter_view f) {
  const tile tl = f.tiles[blockIdx.x];
  const int warp = threadIdx.x >> 5;
  if (32 * warp >= tl.count) {
    return;
  }
  const bool valid = static_cast<int>(threadIdx.x) < tl.count;
  const int k = tl.start + threadIdx.x;
  const double e = valid ? f.w[k] : 0.0;
  const double incl = warp_inclusive_scan(e);
  if (valid) {
    f.ew[k] = e;
    f.pre[k] = incl;
  }
  if ((threadIdx.x & 31) == 31) {
    f.chunk_sum[f.chunk_first[tl.group] + tl.local / 32 + warp] = incl;
  }
}

// Per-tile "any weight non-zero" and maximum log weight (NaN as -Inf),
// as the step kernel does after compare.
__global__ void k_reduce_log_weights(filter_view f) {
  __shared__ double red[33];
  const tile tl = f.tiles[blockIdx.x];
  const bool valid = static_cast<int>(threadIdx.x) < tl.count;
  const double w = valid ? f.w[tl.start + threadIdx.x] : 0.0;
  const int nz = __syncthreads_or(valid && w != 0);
  const double mx = block_max(valid && !(w != w) ? w : -INFINITY, red);
  if (threadIdx.x == 0) {
    if (nz) {
      atomicOr(f.gnz + tl.group, 1);
    }
    atomicMax(f.gkey + tl.group, ordered_key(mx));
  }
}

// One group: tile offsets and total; the log-likelihood increment when
// `lse` is set; the systematic targets for a given uniform u.
__global__ void k_group_given_u(filter_view f, double u, int lse,
                                int force_serial) {
  const int g = 0;
  const int lane = threadIdx.x;
  const int n = f.n_particles[g];
  const double tot = group_chunk_offsets(f, g, lane);
  if (lane == 0) {
    if (lse) {
      f.ll[g] = math::log(tot / n) + ordered_value(f.gkey[g]);
    }
    f.gu[g] = u;
    f.gtot[g] = tot;
    f.guu0[g] = tot * u / n;
    f.gdu[g] = tot / n;
    f.mode[g] = MODE_RESAMPLE;
    f.gflag[g] = force_serial;
  }
}

std::size_t hook_scratch_bytes(std::size_t n, int tile_size) {
  const std::size_t nt = (n + tile_size - 1) / tile_size;
  const std::size_t nc = (n + 31) / 32;
  // w, ew, pre (n doubles each), chunk_sum, chunk_off (nc doubles each),
  // idx (n ints), tiles (nt), 7 doubles + 1 key + 8 ints of group data
  return 256 * 16 + 3 * n * 8 + 2 * nc * 8 + n * 4 + nt * sizeof(tile) +
    7 * 8 + 8 + 8 * 4;
}

// Lay the hook's arrays out in one device region (256-byte aligned
// pieces) and fill the per-group scalars and tiles.  `base` must hold
// hook_scratch_bytes(n) bytes.  Every per-group scalar is rewritten, so
// nothing an earlier call left in the same memory is read.
void hook_layout(char* base, std::size_t n, const tile* tiles, int n_tiles,
                 hook_buffers& hb, cudaStream_t s) {
  std::size_t off = 0;
  auto take = [&](std::size_t bytes) {
    char* p = base + off;
    off += (bytes + 255) / 256 * 256;
    return p;
  };
  const std::size_t nt = static_cast<std::size_t>(n_tiles);
  filter_view& f = hb.f;
  f.w = reinterpret_cast<double*>(take(n * 8));
  f.ew = reinterpret_cast<double*>(take(n * 8));
  f.pre = reinterpret_cast<double*>(take(n * 8));
  const std::size_t nc = (n + 31) / 32;
  f.chunk_sum = reinterpret_cast<double*>(take(nc * 8));
  f.chunk_off = reinterpret_cast<double*>(take(nc * 8));
  f.idx = reinterpret_cast<int*>(take(n * 4));
  tile* t_dev = reinterpret_cast<tile*>(take(nt * sizeof(tile)));
  double* dbl = reinterpret_cast<double*>(take(7 * 8));
  f.ll = dbl;
  f.gu = dbl + 1;
  f.guu0 = dbl + 2;
  f.gdu = dbl + 3;
  f.gtot = dbl + 4;
  f.gkey = reinterpret_cast<unsigned long long*>(take(8));
  int* ints = reinterpret_cast<int*>(take(8 * 4));
  f.active = ints;
  f.n_particles = ints + 1;
  f.offset = ints + 2;
  f.chunk_first = ints + 3;
  f.chunk_count = ints + 4;
  f.gnz = ints + 5;
  f.gflag = ints + 6;
  f.mode = ints + 7;
  f.tiles = t_dev;
  f.frng = nullptr;
  f.set_initial = nullptr;
  f.force_serial = nullptr;
  const int h_ints[8] = {1, static_cast<int>(n), 0, 0,
                         static_cast<int>(nc), 0, 0, MODE_RESAMPLE};
  DUST2_CUDA(cudaMemcpyAsync(ints, h_ints, sizeof(h_ints),
                             cudaMemcpyHostToDevice, s));
  const unsigned long long key0 = 0;  // below every ordered key
  DUST2_CUDA(cudaMemcpyAsync(f.gkey, &key0, 8, cudaMemcpyHostToDevice, s));
  DUST2_CUDA(cudaMemcpyAsync(t_dev, tiles, nt * sizeof(tile),
                             cudaMemcpyHostToDevice, s));
  hb.n_tiles = n_tiles;
}

// Systematic resampling of raw weights already in hb.f.w; indices left
// in hb.f.idx (device).
void hook_resample(hook_buffers& hb, double u, int tile_size, int serial,
                   int* fallback_count, cudaStream_t s) {
  k_weights_raw<<<hb.n_tiles, tile_size, 0, s>>>(hb.f);
  k_group_given_u<<<1, 32, 0, s>>>(hb.f, u, 0, serial);
  k_resample<<<hb.n_tiles, tile_size, 0, s>>>(hb.f);
  k_fallback_count<<<1, FALLBACK_THREADS, 0, s>>>(hb.f, fallback_count);
  DUST2_CUDA(cudaGetLastError());
}

}  // namespace engine
}  // namespace dust2gpu

namespace {

using namespace dust2gpu::engine;
using dust2gpu::device_array;

constexpr int HOOK_TILE = 256;

std::vector<tile> one_group_tiles(std::size_t n) {
  group_layout L(std::vector<int>{static_cast<int>(n)}, HOOK_TILE);
  return L.tiles;
}

}  // namespace

extern "C" {

int dust2_gb300_resample_weight(const double* w, size_t n, double u,
                                size_t* idx) {
  try {
    if (n < 1 || n > (1u << 30)) {
      throw std::runtime_error("'n' must be in [1, 2^30]");
    }
    const auto tiles = one_group_tiles(n);
    device_array<char> scratch(hook_scratch_bytes(n, HOOK_TILE));
    device_array<int> count(1);
    cudaStream_t s;
    DUST2_CUDA(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
    hook_buffers hb;
    hook_layout(scratch.data(), n, tiles.data(),
                static_cast<int>(tiles.size()), hb, s);
    DUST2_CUDA(cudaMemsetAsync(count.data(), 0, sizeof(int), s));
    DUST2_CUDA(cudaMemcpyAsync(hb.f.w, w, n * 8, cudaMemcpyHostToDevice, s));
    hook_resample(hb, u, HOOK_TILE, 0, count.data(), s);
    std::vector<int> out(n);
    DUST2_CUDA(cudaMemcpyAsync(out.data(), hb.f.idx, n * 4,
                               cudaMemcpyDeviceToHost, s));
    DUST2_CUDA(cudaStreamSynchronize(s));
    cudaStreamDestroy(s);
    for (size_t i = 0; i < n; ++i) {
      idx[i] = static_cast<size_t>(out[i]);
    }
    return DUST2_GB300_OK;
  } catch (const std::exception& e) {
    dust2gpu::engine::set_last_error(e.what());
    return DUST2_GB300_ERROR;
  }
}

int dust2_gb300_scale_log_weights(double* w, size_t n, double* result) {
  try {
    if (n < 1 || n > (1u << 30)) {
      throw std::runtime_error("'n' must be in [1, 2^30]");
    }
    // filter_details.hpp:13-15: a single weight is returned as is
    if (n == 1) {
      *result = w[0];
      return DUST2_GB300_OK;
    }
    const auto tiles = one_group_tiles(n);
    device_array<char> scratch(hook_scratch_bytes(n, HOOK_TILE));
    cudaStream_t s;
    DUST2_CUDA(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
    hook_buffers hb;
    hook_layout(scratch.data(), n, tiles.data(),
                static_cast<int>(tiles.size()), hb, s);
    DUST2_CUDA(cudaMemcpyAsync(hb.f.w, w, n * 8, cudaMemcpyHostToDevice, s));
    k_reduce_log_weights<<<hb.n_tiles, HOOK_TILE, 0, s>>>(hb.f);
    unsigned long long key = 0;
    DUST2_CUDA(cudaMemcpyAsync(&key, hb.f.gkey, 8, cudaMemcpyDeviceToHost, s));
    DUST2_CUDA(cudaStreamSynchronize(s));
    // decode the ordered key on the host
    const unsigned long long bits =
      (key >> 63) ? (key & 0x7fffffffffffffffull) : ~key;
    const double mx = dust2gpu::math::from_bits(bits);
    if (mx == -INFINITY) {
      // all -Inf (or NaN): weights stay log weights with NaN -> -Inf
      for (size_t i = 0; i < n; ++i) {
        if (std::isnan(w[i])) {
          w[i] = -INFINITY;
        }
      }
      *result = -INFINITY;
      cudaStreamDestroy(s);
      return DUST2_GB300_OK;
    }
    DUST2_CUDA(cudaMemsetAsync(hb.f.gnz, 0xff, sizeof(int), s));
    k_weights<<<hb.n_tiles, HOOK_TILE, 0, s>>>(hb.f);
    k_group_given_u<<<1, 32, 0, s>>>(hb.f, 0.0, 1, 0);
    DUST2_CUDA(cudaGetLastError());
    DUST2_CUDA(cudaMemcpyAsync(w, hb.f.ew, n * 8, cudaMemcpyDeviceToHost, s));
    DUST2_CUDA(cudaMemcpyAsync(result, hb.f.ll, 8, cudaMemcpyDeviceToHost, s));
    DUST2_CUDA(cudaStreamSynchronize(s));
    cudaStreamDestroy(s);
    return DUST2_GB300_OK;
  } catch (const std::exception& e) {
    dust2gpu::engine::set_last_error(e.what());
    return DUST2_GB300_ERROR;
  }
}

}  // extern "C"
