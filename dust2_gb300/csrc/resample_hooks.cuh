// Shared pieces of the single-group resampling entry points: the layout
// of their device arrays in one region, and the kernel sequence.
#pragma once

#include <cuda_runtime.h>

#include <string>
#include <vector>

#include "engine/filter.cuh"
#include "engine/layout.hpp"

namespace dust2gpu {
namespace engine {

struct hook_buffers {
  filter_view f{};
  int n_tiles = 0;
};

// Bytes of device memory the arrays for n weights occupy.
std::size_t hook_scratch_bytes(std::size_t n, int tile_size);

// Lay the arrays out in `base` (hook_scratch_bytes(n) bytes, 256-byte
// aligned) and fill the per-group scalars and the n_tiles tiles (a host
// array; nothing is allocated on the host or the device).
void hook_layout(char* base, std::size_t n, const tile* tiles, int n_tiles,
                 hook_buffers& hb, cudaStream_t s);

// Systematic resampling of the raw weights in hb.f.w with uniform u;
// indices (group-local) are left in hb.f.idx.
void hook_resample(hook_buffers& hb, double u, int tile_size, int serial,
                   int* fallback_count, cudaStream_t s);

}  // namespace engine
}  // namespace dust2gpu
