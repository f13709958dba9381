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
// aligned) and fill the per-group scalars and tiles.
void hook_layout(char* base, std::size_t n, int tile_size,
                 const std::vector<tile>& tiles, hook_buffers& hb,
                 cudaStream_t s);

// As hook_layout, with the tiles given as a plain array (no container),
// for the entry point that must not allocate.
void hook_layout_fixed(char* base, std::size_t n, int tile_size,
                       const tile* tiles, int n_tiles, hook_buffers& hb,
                       cudaStream_t s);

// Systematic resampling of the raw weights in hb.f.w with uniform u;
// indices (group-local) are left in hb.f.idx.
void hook_resample(hook_buffers& hb, double u, int tile_size, int serial,
                   int* fallback_count, cudaStream_t s);

}  // namespace engine
}  // namespace dust2gpu
