// Array layout of the single-group resampler for callers that supply the
// tiles as a plain array and the memory as one region (used by the entry
// point that allocates nothing; see resample_noalloc.cu).
#include <cuda_runtime.h>

#include "engine/device.cuh"
#include "engine/filter.cuh"
#include "resample_hooks.cuh"

namespace dust2gpu {
namespace engine {

void hook_layout_fixed(char* base, std::size_t n, int tile_size,
                       const tile* tiles, int n_tiles, hook_buffers& hb,
                       cudaStream_t s) {
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
  // every per-group scalar is rewritten here, so nothing left from an
  // earlier call in the same memory is read
  const int h_ints[8] = {1, static_cast<int>(n), 0, 0,
                         static_cast<int>(nc), 0, 0, MODE_RESAMPLE};
  DUST2_CUDA(cudaMemcpyAsync(ints, h_ints, sizeof(h_ints),
                             cudaMemcpyHostToDevice, s));
  const unsigned long long key0 = 0;
  DUST2_CUDA(cudaMemcpyAsync(f.gkey, &key0, 8, cudaMemcpyHostToDevice, s));
  DUST2_CUDA(cudaMemcpyAsync(t_dev, tiles, nt * sizeof(tile),
                             cudaMemcpyHostToDevice, s));
  hb.n_tiles = n_tiles;
  (void)tile_size;
}

}  // namespace engine
}  // namespace dust2gpu
