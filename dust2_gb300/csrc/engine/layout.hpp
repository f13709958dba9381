// How particles of (possibly uneven) parameter groups are laid out in
// device memory, and how they are cut into tiles of one CUDA block each.
//
// dust2 stores state particle-major, `state_[(n_particles*g + j)*n_state
// + s]` (inst/include/dust2/discrete/system.hpp:72-73), with the same
// number of particles in every group.  Here state is structure-of-arrays,
// `state[s * stride + k]` with k the global particle index (group-major),
// so that consecutive threads touch consecutive addresses; groups may have
// different particle counts (the batched workloads need that), and a tile
// never straddles two groups, so a block loads its group's parameters
// once into shared memory and reduces over its group with block-wide
// primitives.
#pragma once

#include <algorithm>
#include <stdexcept>
#include <vector>

namespace dust2gpu {
namespace engine {

struct tile {
  int group;  // parameter group of every particle in the tile, or -1
              // for a packed tile holding particles of several groups
  int start;  // global index of the first particle
  int count;  // particles in the tile (<= tile size)
  int local;  // index of the first particle within its group (-1 mixed)
};

struct group_layout {
  std::vector<int> n_particles;  // per group
  std::vector<int> offset;       // global index of a group's first particle
  std::vector<int> tile_first;   // first tile of each group
  std::vector<int> tile_count;   // tiles in each group
  // Chunks: runs of 32 particles of one group (warp-sized, group-local
  // indices 32c .. 32c+31), the units of the filter's weight sums.
  std::vector<int> chunk_first;  // first chunk of each group
  std::vector<int> chunk_count;  // chunks in each group
  int n_chunks = 0;
  std::vector<tile> tiles;
  // Packed tiles: consecutive runs of tile_size particles whatever their
  // group, used by the per-particle kernels that need no reduction over a
  // group when groups are small (many one-particle groups would otherwise
  // leave one busy thread per block).  particle_group gives each
  // particle's group.
  std::vector<tile> packed;
  std::vector<int> particle_group;
  bool use_packed = false;
  int n_groups = 0;
  int n_total = 0;
  int stride = 0;                // SoA stride, a multiple of 32
  int tile_size = 0;
  bool uniform = true;           // all groups have the same particle count

  group_layout() = default;

  group_layout(const std::vector<int>& n, int tile_size_) :
    n_particles(n), tile_size(tile_size_) {
    if (n.empty()) {
      throw std::runtime_error("Expected at least one group");
    }
    if (tile_size <= 0 || tile_size % 32 != 0 || tile_size > 1024) {
      throw std::runtime_error("tile size must be a multiple of 32 <= 1024");
    }
    n_groups = static_cast<int>(n.size());
    long total = 0;
    for (int g = 0; g < n_groups; ++g) {
      if (n[g] < 1) {
        throw std::runtime_error("'n_particles' must be at least 1");
      }
      if (n[g] != n[0]) {
        uniform = false;
      }
      offset.push_back(static_cast<int>(total));
      tile_first.push_back(static_cast<int>(tiles.size()));
      const int nt = (n[g] + tile_size - 1) / tile_size;
      tile_count.push_back(nt);
      chunk_first.push_back(n_chunks);
      chunk_count.push_back((n[g] + 31) / 32);
      n_chunks += (n[g] + 31) / 32;
      for (int t = 0; t < nt; ++t) {
        const int local = t * tile_size;
        const int count = std::min(tile_size, n[g] - local);
        tiles.push_back(tile{g, static_cast<int>(total) + local, count, local});
      }
      total += n[g];
      if (total > (1L << 30)) {
        throw std::runtime_error("too many particles");
      }
    }
    n_total = static_cast<int>(total);
    stride = ((n_total + 31) / 32) * 32;
    // smaller groups than a tile on average: pack them
    use_packed = static_cast<long>(n_total) < static_cast<long>(n_groups) *
      tile_size;
    if (use_packed) {
      particle_group.resize(n_total);
      for (int g = 0; g < n_groups; ++g) {
        std::fill(particle_group.begin() + offset[g],
                  particle_group.begin() + offset[g] + n[g], g);
      }
      for (int start = 0; start < n_total; start += tile_size) {
        const int count = std::min(tile_size, n_total - start);
        const int g0 = particle_group[start];
        const int g1 = particle_group[start + count - 1];
        packed.push_back(g0 == g1 ?
                         tile{g0, start, count, start - offset[g0]} :
                         tile{-1, start, count, -1});
      }
    }
  }

  // The tiles of the per-particle kernels (packed when that helps).
  const std::vector<tile>& run_tiles() const {
    return use_packed ? packed : tiles;
  }

  int n_tiles() const {
    return static_cast<int>(tiles.size());
  }
};

// One-warp tiles of at most `per_tile` particles each (never spanning two
// groups), for the filter's step kernel on small problems: a warp issues
// one FP64 instruction per 64 cycles of its SM partition however many of
// its lanes are active, so a warp's time is its FP64 instruction count,
// which grows with the divergence of its lanes; with fewer particles per
// warp, one warp per partition, a small filter steps faster.
inline std::vector<tile> warp_tiles(const group_layout& L, int per_tile) {
  std::vector<tile> out;
  for (int g = 0; g < L.n_groups; ++g) {
    for (int local = 0; local < L.n_particles[g]; local += per_tile) {
      const int count = std::min(per_tile, L.n_particles[g] - local);
      out.push_back(tile{g, L.offset[g] + local, count, local});
    }
  }
  return out;
}

}  // namespace engine
}  // namespace dust2gpu
