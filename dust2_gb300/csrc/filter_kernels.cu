// System-independent kernels of the particle filter: weight
// normalisation, per-group log-sum-exp and resampling (see
// engine/filter.cuh for the algorithm and its exactness argument).
#include <cfloat>
#include <cmath>

#include <cooperative_groups.h>

#include "dust2gpu/exact_sum.hpp"
#include "dust2gpu/math.hpp"
#include "dust2gpu/random.hpp"
#include "engine/device.cuh"
#include "engine/filter.cuh"

namespace dust2gpu {
namespace engine {

__global__ void k_filter_reset(filter_view f, int n_groups) {
  const int g = blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= n_groups) {
    return;
  }
  f.ll[g] = 0;
  f.gkey[g] = ordered_key(-INFINITY);
  f.gnz[g] = 0;
  f.gflag[g] = 0;
  f.mode[g] = MODE_KEEP;
}

// Weight sums are built in a fixed structure that does not depend on how
// particles are cut into tiles: each 32-particle chunk of a group (one
// warp) is scanned by a warp scan, and each group's chunk totals by warp
// scans of 32 chunks with a running carry.  The log-likelihood and the
// resampling indices are therefore the same for any tile size.

// A particle's weight relative to the group's largest, exp(w - max); a
// NaN log weight counts as weight 0.
__device__ __forceinline__ double scaled_weight(const filter_view& f, int k,
                                                double mx) {
  const double w = f.w[k];
  return (w != w) ? 0.0 : math::exp(w - mx);
}

// exp(w - max), the chunk-local inclusive prefix sums and chunk totals.
__global__ void k_weights(filter_view f) {
  const tile tl = f.tiles[blockIdx.x];
  const int g = tl.group;
  if (!f.active[g] || !f.gnz[g] || f.n_particles[g] == 1) {
    return;
  }
  const double mx = ordered_value(f.gkey[g]);
  if (mx == -INFINITY) {
    return;
  }
  const int warp = threadIdx.x >> 5;
  if (32 * warp >= tl.count) {
    return;  // the whole warp is past the tile's particles
  }
  const bool valid = static_cast<int>(threadIdx.x) < tl.count;
  const int k = tl.start + threadIdx.x;
  const double e = valid ? scaled_weight(f, k, mx) : 0.0;
  const double incl = warp_inclusive_scan(e);
  if (valid) {
    f.ew[k] = e;
    f.pre[k] = incl;
  }
  if ((threadIdx.x & 31) == 31) {
    f.chunk_sum[f.chunk_first[g] + tl.local / 32 + warp] = incl;
  }
}

// Whether a group's weights are summed at this observation: some weight
// is not 0, more than one particle, and not every log weight -Inf.
__device__ __forceinline__ bool group_has_sum(const filter_view& f, int g) {
  return f.gnz[g] != 0 && f.n_particles[g] > 1 &&
    ordered_value(f.gkey[g]) != -INFINITY;
}

// The next draw of a group's filter stream (filter.hpp:75), taken before
// it is known to be needed; group_finish keeps it, and the advanced
// stream, only for a group with data.
struct group_uniform {
  random::rng_state r;
  double u;
};

__device__ group_uniform draw_group_uniform(const filter_view& f, int g) {
  group_uniform d{};
  for (int w = 0; w < 4; ++w) {
    d.r.state[w] = f.frng[8 * g + w];
  }
  d.r.deterministic = false;
  d.u = random::random_real(d.r);
  return d;
}

// One thread, given the group's weight total and the draw: log-likelihood
// increment, mode and resampling uniform; then clear the per-observation
// reductions.
__device__ void group_finish(const filter_view& f, int g, double tot,
                             const group_uniform& d) {
  const int n = f.n_particles[g];
  const bool nz = f.gnz[g] != 0;
  const double mx = ordered_value(f.gkey[g]);
  int mode = MODE_KEEP;
  if (nz) {
    const double mean = tot / n;
    double inc;
    if (n == 1) {
      inc = f.w[f.offset[g]];
      mode = MODE_FIRST;
    } else if (mx == -INFINITY) {
      inc = -INFINITY;
      mode = MODE_FIRST;
    } else {
      inc = math::log(mean) + mx;
      mode = MODE_RESAMPLE;
    }
    f.ll[g] += inc;
    for (int w = 0; w < 4; ++w) {
      f.frng[8 * g + w] = d.r.state[w];
    }
    f.gu[g] = d.u;
    f.gtot[g] = tot;
    f.guu0[g] = tot * d.u / n;
    f.gdu[g] = mean;
  }
  f.mode[g] = mode;
  f.gkey[g] = ordered_key(-INFINITY);
  f.gnz[g] = 0;
  f.gflag[g] = (mode == MODE_RESAMPLE && *f.force_serial) ? 1 : 0;
}

// One warp of a running group: chunk offsets, then group_finish.
__device__ void group_update(const filter_view& f, int g, int lane) {
  const double tot = group_has_sum(f, g) ?
    group_chunk_offsets(f, g, lane) : 0.0;
  if (lane == 0) {
    group_finish(f, g, tot, draw_group_uniform(f, g));
  }
}

// group_chunk_offsets with the whole block: warp w scans windows w,
// w + (warps), ... of 32 chunks at once, thread 0 accumulates the window
// totals in window order (the running carry of the one-warp loop), and
// each warp adds its window's carry.  Every sum is the one the one-warp
// loop forms, so the results are the same bits; a group of 32,768
// particles takes one pass instead of 32 dependent ones.  The total is
// returned to thread 0.
__device__ double group_chunk_offsets_block(const filter_view& f, int g) {
  __shared__ double win_total[32];
  __shared__ double win_carry[32];
  const int lane = threadIdx.x & 31;
  const int warp = threadIdx.x >> 5;
  const int n_warps = blockDim.x >> 5;
  const int c0 = f.chunk_first[g];
  const int nc = f.chunk_count[g];
  const int n_win = (nc + 31) >> 5;
  double carry = 0;  // thread 0
  for (int wb = 0; wb < n_win; wb += n_warps) {
    const int w = wb + warp;
    const int c = 32 * w + lane;
    double v = 0, excl = 0;
    if (w < n_win) {
      v = c < nc ? f.chunk_sum[c0 + c] : 0.0;
      const double incl = warp_inclusive_scan(v);
      excl = __shfl_up_sync(0xffffffffu, incl, 1);
      if (lane == 0) {
        excl = 0;
      }
      if (lane == 31) {
        win_total[warp] = incl;
      }
    }
    __syncthreads();
    if (threadIdx.x == 0) {
      const int m = min(n_warps, n_win - wb);
      for (int j = 0; j < m; ++j) {
        win_carry[j] = carry;
        carry = carry + win_total[j];
      }
    }
    __syncthreads();
    if (w < n_win && c < nc) {
      const double off = win_carry[warp] + excl;
      f.chunk_off[c0 + c] = off;
      f.chunk_sum[c0 + c] = off + v;
    }
  }
  return carry;
}

// One block (a multiple of 32 threads, at most 1024) per group.
__global__ void k_group(filter_view f, int n_groups) {
  const int g = blockIdx.x;
  if (g >= n_groups || !f.active[g]) {
    return;
  }
  const double tot = group_has_sum(f, g) ?
    group_chunk_offsets_block(f, g) : 0.0;
  __syncthreads();  // every thread has read the reductions group_finish clears
  if (threadIdx.x == 0) {
    group_finish(f, g, tot, draw_group_uniform(f, g));
  }
}

// What the resampling search of one group reads: its chunk ends and
// offsets (left by k_group), its chunk-local prefix sums and the targets'
// start and spacing.  The arrays may be the global ones or copies.
struct search_view {
  const double* chunk_end;  // [nc]
  const double* chunk_off;  // [nc]
  const double* pre;        // [n]
  int n;
  int nc;
  double uu0;
  double du;
};

__device__ __forceinline__ search_view group_search(const filter_view& f,
                                                    int g) {
  const int c0 = f.chunk_first[g];
  return search_view{f.chunk_sum + c0, f.chunk_off + c0,
                     f.pre + f.offset[g], f.n_particles[g],
                     f.chunk_count[g], f.guu0[g], f.gdu[g]};
}

// Prefix sum Q_m (weights 0..m of the group) for group-local index m.
__device__ __forceinline__ double prefix_at(const search_view& sv, int m) {
  return sv.chunk_off[m >> 5] + sv.pre[m];
}

// The resampling index of particle i of a group being resampled; an
// ambiguous decision is recorded in *flag.
__device__ int resample_index(const search_view& sv, int i, int* flag) {
  const int n = sv.n;
  const double uu = sv.uu0 + static_cast<double>(i) * sv.du;
  // first chunk whose last prefix (its end, left in chunk_sum by k_group)
  // reaches uu; every value compared is >= +0, so the comparisons are
  // taken on the bits
  const int nc = sv.nc;
  int lo = 0, hi = nc;
  while (lo < hi) {
    const int mid = (lo + hi) >> 1;
    if (math::le_nonneg(uu, sv.chunk_end[mid])) {
      hi = mid;
    } else {
      lo = mid + 1;
    }
  }
  int m;
  if (lo == nc) {
    m = n - 1;  // past the end: the serial loop stops at j == n
  } else {
    const int first = lo * 32;
    const int last = min(n, first + 32) - 1;
    int a = first, b = last;
    const double off = sv.chunk_off[lo];
    const double* pre = sv.pre;
    while (a < b) {
      const int mid = (a + b) >> 1;
      if (math::le_nonneg(uu, off + pre[mid])) {
        b = mid;
      } else {
        a = mid + 1;
      }
    }
    m = a;
  }
  // Robustness of the decision against serial-summation rounding.  The
  // serial loop returns m exactly when its prefix of m weights is below
  // the target (needed only for m > 0: index 0 results whether the target
  // is below or inside the first weight) and its prefix of m + 1 weights
  // reaches it (needed only for m < n - 1: the loop stops at the last
  // particle anyway).
  //
  // Bound, with u = 2^-53: a serial prefix of k weights differs from the
  // exact sum S_k by at most (k - 1) u S_k.  A prefix here is a sum of
  // non-negative terms by a tree of depth at most L = 18 + ceil(nc / 32)
  // (5 levels within a chunk, 5 for the chunk total, 5 across a window
  // of 32 chunks, one per earlier window, and the joins), so within
  // L u S_k; each weight may differ from the other side's exp by 2 ulp
  // (4 u S_k); the target computed from either total differs by at most
  // (n + L + 10) u uu.  So a decision is safe when the prefix is farther
  // than (k + n + 2L + 16) u max(S_k, uu) from the target (5% slack on
  // top).
  const double L = 18.0 + static_cast<double>((nc + 31) >> 5);
  const double eps = 0x1.0p-53 * 1.05;
  bool ok = true;
  if (m > 0) {
    const double p = prefix_at(sv, m - 1);
    const double margin = eps * (m + n + 2 * L + 16) * fmax(p, uu);
    ok = ok && p < uu - margin;
  }
  if (m < n - 1) {
    const double q = prefix_at(sv, m);
    const double margin = eps * (m + 1 + n + 2 * L + 16) * fmax(q, uu);
    ok = ok && q >= uu + margin;
  }
  if (!ok) {
    atomicOr(flag, 1);
  }
  return m;
}

__global__ void k_resample(filter_view f) {
  const tile tl = f.tiles[blockIdx.x];
  const int g = tl.group;
  if (!f.active[g]) {
    return;
  }
  const int mode = f.mode[g];
  if (mode == MODE_KEEP || static_cast<int>(threadIdx.x) >= tl.count) {
    return;
  }
  const int k = tl.start + threadIdx.x;
  if (mode == MODE_FIRST) {
    f.idx[k] = 0;
    return;
  }
  f.idx[k] = resample_index(group_search(f, g), tl.local + threadIdx.x,
                            f.gflag + g);
}

// The reference algorithm (filter_details.hpp:45-74) for groups with an
// ambiguous parallel decision.  Its running sum ww_j = fl(ww_{j-1} + w_j)
// is reproduced exactly (exact_running_sums); the reference's walk over
// particles then equals, for each particle, the first j with ww_j >= uu_i
// (ww is non-decreasing because the weights are non-negative and
// rounding is monotone), which the whole block finds by binary search.
// The running sums overwrite this group's `pre` entries.
//
// Exact running sums in parallel (dust2gpu/exact_sum.hpp): within one
// binade of the running sum, every step adds an integer number of grid
// units that does not depend on the sum, so the block scans the units of
// a window of weights, and every position before the first one that
// leaves the binade (or is a halfway case) gets its exact value.  That
// one step is taken with a real FP64 add, and the next window starts
// after it.  A run of weights whose breaks come within 32 positions of
// each other (the first steps, when the sum is small) is added one by one
// by thread 0, which bounds the cost by about that of the plain loop.
// A sum that is Inf, NaN or negative (weights outside the contract)
// continues one by one.  The steps taken are the reference's own, so the
// sums are the same bits; a group of 32,768 particles takes ~50
// block-wide windows instead of 32,768 dependent FP64 adds.

// Inclusive block scan of saturating sums (blockDim.x a multiple of 32,
// at most 1024).  Ends with the block synchronised.
__device__ unsigned long long block_scan_sat(unsigned long long v,
                                             unsigned long long* warp_tot) {
  const int lane = threadIdx.x & 31;
  const int warp = threadIdx.x >> 5;
  const int n_warps = blockDim.x >> 5;
  for (int off = 1; off < 32; off <<= 1) {
    const unsigned long long t = __shfl_up_sync(0xffffffffu, v, off);
    if (lane >= off) {
      v = exact_sum::sat_add(v, t);
    }
  }
  if (lane == 31) {
    warp_tot[warp] = v;
  }
  __syncthreads();
  if (warp == 0) {
    unsigned long long x = lane < n_warps ? warp_tot[lane] : 0;
    for (int off = 1; off < 32; off <<= 1) {
      const unsigned long long t = __shfl_up_sync(0xffffffffu, x, off);
      if (lane >= off) {
        x = exact_sum::sat_add(x, t);
      }
    }
    if (lane < n_warps) {
      warp_tot[lane] = x;
    }
  }
  __syncthreads();
  if (warp > 0) {
    v = exact_sum::sat_add(v, warp_tot[warp - 1]);
  }
  __syncthreads();  // warp_tot may be rewritten by the next call
  return v;
}

// ser[j] = fl(ser[j-1] + w[j]), ser[0] = w[0], for n >= 1 non-negative
// weights, by the whole block; returns ser[n-1] to every thread.
__device__ double exact_running_sums(const double* w, double* ser, int n) {
  __shared__ unsigned long long warp_tot[32];
  __shared__ int first_break;
  __shared__ int s_j0;
  __shared__ double s_sum;
  const int nb = static_cast<int>(blockDim.x);
  const int t = threadIdx.x;
  if (t == 0) {
    s_j0 = 0;
    s_sum = w[0];  // fl(0 + w_0)
    ser[0] = w[0];
  }
  __syncthreads();
  for (;;) {
    const int j0 = s_j0;
    const double sum = s_sum;
    if (j0 >= n - 1) {
      break;
    }
    const exact_sum::grid gr = exact_sum::grid_of(sum);
    if (!gr.ok) {  // Inf, NaN or negative: the rest one by one
      if (t == 0) {
        double acc = sum;
        for (int j = j0 + 1; j < n; ++j) {
          acc = acc + w[j];
          ser[j] = acc;
        }
        s_sum = acc;
      }
      __syncthreads();
      break;
    }
    const int j = j0 + 1 + t;
    bool tie = false;
    const unsigned long long r =
      j < n ? exact_sum::grid_units(w[j], gr.e_grid, &tie) : 0;
    if (t == 0) {
      first_break = nb;
    }
    const unsigned long long m = gr.count + block_scan_sat(r, warp_tot);
    if (j < n && exact_sum::is_break(m, tie)) {
      atomicMin(&first_break, t);
    }
    __syncthreads();
    const int first = first_break;
    if (t < first && j < n) {
      ser[j] = exact_sum::grid_value(gr, m);
    }
    __syncthreads();
    if (t == 0) {
      const int jb = j0 + 1 + first;
      if (first < 32 && jb < n) {
        const int stop = min(n - 1, j0 + 128);
        double acc = ser[jb - 1];
        for (int q = jb; q <= stop; ++q) {
          acc = acc + w[q];
          ser[q] = acc;
        }
        s_sum = acc;
        s_j0 = stop;
      } else if (first < nb && jb < n) {
        const double v = ser[jb - 1] + w[jb];
        ser[jb] = v;
        s_sum = v;
        s_j0 = jb;
      } else {
        const int last = min(n - 1, j0 + nb);
        s_sum = ser[last];
        s_j0 = last;
      }
    }
    __syncthreads();
  }
  return s_sum;
}

// The whole block resamples group g serially and counts it.
__device__ void serial_fallback(const filter_view& f, int g, int* count) {
  __shared__ double total;
  const int n = f.n_particles[g];
  const double* w = f.ew + f.offset[g];
  double* ser = f.pre + f.offset[g];
  int* idx = f.idx + f.offset[g];
  const double run = exact_running_sums(w, ser, n);
  if (threadIdx.x == 0) {
    total = run;
    count[g] += 1;
    f.gflag[g] = 0;
  }
  __syncthreads();
  const double tot = total;
  const double u = f.gu[g];
  const double uu0 = tot * u / n;
  const double du = tot / n;
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    const double uu = uu0 + static_cast<double>(i) * du;
    int a = 0, b = n;  // first m with ser[m] >= uu, or n
    while (a < b) {
      const int mid = (a + b) >> 1;
      if (math::le_nonneg(uu, ser[mid])) {
        b = mid;
      } else {
        a = mid + 1;
      }
    }
    idx[i] = a == n ? n - 1 : a;
  }
}

__global__ void __launch_bounds__(FALLBACK_THREADS)
k_fallback_count(filter_view f, int* count) {
  const int g = blockIdx.x;
  if (!f.active[g] || f.mode[g] != MODE_RESAMPLE || !f.gflag[g]) {
    return;
  }
  serial_fallback(f, g, count);
}

// The tail of an observation for groups of at most TAIL_MAX_PARTICLES
// particles, as one launch: k_weights, k_group, k_resample,
// k_fallback_count and k_reorder.  Each group is a cluster of
// TAIL_CLUSTER blocks (warp w of block r holds the group's chunk
// 4r + w), so the FP64 work of the group is spread over the FP64 units of
// TAIL_CLUSTER SMs, one warp per SM partition, and the phases are
// separated by cluster barriers, whose release/acquire semantics make the
// global writes of one phase visible to the next.  Every value is
// computed by the same device functions in the same order as by the
// separate kernels, so the results are the same bits.  To shorten the
// chain of dependent loads, the group's filter draw is taken before the
// weights are summed, and each block searches shared-memory copies of the
// group's prefix sums.  Every block of a running group takes all four
// barriers whatever the data (the fourth as arrive and wait around the
// state copy when no serial fallback runs; that choice is the same in
// every block), so no barrier can wait for a block that has left.  The
// state of every group moves from src to dst (in place for groups that
// keep their particles), as k_reorder does.
__global__ void __cluster_dims__(TAIL_CLUSTER, 1, 1)
__launch_bounds__(TAIL_BLOCK)
k_tail_cluster(filter_view f, int* count, const double* __restrict__ src,
               double* __restrict__ dst, int stride, int n_state) {
  __shared__ int flag;  // ambiguous decisions, used in block rank 0
  // copies of the group's search arrays (n <= TAIL_MAX_PARTICLES)
  __shared__ double s_end[TAIL_MAX_PARTICLES / 32];
  __shared__ double s_off[TAIL_MAX_PARTICLES / 32];
  __shared__ double s_pre[TAIL_MAX_PARTICLES];
  namespace cg = cooperative_groups;
  cg::cluster_group cluster = cg::this_cluster();
  const int g = blockIdx.x / TAIL_CLUSTER;
  const int rank = static_cast<int>(cluster.block_rank());
  const int i = rank * TAIL_BLOCK + static_cast<int>(threadIdx.x);
  const bool active = f.active[g] != 0;
  const int n = f.n_particles[g];
  const int base = f.offset[g];
  const int k = base + i;
  int from = k;  // the source of this particle's state
  bool arrived = false;  // barrier 4 arrived on, still to be waited for
  if (active) {
    const bool summed = group_has_sum(f, g);
    group_uniform draw{};
    if (rank == 0 && threadIdx.x == 0) {
      flag = 0;
      draw = draw_group_uniform(f, g);  // independent of the weights
    }
    if (summed && 32 * (i >> 5) < n) {
      const bool valid = i < n;
      const double e =
        valid ? scaled_weight(f, k, ordered_value(f.gkey[g])) : 0.0;
      const double incl = warp_inclusive_scan(e);
      if (valid) {
        f.ew[k] = e;
        f.pre[k] = incl;
      }
      if ((i & 31) == 31) {
        f.chunk_sum[f.chunk_first[g] + (i >> 5)] = incl;
      }
    }
    cluster.sync();  // 1: chunk totals and the zeroed flag are in place
    if (rank == 0 && threadIdx.x < 32) {
      const double tot =
        summed ? group_chunk_offsets(f, g, threadIdx.x) : 0.0;
      if (threadIdx.x == 0) {
        group_finish(f, g, tot, draw);
      }
    }
    cluster.sync();  // 2: mode, offsets and the target spacing
    const int mode = f.mode[g];
    const double uu0 = f.guu0[g];
    const double du = f.gdu[g];
    const int c0 = f.chunk_first[g];
    const int nc = f.chunk_count[g];
    int* flag0 = cluster.map_shared_rank(&flag, 0);
    if (mode == MODE_RESAMPLE) {
      for (int j = threadIdx.x; j < nc; j += TAIL_BLOCK) {
        s_end[j] = f.chunk_sum[c0 + j];
        s_off[j] = f.chunk_off[c0 + j];
      }
      for (int j = threadIdx.x; j < n; j += TAIL_BLOCK) {
        s_pre[j] = f.pre[base + j];
      }
      __syncthreads();
      if (i < n) {
        const search_view sv{s_end, s_off, s_pre, n, nc, uu0, du};
        const int m = resample_index(sv, i, flag0);
        f.idx[k] = m;
        from = base + m;
      }
    } else if (mode == MODE_FIRST && i < n) {
      f.idx[k] = 0;
      from = base;
    }
    cluster.sync();  // 3: every decision and its flag
    // the same for every block: rank 0's flag is final and no longer
    // written, the force flag is read-only
    const bool serial = mode == MODE_RESAMPLE &&
      (*flag0 != 0 || *f.force_serial != 0);
    if (serial) {
      if (rank == 0) {
        serial_fallback(f, g, count);
      }
      cluster.sync();  // 4: the serial indices are in place
      if (i < n) {
        from = base + f.idx[k];
      }
    } else {
      // 4, split: rank 0's shared memory must outlive every block's read
      // of its flag, but the copy below need not wait
      cluster.barrier_arrive();
      arrived = true;
    }
  }
  if (i < n) {
    for (int s = 0; s < n_state; ++s) {
      dst[static_cast<long>(s) * stride + k] =
        src[static_cast<long>(s) * stride + from];
    }
  }
  if (arrived) {
    cluster.barrier_wait();
  }
}

// After the reorder of a data time: the saved state entries of each
// particle of the running groups, and where its state came from (the
// group-local resampling index; itself when the group was not resampled).
__global__ void k_save_history(const double* state, int stride,
                               const int* index_state, int n_save,
                               const tile* tiles, const int* active,
                               const int* mode, const int* idx,
                               double* hist_state, int* hist_order) {
  const tile tl = tiles[blockIdx.x];
  if (!active[tl.group] || static_cast<int>(threadIdx.x) >= tl.count) {
    return;
  }
  const int k = tl.start + threadIdx.x;
  for (int s = 0; s < n_save; ++s) {
    hist_state[static_cast<long>(s) * stride + k] =
      state[static_cast<long>(index_state[s]) * stride + k];
  }
  if (hist_order != nullptr) {
    hist_order[k] = mode[tl.group] == MODE_KEEP ? tl.local + threadIdx.x :
      idx[k];
  }
}

// trajectories.hpp:199-268 (export_snapshots with reorder): as
// k_export_history, writing only at the snapshot data times.
// out: [snapshot][group][particle][state]
__global__ void k_export_snapshots(const double* snap_state,
                                   const int* hist_order, int n_times,
                                   const int* snap_obs, int n_snap,
                                   int n_state, int stride,
                                   const int* group_offset, const int* groups,
                                   int n_groups_out, const int* select,
                                   int n_particles_out, double* out) {
  const long t = static_cast<long>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (t >= static_cast<long>(n_groups_out) * n_particles_out) {
    return;
  }
  const int go = static_cast<int>(t / n_particles_out);
  const int jo = static_cast<int>(t % n_particles_out);
  const int base = group_offset[groups[go]];
  int j = select != nullptr ? select[go] : jo;
  int sn = n_snap - 1;
  for (int i = n_times - 1; i >= 0 && sn >= 0; --i) {
    if (snap_obs[sn] == i) {
      const double* ss = snap_state + static_cast<long>(sn) * n_state * stride;
      double* dst = out + ((static_cast<long>(sn) * n_groups_out + go) *
                           n_particles_out + jo) * n_state;
      for (int s = 0; s < n_state; ++s) {
        dst[s] = ss[static_cast<long>(s) * stride + base + j];
      }
      --sn;
    }
    if (hist_order != nullptr) {
      j = hist_order[static_cast<long>(i) * stride + base + j];
    }
  }
}

// trajectories.hpp:135-190 (export_state with reorder): one thread per
// output particle walks back through the saved indices from the last data
// time (hist_order null: no reordering, as for deterministic likelihoods).
// out: [time][group][particle][state].
__global__ void k_export_history(const double* hist_state,
                                 const int* hist_order, int n_times,
                                 int n_save, int stride,
                                 const int* group_offset, const int* groups,
                                 int n_groups_out, const int* select,
                                 int n_particles_out, double* out) {
  const long t = static_cast<long>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (t >= static_cast<long>(n_groups_out) * n_particles_out) {
    return;
  }
  const int go = static_cast<int>(t / n_particles_out);
  const int jo = static_cast<int>(t % n_particles_out);
  const int base = group_offset[groups[go]];
  int j = select != nullptr ? select[go] : jo;
  for (int i = n_times - 1; i >= 0; --i) {
    const double* hs = hist_state + static_cast<long>(i) * n_save * stride;
    double* dst = out + ((static_cast<long>(i) * n_groups_out + go) *
                         n_particles_out + jo) * n_save;
    for (int s = 0; s < n_save; ++s) {
      dst[s] = hs[static_cast<long>(s) * stride + base + j];
    }
    if (hist_order != nullptr) {
      j = hist_order[static_cast<long>(i) * stride + base + j];
    }
  }
}

}  // namespace engine
}  // namespace dust2gpu
