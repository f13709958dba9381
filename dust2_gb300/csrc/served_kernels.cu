// System-independent kernels of the likelihood server (engine/served.cuh):
// request start, end-of-tick bookkeeping, and the reorder of running
// sessions only.
#include <cmath>

#include "engine/device.cuh"
#include "engine/filter.cuh"
#include "engine/served.cuh"

namespace dust2gpu {
namespace engine {

// Reset the filter state of the listed slots (filter.hpp:156-175: ll = 0)
// and mark them running from their first observation.
__global__ void k_served_begin(served_start_list list, filter_view f,
                               int* active, int* obs, int* starting,
                               int* slot_error) {
  const int i = threadIdx.x;
  if (i >= list.n) {
    return;
  }
  const int g = list.slot[i];
  active[g] = 1;
  starting[g] = 1;
  obs[g] = 0;
  f.ll[g] = 0;
  f.gkey[g] = ordered_key(-INFINITY);
  f.gnz[g] = 0;
  f.gflag[g] = 0;
  f.mode[g] = MODE_KEEP;
  slot_error[g] = 0;
}

// After a tick: each running slot moves to its next observation and stops
// after its last; the "starting" marks of the tick are cleared.
__global__ void k_served_advance(int* active, const served_slot* slots,
                                 int* obs, int* starting, int n_slots) {
  const int g = blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= n_slots) {
    return;
  }
  starting[g] = 0;
  if (!active[g]) {
    return;
  }
  const int o = obs[g] + 1;
  obs[g] = o;
  if (o >= slots[g].n_obs) {
    active[g] = 0;
  }
}

// k_reorder (discrete/system.hpp:170-181) restricted to running slots;
// idle sessions keep their state where it is.
__global__ void k_reorder_active(const double* __restrict__ src,
                                 double* __restrict__ dst, int stride,
                                 int n_state, const tile* __restrict__ tiles,
                                 const int* __restrict__ active,
                                 const int* __restrict__ group_offset,
                                 const int* __restrict__ index,
                                 const int* __restrict__ group_mode) {
  const tile tl = tiles[blockIdx.x];
  if (!active[tl.group] || static_cast<int>(threadIdx.x) >= tl.count) {
    return;
  }
  const int k = tl.start + threadIdx.x;
  const bool move = group_mode[tl.group] != MODE_KEEP;
  const int from = move ? group_offset[tl.group] + index[k] : k;
  for (int s = 0; s < n_state; ++s) {
    dst[static_cast<long>(s) * stride + k] =
      src[static_cast<long>(s) * stride + from];
  }
}

}  // namespace engine
}  // namespace dust2gpu
