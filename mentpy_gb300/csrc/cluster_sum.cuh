// Sums and barriers over the blocks that share one run: a single block, or
// a thread-block cluster whose blocks each take a slice of every pass over
// the run's window (windows kept in a global workspace slot).
#pragma once

#include <cooperative_groups.h>

namespace mbqc {

// Sum of NV values (the same in every thread of each block) over the cluster:
// rank r's partials from its shared memory, in rank order.  cred holds two
// buffers of 4 (alternating calls): a buffer is written again two calls
// later, after a cluster barrier that every reader of it has passed.
template <int CS, int NV>
__device__ __forceinline__ void cluster_sum(float (&v)[NV], float *cred, int &cpar) {
  if constexpr (CS > 1) {
    namespace cg = cooperative_groups;
    cg::cluster_group cl = cg::this_cluster();
    float *buf = cred + cpar * 4;
    if (threadIdx.x == 0) {
#pragma unroll
      for (int j = 0; j < NV; ++j) buf[j] = v[j];
    }
    cl.sync();
#pragma unroll
    for (int j = 0; j < NV; ++j) v[j] = 0.f;
#pragma unroll
    for (int r = 0; r < CS; ++r) {
      const float *rb = cl.map_shared_rank(buf, r);
#pragma unroll
      for (int j = 0; j < NV; ++j) v[j] += rb[j];
    }
    cpar ^= 1;
  }
}

// a barrier over the run's blocks (the block, or the cluster)
template <int CS>
__device__ __forceinline__ void run_barrier() {
  if constexpr (CS > 1)
    cooperative_groups::this_cluster().sync();
  else
    __syncthreads();
}

}  // namespace mbqc
