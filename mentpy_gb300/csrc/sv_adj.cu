// Instantiations of the statevector adjoint kernel for one window size
// (compiled once per size with -DSV_W=<w>, w <= 8).
#include "dispatch.h"
#include "sv_adj.cuh"

#ifndef SV_W
#error "compile with -DSV_W=<window>"
#endif

#define MBQC_CAT2(a, b) a##b
#define MBQC_CAT(a, b) MBQC_CAT2(a, b)

namespace mbqc {

template <typename T>
static int launch_adj(const SvAdjArgs &a, const AdjLaunch &l, cudaStream_t s) {
  constexpr int LL = adj_ll(SV_W, sizeof(T) == 8);
  if constexpr (LL > 5) {
    return fail(MBQC_E_UNSUPPORTED, "FP64 adjoint: window %d > 7", SV_W);
  } else {
  auto k = sv_adj_reg<T, SV_W, LL>;
  if (l.query) {
    int occ = 0;
    if (cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)l.smem) != cudaSuccess)
      return fail(MBQC_E_UNSUPPORTED, "adjoint: %zu bytes of shared memory per block", l.smem);
    int rc = cuda_check(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k, l.threads, l.smem),
                        "occupancy");
    if (rc) return rc;
    *l.occ = occ;
    return MBQC_OK;
  }
  cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)l.smem);
  k<<<l.blocks, l.threads, l.smem, s>>>(a);
  return check_launch("sv_adj_reg");
  }
}

int MBQC_CAT(launch_sv_adj_f32_w, SV_W)(const SvAdjArgs &a, const AdjLaunch &l, cudaStream_t s) {
  return launch_adj<float>(a, l, s);
}
int MBQC_CAT(launch_sv_adj_f64_w, SV_W)(const SvAdjArgs &a, const AdjLaunch &l, cudaStream_t s) {
  return launch_adj<double>(a, l, s);
}

}  // namespace mbqc
