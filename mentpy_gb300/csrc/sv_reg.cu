// Instantiations of the register-resident statevector kernel for one window
// size (compiled once per size with -DSV_W=<w>).
#include "dispatch.h"
#include "sv_reg.cuh"

#ifndef SV_W
#error "compile with -DSV_W=<window>"
#endif

#define MBQC_CAT2(a, b) a##b
#define MBQC_CAT(a, b) MBQC_CAT2(a, b)

namespace mbqc {

// Dynamic shared memory of a launch: the block's warps, each with a chunk of
// a.kc steps (above the default 48 KB the kernel opts in once).
template <typename T, int W, int LL, bool GEN, bool HOST = false>
static int launch_one(const SvArgs &a, int blocks, int threads, cudaStream_t s, const char *what) {
  auto k = sv_fwd_reg<T, W, LL, GEN, HOST>;
  const size_t smem = (size_t)(threads / 32) * sv_warp_smem(W, LL, (int)sizeof(T) * 2, a.kc, GEN);
  if (smem > 48 * 1024) {
    static bool opted = false;
    if (!opted) {
      int rc = cuda_check(cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, 64 * 1024),
                          "sv_fwd_reg shared memory");
      if (rc) return rc;
      opted = true;
    }
  }
  return cuda_check(launch_pdl(k, dim3(blocks), dim3(threads), smem, s, a), what);
}

template <typename T, int W, int LL>
static int launch_ll(int ll, const SvArgs &a, int blocks, int threads, cudaStream_t s) {
  if constexpr (LL > 5 || LL > W) {
    return fail(MBQC_E_UNSUPPORTED, "statevector register kernel: no variant ll=%d for window %d", ll, W);
  } else {
    constexpr bool exists = (W - LL <= 5) && (sizeof(T) == 4 || LL == sv_f64_ll(W));
    if (ll == LL) {
      if constexpr (exists) {
        if constexpr (sizeof(T) == 4) {
          if (a.flags & MBQC_F_HOST_INPUTS) return launch_one<T, W, LL, false, true>(a, blocks, threads, s, "sv_fwd_reg");
        }
        return launch_one<T, W, LL, false>(a, blocks, threads, s, "sv_fwd_reg");
      } else {
        return fail(MBQC_E_UNSUPPORTED, "statevector register kernel: no variant ll=%d for window %d",
                    ll, W);
      }
    }
    return launch_ll<T, W, LL + 1>(ll, a, blocks, threads, s);
  }
}

int MBQC_CAT(launch_sv_reg_f32_w, SV_W)(int ll, const SvArgs &a, int blocks, int threads, cudaStream_t s) {
  return launch_ll<float, SV_W, 0>(ll, a, blocks, threads, s);
}
int MBQC_CAT(launch_sv_reg_f64_w, SV_W)(int ll, const SvArgs &a, int blocks, int threads, cudaStream_t s) {
  return launch_ll<double, SV_W, 0>(ll, a, blocks, threads, s);
}
int MBQC_CAT(launch_sv_reg_gen_f32_w, SV_W)(const SvArgs &a, int blocks, int threads, cudaStream_t s) {
  return launch_one<float, SV_W, sv_gen_ll(SV_W), true>(a, blocks, threads, s, "sv_fwd_reg (general planes)");
}
int MBQC_CAT(launch_sv_reg_gen_f64_w, SV_W)(const SvArgs &a, int blocks, int threads, cudaStream_t s) {
  return launch_one<double, SV_W, sv_f64_ll(SV_W), true>(a, blocks, threads, s, "sv_fwd_reg (general planes)");
}

}  // namespace mbqc
