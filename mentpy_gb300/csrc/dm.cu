// Density-matrix entry point of the C ABI and the kernel instantiations.
#include <cuda_runtime.h>

#include <cstdlib>

#include <algorithm>

#include "dispatch.h"
#include "dm.cuh"
#include "dm_fact.cuh"

namespace mbqc {

constexpr int kDmMaxWindow = kDmFactSmemMaxWindow;  // shared-memory kernels
constexpr int kDmFullMaxWindow = 7;                  // full-matrix kernel

// Factored kernel (dm_fact.cuh) unless MBQC_DM_FACT=0 in the environment.
static bool dm_fact_enabled() {
  static int on = -1;
  if (on < 0) {
    const char *e = getenv("MBQC_DM_FACT");
    on = (e && e[0] == '0') ? 0 : 1;
  }
  return on != 0;
}

template <int W>
static int launch_dm_fact(const DmArgs &a, int64_t batch, cudaStream_t s) {
  constexpr int TPR = DmFactCfg<W>::TPR, G = 256 / TPR;
  const size_t smem = (size_t)G * dm_fact_slice_bytes<W>(a.maxm);
  if (smem > (size_t)227 * 1024)
    return fail(MBQC_E_UNSUPPORTED, "dm_forward: %d steps need %zu bytes of shared memory", a.maxm, smem);
  auto k = dm_fwd_fact<W, TPR>;
  int rc = cuda_check(cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem),
                      "dm smem attribute");
  if (!rc)  // the largest shared-memory carveout: several blocks of runs per SM
    rc = cuda_check(cudaFuncSetAttribute(k, cudaFuncAttributePreferredSharedMemoryCarveout,
                                         (int)cudaSharedmemCarveoutMaxShared),
                    "dm carveout attribute");
  if (rc) return rc;
  const int64_t blocks = (batch + G - 1) / G;
  if (blocks > 0x7fffffff) return fail(MBQC_E_INVALID, "dm_forward: batch too large");
  k<<<(int)blocks, 256, smem, s>>>(a);
  return check_launch("dm_fwd_fact");
}

// Windows 9..11: R in the workspace, one 1024-thread block per resident run.
static int64_t dm_ws_slots(int64_t batch) { return std::min<int64_t>(batch, (int64_t)sm_count()); }

template <int W>
static int launch_dm_fact_ws(const DmArgs &a, int64_t batch, void *ws, size_t ws_bytes, cudaStream_t s) {
  const size_t per = (size_t)DmFactCfg<W>::N * sizeof(float2);
  const int64_t slots = std::min<int64_t>(dm_ws_slots(batch), (int64_t)(ws_bytes / per));
  if (!ws || slots < 1)
    return fail(MBQC_E_INVALID, "dm_forward: window %d needs a workspace of at least %zu bytes", W, per);
  const size_t smem = dm_fact_slice_bytes<W>(a.maxm);
  if (smem > (size_t)227 * 1024)
    return fail(MBQC_E_UNSUPPORTED, "dm_forward: %d steps need %zu bytes of shared memory", a.maxm, smem);
  auto k = dm_fwd_fact_ws<W>;
  int rc = cuda_check(cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem),
                      "dm smem attribute");
  if (rc) return rc;
  k<<<(int)slots, 1024, smem, s>>>(a, static_cast<float2 *>(ws));
  return check_launch("dm_fwd_fact_ws");
}

template <int W>
static int launch_dm(const DmArgs &a, int64_t batch, cudaStream_t s) {
  using Cfg = DmCfg<W>;
  const size_t smem = dm_smem_bytes<W>(a.maxm);
  if (smem > (size_t)227 * 1024)
    return fail(MBQC_E_UNSUPPORTED, "dm_forward: %d steps need %zu bytes of shared memory", a.maxm, smem);
  auto k = dm_fwd_smem<W>;
  int rc = cuda_check(cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem),
                      "dm smem attribute");
  if (rc) return rc;
  const int64_t blocks = (batch + Cfg::GROUPS - 1) / Cfg::GROUPS;
  if (blocks > 0x7fffffff) return fail(MBQC_E_INVALID, "dm_forward: batch too large");
  k<<<(int)blocks, 256, smem, s>>>(a);
  return check_launch("dm_fwd_smem");
}

static int dm_dispatch(int w, bool fact, const DmArgs &a, int64_t batch, void *ws, size_t ws_bytes,
                       cudaStream_t s) {
  if (w > kDmMaxWindow) {
    if (!fact)
      return fail(MBQC_E_UNSUPPORTED, "dm_forward: window %d needs plans whose last step shrinks the window", w);
    switch (w) {
      case 9: return launch_dm_fact_ws<9>(a, batch, ws, ws_bytes, s);
      case 10: return launch_dm_fact_ws<10>(a, batch, ws, ws_bytes, s);
      case 11: return launch_dm_fact_ws<11>(a, batch, ws, ws_bytes, s);
      default: return fail(MBQC_E_UNSUPPORTED, "dm_forward: window %d > %d", w, kDmFactMaxWindow);
    }
  }
  if (fact) {
    switch (w) {
      case 2: return launch_dm_fact<2>(a, batch, s);
      case 3: return launch_dm_fact<3>(a, batch, s);
      case 4: return launch_dm_fact<4>(a, batch, s);
      case 5: return launch_dm_fact<5>(a, batch, s);
      case 6: return launch_dm_fact<6>(a, batch, s);
      case 7: return launch_dm_fact<7>(a, batch, s);
      case 8: return launch_dm_fact<8>(a, batch, s);
      default: break;
    }
  }
  switch (w) {
    case 1: return launch_dm<1>(a, batch, s);
    case 2: return launch_dm<2>(a, batch, s);
    case 3: return launch_dm<3>(a, batch, s);
    case 4: return launch_dm<4>(a, batch, s);
    case 5: return launch_dm<5>(a, batch, s);
    case 6: return launch_dm<6>(a, batch, s);
    case 7: return launch_dm<7>(a, batch, s);
    default:
      return fail(MBQC_E_UNSUPPORTED, "dm_forward: window %d > %d (or, at window 8, a plan whose last step "
                  "does not shrink the window)", w, kDmFullMaxWindow);
  }
}

}  // namespace mbqc

using namespace mbqc;

extern "C" int mbqc_dm_forward(const mbqc_plan *plan, int64_t batch, int32_t window,
                               const int32_t *run_circuit, const double *angles, int64_t angle_stride,
                               const float *psi_in, int64_t in_stride, float *rho_out,
                               int64_t out_stride, double noise, int8_t *outcomes, double *probs,
                               int64_t outcome_stride, int32_t *status, mbqc_stream_t stream) {
  return mbqc_dm_forward_ex(plan, batch, window, run_circuit, angles, angle_stride, psi_in, in_stride,
                            rho_out, out_stride, noise, outcomes, probs, outcome_stride, status, 0u, 0ull,
                            stream);
}

extern "C" int mbqc_dm_forward_ex(const mbqc_plan *plan, int64_t batch, int32_t window,
                                  const int32_t *run_circuit, const double *angles, int64_t angle_stride,
                                  const float *psi_in, int64_t in_stride, float *rho_out,
                                  int64_t out_stride, double noise, int8_t *outcomes, double *probs,
                                  int64_t outcome_stride, int32_t *status, uint32_t flags, uint64_t seed,
                                  mbqc_stream_t stream) {
  return mbqc_dm_forward_ws(plan, batch, window, run_circuit, angles, angle_stride, psi_in, in_stride, rho_out,
                            out_stride, noise, outcomes, probs, outcome_stride, status, flags, seed, nullptr, 0,
                            stream);
}

extern "C" int mbqc_dm_forward_workspace(const mbqc_plan *plan, int64_t batch, int32_t window, size_t *bytes) {
  if (!plan || !bytes) return fail(MBQC_E_INVALID, "dm_forward_workspace: null argument");
  if (batch < 0) return fail(MBQC_E_INVALID, "dm_forward_workspace: negative batch");
  *bytes = 0;
  if (window > kDmMaxWindow && window <= kDmFactMaxWindow)
    *bytes = (size_t)dm_ws_slots(batch) * ((size_t)1 << (2 * (window - 1))) * sizeof(float2);
  return MBQC_OK;
}

extern "C" int mbqc_dm_forward_ws(const mbqc_plan *plan, int64_t batch, int32_t window,
                                  const int32_t *run_circuit, const double *angles, int64_t angle_stride,
                                  const float *psi_in, int64_t in_stride, float *rho_out,
                                  int64_t out_stride, double noise, int8_t *outcomes, double *probs,
                                  int64_t outcome_stride, int32_t *status, uint32_t flags, uint64_t seed,
                                  void *workspace, size_t workspace_bytes, mbqc_stream_t stream) {
  if (!plan) return fail(MBQC_E_INVALID, "dm_forward: null plan");
  if (batch < 0) return fail(MBQC_E_INVALID, "dm_forward: negative batch");
  if (batch == 0) return MBQC_OK;
  if (!psi_in || !rho_out) return fail(MBQC_E_INVALID, "dm_forward: null buffer");
  if (!(noise >= 0.0 && noise <= 1.0)) return fail(MBQC_E_INVALID, "dm_forward: noise %g", noise);
  const PlanView v = view_of(plan);
  int maxm = 1, max_in = 0, max_out = 0, max_a = 0;
  // the factored kernel needs >= 1 step and a last step that shrinks the
  // window (its final slot is then |0>, not an output)
  bool fact = (dm_fact_enabled() || window > kDmMaxWindow) && !(flags & MBQC_F_DM_FULL_MATRIX) && window >= 2 &&
              window <= kDmFactMaxWindow;
  for (int c = 0; c < v.n_circuits; ++c) {
    const DevCircuit &hc = host_circuit(plan, c);
    if (run_circuit == nullptr && c > 0) break;
    if (hc.w != window) {
      if (run_circuit == nullptr)
        return fail(MBQC_E_INVALID, "dm_forward: circuit 0 has window %d, not %d", hc.w, window);
      continue;
    }
    if (hc.n_steps < 1 || !(host_steps(plan, c)[hc.n_steps - 1].mask & kDead)) fact = false;
    maxm = std::max(maxm, hc.n_steps);
    max_in = std::max(max_in, hc.n_in);
    max_out = std::max(max_out, hc.n_out);
    max_a = std::max(max_a, hc.n_angles);
  }
  if (max_a > 0 && (!angles || angle_stride < max_a))
    return fail(MBQC_E_INVALID, "dm_forward: angle stride %lld < %d", (long long)angle_stride, max_a);
  if (in_stride != 0 && in_stride < ((int64_t)1 << max_in))
    return fail(MBQC_E_INVALID, "dm_forward: input stride too small");
  if (out_stride < ((int64_t)1 << (2 * max_out)))
    return fail(MBQC_E_INVALID, "dm_forward: output stride too small");
  if ((outcomes || probs) && outcome_stride < maxm)
    return fail(MBQC_E_INVALID, "dm_forward: outcome stride too small");
  DmArgs a{};
  a.circ = v.d_circ;
  a.steps = v.d_steps;
  a.maps = v.d_map;
  a.run_circuit = run_circuit;
  a.B = batch;
  a.angles = angles;
  a.astride = angle_stride;
  a.psi_in = reinterpret_cast<const float2 *>(psi_in);
  a.istride = in_stride;
  a.rho_out = reinterpret_cast<float2 *>(rho_out);
  a.out_stride = out_stride;
  a.noise = noise;
  a.outcomes = outcomes;
  a.ostride = outcome_stride;
  a.probs = probs;
  a.status = status;
  a.maxm = maxm;
  a.flags = flags;
  a.seed = seed;
  return dm_dispatch(window, fact, a, batch, workspace, workspace_bytes, (cudaStream_t)stream);
}
