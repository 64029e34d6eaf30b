// Density-matrix adjoint entry points of the C ABI (windows 1..10).
#include <cuda_runtime.h>

#include <algorithm>

#include "dispatch.h"
#include "dm_adj.cuh"

namespace mbqc {

struct DmAdjGeometry {
  int blocks, maxm, max_a, max_out;
  size_t smem, ws_bytes;
  int64_t slots;
};

// Workspace: [slots][maxm][4^w] pre-step matrices, then (windows above
// kDmAdjSmemMaxWindow) [slots][4^w] for the matrix itself.
template <int W>
static int dm_adj_geom(int64_t batch, int maxm, size_t ws_cap, DmAdjGeometry &g) {
  using Cfg = DmCfg<W>;
  using ACfg = DmAdjCfg<W>;
  g.smem = DmAdjSmem<W>::bytes(maxm);
  if (g.smem > (size_t)227 * 1024)
    return fail(MBQC_E_UNSUPPORTED, "dm_adjoint: %d steps need %zu bytes of shared memory", maxm, g.smem);
  auto k = dm_adj_smem<W>;
  int rc = cuda_check(cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)g.smem),
                      "dm adjoint smem attribute");
  if (rc) return rc;
  int occ = 0;
  rc = cuda_check(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k, ACfg::BLOCK, g.smem), "occupancy");
  if (rc) return rc;
  if (occ < 1) return fail(MBQC_E_UNSUPPORTED, "dm_adjoint: kernel does not fit on an SM");
  const size_t per_slot = ((size_t)maxm + (ACfg::kWs ? 1 : 0)) * Cfg::N * sizeof(float2);
  int64_t blocks = std::min<int64_t>((batch + ACfg::GROUPS - 1) / ACfg::GROUPS, (int64_t)sm_count() * occ);
  // bound the workspace; fewer runs in flight if needed
  while (blocks > 1 && (size_t)blocks * ACfg::GROUPS * per_slot > ws_cap) blocks = (blocks + 1) / 2;
  g.blocks = (int)std::max<int64_t>(blocks, 1);
  g.slots = (int64_t)g.blocks * ACfg::GROUPS;
  g.ws_bytes = (size_t)g.slots * per_slot;
  g.maxm = maxm;
  return MBQC_OK;
}

template <int W>
static int dm_adj_launch(DmAdjArgs a, const DmAdjGeometry &g, cudaStream_t s) {
  a.rho_ws = DmAdjCfg<W>::kWs ? a.hist + g.slots * (int64_t)g.maxm * DmCfg<W>::N : nullptr;
  dm_adj_smem<W><<<g.blocks, DmAdjCfg<W>::BLOCK, g.smem, s>>>(a);
  return check_launch("dm_adj_smem");
}

static int dm_adj_geometry(int w, int64_t batch, int maxm, DmAdjGeometry &g) {
  // pre-step history: 2 GiB at most in shared-memory windows, 16 GiB above
  const size_t cap = w > kDmAdjSmemMaxWindow ? (size_t)16 << 30 : (size_t)2 << 30;
  switch (w) {
    case 1: return dm_adj_geom<1>(batch, maxm, cap, g);
    case 2: return dm_adj_geom<2>(batch, maxm, cap, g);
    case 3: return dm_adj_geom<3>(batch, maxm, cap, g);
    case 4: return dm_adj_geom<4>(batch, maxm, cap, g);
    case 5: return dm_adj_geom<5>(batch, maxm, cap, g);
    case 6: return dm_adj_geom<6>(batch, maxm, cap, g);
    case 7: return dm_adj_geom<7>(batch, maxm, cap, g);
    case 8: return dm_adj_geom<8>(batch, maxm, cap, g);
    case 9: return dm_adj_geom<9>(batch, maxm, cap, g);
    case 10: return dm_adj_geom<10>(batch, maxm, cap, g);
    default: return fail(MBQC_E_UNSUPPORTED, "dm_adjoint: window %d > %d", w, kDmAdjMaxWindow);
  }
}

static int plan_extents(const mbqc_plan *plan, int window, const int32_t *run_circuit, int &maxm, int &max_in,
                        int &max_out, int &max_a) {
  const PlanView v = view_of(plan);
  maxm = 1;
  max_in = max_out = max_a = 0;
  for (int c = 0; c < v.n_circuits; ++c) {
    const DevCircuit &hc = host_circuit(plan, c);
    if (run_circuit == nullptr && c > 0) break;
    if (hc.w != window) {
      if (run_circuit == nullptr)
        return fail(MBQC_E_INVALID, "dm_adjoint: circuit 0 has window %d, not %d", hc.w, window);
      continue;
    }
    if (hc.has_z)
      return fail(MBQC_E_UNSUPPORTED, "dm_adjoint: circuit %d measures in the Z basis (drawn or unprojected "
                  "outcomes have no adjoint here)", c);
    maxm = std::max(maxm, hc.n_steps);
    max_in = std::max(max_in, hc.n_in);
    max_out = std::max(max_out, hc.n_out);
    max_a = std::max(max_a, hc.n_angles);
  }
  return MBQC_OK;
}

}  // namespace mbqc

using namespace mbqc;

extern "C" {

int mbqc_dm_adjoint_workspace(const mbqc_plan *plan, int64_t batch, int32_t window,
                              const int32_t *run_circuit, size_t *bytes) {
  if (!plan || !bytes || batch < 0) return fail(MBQC_E_INVALID, "dm_adjoint_workspace: bad arguments");
  *bytes = 0;
  if (batch == 0) return MBQC_OK;
  int maxm, mi, mo, ma;
  int rc = plan_extents(plan, window, run_circuit, maxm, mi, mo, ma);
  if (rc) return rc;
  DmAdjGeometry g;
  rc = dm_adj_geometry(window, batch, maxm, g);
  if (rc) return rc;
  *bytes = g.ws_bytes;
  return MBQC_OK;
}

int mbqc_dm_adjoint(const mbqc_plan *plan, int64_t batch, int32_t window, const int32_t *run_circuit,
                    const double *angles, int64_t angle_stride, const float *psi_in, int64_t in_stride,
                    double noise, const float *grad_out, int64_t gout_stride, float *rho_out,
                    int64_t out_stride, double *grad_angles, int64_t grad_stride, int8_t *outcomes,
                    int64_t outcome_stride, int32_t *status, void *workspace, size_t workspace_bytes,
                    mbqc_stream_t stream) {
  if (!plan) return fail(MBQC_E_INVALID, "dm_adjoint: null plan");
  if (batch < 0) return fail(MBQC_E_INVALID, "dm_adjoint: negative batch");
  if (batch == 0) return MBQC_OK;
  if (!psi_in || !grad_out || !grad_angles) return fail(MBQC_E_INVALID, "dm_adjoint: null buffer");
  if (!(noise >= 0.0 && noise <= 1.0)) return fail(MBQC_E_INVALID, "dm_adjoint: noise %g", noise);
  int maxm, max_in, max_out, max_a;
  int rc = plan_extents(plan, window, run_circuit, maxm, max_in, max_out, max_a);
  if (rc) return rc;
  if (max_a > 0 && (!angles || angle_stride < max_a || grad_stride < max_a))
    return fail(MBQC_E_INVALID, "dm_adjoint: angle/gradient stride < %d", max_a);
  if (in_stride != 0 && in_stride < ((int64_t)1 << max_in))
    return fail(MBQC_E_INVALID, "dm_adjoint: input stride too small");
  if (gout_stride < ((int64_t)1 << (2 * max_out)) || (rho_out && out_stride < ((int64_t)1 << (2 * max_out))))
    return fail(MBQC_E_INVALID, "dm_adjoint: output stride too small");
  if (outcomes && outcome_stride < maxm) return fail(MBQC_E_INVALID, "dm_adjoint: outcome stride too small");
  DmAdjGeometry g;
  rc = dm_adj_geometry(window, batch, maxm, g);
  if (rc) return rc;
  if (!workspace || workspace_bytes < g.ws_bytes)
    return fail(MBQC_E_INVALID, "dm_adjoint: workspace of %zu bytes, %zu needed", workspace_bytes, g.ws_bytes);
  const PlanView v = view_of(plan);
  DmAdjArgs a{};
  a.f.circ = v.d_circ;
  a.f.steps = v.d_steps;
  a.f.maps = v.d_map;
  a.f.run_circuit = run_circuit;
  a.f.B = batch;
  a.f.angles = angles;
  a.f.astride = angle_stride;
  a.f.psi_in = reinterpret_cast<const float2 *>(psi_in);
  a.f.istride = in_stride;
  a.f.rho_out = reinterpret_cast<float2 *>(rho_out);
  a.f.out_stride = out_stride;
  a.f.noise = noise;
  a.f.outcomes = outcomes;
  a.f.ostride = outcome_stride;
  a.f.probs = nullptr;
  a.f.status = status;
  a.f.maxm = maxm;
  a.grad_out = reinterpret_cast<const float2 *>(grad_out);
  a.gout_stride = gout_stride;
  a.grad = grad_angles;
  a.grad_stride = grad_stride;
  a.hist = reinterpret_cast<float2 *>(workspace);
  a.n_slots = g.slots;
  cudaStream_t s = (cudaStream_t)stream;
  switch (window) {
    case 1: return dm_adj_launch<1>(a, g, s);
    case 2: return dm_adj_launch<2>(a, g, s);
    case 3: return dm_adj_launch<3>(a, g, s);
    case 4: return dm_adj_launch<4>(a, g, s);
    case 5: return dm_adj_launch<5>(a, g, s);
    case 6: return dm_adj_launch<6>(a, g, s);
    case 7: return dm_adj_launch<7>(a, g, s);
    case 8: return dm_adj_launch<8>(a, g, s);
    case 9: return dm_adj_launch<9>(a, g, s);
    case 10: return dm_adj_launch<10>(a, g, s);
    default: return fail(MBQC_E_UNSUPPORTED, "dm_adjoint: window %d > %d", window, kDmAdjMaxWindow);
  }
}

}  // extern "C"
