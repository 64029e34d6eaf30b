// Adjoint entry points of the C ABI: workspace sizing, generic adjoint (for
// autograd), fused fidelity-loss gradient.
#include <cuda_runtime.h>

#include "dispatch.h"
#include "sv_adj.cuh"

namespace mbqc {

typedef int (*adj_launcher)(const SvAdjArgs &, const AdjLaunch &, cudaStream_t);

static adj_launcher pick_adj(int w, bool f64) {
#define MBQC_CASE(W) \
  case W:            \
    return f64 ? launch_sv_adj_f64_w##W : launch_sv_adj_f32_w##W;
  switch (w) {
    MBQC_CASE(1)
    MBQC_CASE(2)
    MBQC_CASE(3)
    MBQC_CASE(4)
    MBQC_CASE(5)
    MBQC_CASE(6)
    MBQC_CASE(7)
    MBQC_CASE(8)
    default:
      return nullptr;
  }
#undef MBQC_CASE
}

struct AdjGeometry {
  int blocks, threads, rpw, periods;
  size_t smem;
  int64_t slots;
  size_t ws_bytes;
  bool wide, gen;
  WideAdjGeom wg;
};

// Windows 9..20: one block per run slot (a cluster of 2 or 4 blocks for
// windows above 14 when the batch leaves SMs idle); each slot holds the
// pre-step half-state of every step (and the window itself above w = 14), and
// the slot count is capped by the blocks resident on the GPU and by
// kWideAdjMaxWorkspace.
static int adj_geometry_wide(const DevCircuit &hc, int64_t runs, bool f64, AdjGeometry &g) {
  g.gen = !hc.sv_planes_ok;
  if (f64)
    return g.gen ? fail(MBQC_E_UNSUPPORTED, "FP64 adjoint: XY, X and Y steps only")
                 : fail(MBQC_E_UNSUPPORTED, "FP64 adjoint: window %d > %d", hc.w, kAdjMaxWindow);
  if (hc.w > kWideAdjMaxWindow)
    return fail(MBQC_E_UNSUPPORTED, "adjoint: window %d > %d", hc.w, kWideAdjMaxWindow);
  g.wide = true;
  g.rpw = 1;
  g.periods = 0;
  g.threads = wide_adj_threads(hc.w);
  g.smem = wide_adj_smem(hc.w, hc.n_steps, g.gen);
  int dev = 0, optin = 0;
  int rc = cuda_check(cudaGetDevice(&dev), "cudaGetDevice");
  if (!rc) rc = cuda_check(cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev), "smem");
  if (rc) return rc;
  if (g.smem > (size_t)optin)
    return fail(MBQC_E_UNSUPPORTED, "adjoint: window %d with %d steps needs %zu bytes of shared memory", hc.w,
                hc.n_steps, g.smem);
  int occ = 0;
  AdjLaunch q{0, g.threads, g.smem, true, &occ};
  SvAdjArgs dummy{};
  dummy.W = hc.w;
  g.wg.cluster = 1;
  rc = launch_sv_adj_wide(dummy, g.wg, q, nullptr, g.gen);
  if (rc) return rc;
  if (occ < 1) return fail(MBQC_E_UNSUPPORTED, "adjoint: kernel does not fit on an SM");
  const int64_t D = (int64_t)1 << hc.w;
  const int64_t slot = (hc.w > 14 ? D : 0) + (int64_t)hc.n_steps * (g.gen ? D : D / 2);
  // a batch smaller than the GPU: runs of a window in the workspace are
  // shared by a cluster of 2 or 4 blocks (one block per SM), so that more SMs
  // work on them; blocks below counts run slots (clusters)
  g.wg.cluster = 1;
  if (!g.gen && hc.w > 14) {
    const int64_t sms = sm_count();
    if (runs * 4 <= sms)
      g.wg.cluster = 4;
    else if (runs * 2 <= sms)
      g.wg.cluster = 2;
  }
  int64_t blocks = g.wg.cluster > 1 ? (int64_t)sm_count() / g.wg.cluster : (int64_t)sm_count() * occ;
  if (runs < blocks) blocks = runs;
  const int64_t cap = (int64_t)(kWideAdjMaxWorkspace / ((size_t)slot * 8));
  if (blocks > cap) blocks = cap;
  if (blocks < 1) blocks = 1;
  g.blocks = (int)blocks;
  g.slots = blocks;
  g.ws_bytes = (size_t)blocks * (size_t)slot * 8;
  for (int i = 0; i < 32; ++i) {
    g.wg.in_bits[i] = hc.in_bits[i];
    g.wg.out_bits[i] = hc.out_bits[i];
    g.wg.init_cz[i] = hc.init_cz[i];
  }
  g.wg.out_mask = hc.out_mask;
  g.wg.slot_elems = slot;
  return MBQC_OK;
}

// Persistent grid: as many blocks as fit on the GPU (or as the batch needs);
// the checkpoint workspace is sized by in-flight slots, not by the batch.
static int adj_geometry(const DevCircuit &hc, int64_t runs, bool f64, AdjGeometry &g) {
  g.wide = false;
  g.gen = false;
  if (!hc.sv_planes_ok && !hc.sv_xz_ok)
    return fail(MBQC_E_UNSUPPORTED, "adjoint: statevector steps in XY, X, Y, XZ or YZ only");
  if (hc.w > kAdjMaxWindow || !hc.sv_planes_ok) return adj_geometry_wide(hc, runs, f64, g);
  adj_launcher fn = pick_adj(hc.w, f64);
  if (!fn) return fail(MBQC_E_UNSUPPORTED, "adjoint: window %d", hc.w);
  const int ll = adj_ll(hc.w, f64);
  const size_t cb = f64 ? 16 : 8, gb = f64 ? 8 : 4;
  g.rpw = 32 >> ll;
  const size_t per_warp = AdjSmem::bytes_per_warp(hc.n_steps, hc.n_angles, g.rpw, cb, gb);
  int wpb = 4;
  while (wpb > 1 && per_warp * wpb > (size_t)200 * 1024) wpb >>= 1;
  if (per_warp * wpb > (size_t)220 * 1024)
    return fail(MBQC_E_UNSUPPORTED, "adjoint: %d steps x %d angles exceed shared memory",
                hc.n_steps, hc.n_angles);
  g.threads = 32 * wpb;
  g.smem = per_warp * wpb;
  int occ = 0;
  AdjLaunch q{0, g.threads, g.smem, true, &occ};
  SvAdjArgs dummy{};
  int rc = fn(dummy, q, nullptr);
  if (rc) return rc;
  if (occ < 1) return fail(MBQC_E_UNSUPPORTED, "adjoint: kernel does not fit on an SM");
  const int64_t need = (runs + (int64_t)g.rpw * wpb - 1) / ((int64_t)g.rpw * wpb);
  int64_t blocks = (int64_t)sm_count() * occ;
  if (need < blocks) blocks = need;
  if (blocks < 1) blocks = 1;
  g.blocks = (int)blocks;
  g.slots = blocks * wpb * g.rpw;
  g.periods = (hc.n_steps + hc.w - 1) / hc.w;
  g.ws_bytes = (size_t)g.slots * g.periods * ((size_t)1 << hc.w) * cb;
  return MBQC_OK;
}

static int adj_common(const mbqc_plan *plan, int64_t runs, int64_t J, const double *angles,
                      int64_t astride, const void *psi_in, int64_t istride, const void *grad_out,
                      const void *targets, double *loss, double *grad, int32_t *status, void *ws,
                      size_t ws_bytes, cudaStream_t stream, bool f64) {
  if (!plan) return fail(MBQC_E_INVALID, "adjoint: null plan");
  if (runs < 0) return fail(MBQC_E_INVALID, "adjoint: negative batch");
  const DevCircuit &hc = host_circuit(plan, 0);
  if (runs == 0) return MBQC_OK;
  if (!psi_in || !grad) return fail(MBQC_E_INVALID, "adjoint: null buffer");
  if (hc.n_angles > 0 && (!angles || astride < hc.n_angles))
    return fail(MBQC_E_INVALID, "adjoint: bad angle array");
  AdjGeometry g;
  int rc = adj_geometry(hc, runs, f64, g);
  if (rc) return rc;
  if (!g.wide && hc.map_off < 0) return fail(MBQC_E_UNSUPPORTED, "adjoint: window %d has no index map", hc.w);
  if (!ws || ws_bytes < g.ws_bytes)
    return fail(MBQC_E_INVALID, "adjoint: workspace of %zu bytes, %zu needed", ws_bytes, g.ws_bytes);
  const PlanView v = view_of(plan);
  SvAdjArgs a{};
  a.steps = v.d_steps + hc.step_off;
  a.map = hc.map_off >= 0 ? v.d_map + hc.map_off : nullptr;
  a.M = hc.n_steps;
  a.W = hc.w;
  a.n_in = hc.n_in;
  a.n_out = hc.n_out;
  a.n_angles = hc.n_angles;
  a.B = runs;
  a.J = J;
  a.angles = angles;
  a.astride = astride;
  a.psi_in = psi_in;
  a.istride = istride;
  a.grad_out = grad_out;
  a.targets = targets;
  a.loss = loss;
  a.grad = grad;
  a.status = status;
  a.ckpt = ws;
  a.n_slots = g.slots;
  AdjLaunch l{g.blocks, g.threads, g.smem, false, nullptr};
  if (g.wide) return launch_sv_adj_wide(a, g.wg, l, stream, g.gen);
  return pick_adj(hc.w, f64)(a, l, stream);
}

}  // namespace mbqc

using namespace mbqc;

extern "C" {

int mbqc_sv_adjoint_workspace(const mbqc_plan *plan, int64_t batch, int32_t f64, size_t *bytes) {
  if (!plan || !bytes || batch < 0) return fail(MBQC_E_INVALID, "adjoint_workspace: bad arguments");
  *bytes = 0;
  if (batch == 0) return MBQC_OK;
  AdjGeometry g;
  int rc = adj_geometry(host_circuit(plan, 0), batch, f64 != 0, g);
  if (rc) return rc;
  *bytes = g.ws_bytes;
  return MBQC_OK;
}

int mbqc_sv_adjoint(const mbqc_plan *plan, int64_t batch, const double *angles, int64_t angle_stride,
                    const float *psi_in, int64_t in_stride, const float *grad_out, double *grad_angles,
                    int32_t *status, void *workspace, size_t workspace_bytes, mbqc_stream_t stream) {
  if (!grad_out && batch > 0) return fail(MBQC_E_INVALID, "adjoint: null grad_out");
  return adj_common(plan, batch, 0, angles, angle_stride, psi_in, in_stride, grad_out, nullptr,
                    nullptr, grad_angles, status, workspace, workspace_bytes, (cudaStream_t)stream,
                    false);
}

int mbqc_sv_adjoint_f64(const mbqc_plan *plan, int64_t batch, const double *angles,
                        int64_t angle_stride, const double *psi_in, int64_t in_stride,
                        const double *grad_out, double *grad_angles, int32_t *status, void *workspace,
                        size_t workspace_bytes, mbqc_stream_t stream) {
  if (!grad_out && batch > 0) return fail(MBQC_E_INVALID, "adjoint: null grad_out");
  return adj_common(plan, batch, 0, angles, angle_stride, psi_in, in_stride, grad_out, nullptr,
                    nullptr, grad_angles, status, workspace, workspace_bytes, (cudaStream_t)stream,
                    true);
}

int mbqc_sv_fidelity_grad(const mbqc_plan *plan, int64_t n_vectors, const double *angles,
                          int64_t angle_stride, int64_t n_inputs, const float *psi_in,
                          const float *targets, double *loss, double *grad, int32_t *status,
                          void *workspace, size_t workspace_bytes, mbqc_stream_t stream) {
  if (n_vectors < 0 || n_inputs <= 0) return fail(MBQC_E_INVALID, "fidelity_grad: bad sizes");
  if (!targets || !loss || !grad) return fail(MBQC_E_INVALID, "fidelity_grad: null buffer");
  if (!plan) return fail(MBQC_E_INVALID, "fidelity_grad: null plan");
  const DevCircuit &hc = host_circuit(plan, 0);
  cudaStream_t s = (cudaStream_t)stream;
  if (n_vectors == 0) return MBQC_OK;
  int rc = cuda_check(cudaMemsetAsync(loss, 0, sizeof(double) * n_vectors, s), "zero loss");
  if (!rc && hc.n_angles)
    rc = cuda_check(cudaMemsetAsync(grad, 0, sizeof(double) * n_vectors * hc.n_angles, s), "zero grad");
  if (rc) return rc;
  return adj_common(plan, n_vectors * n_inputs, n_inputs, angles, angle_stride, psi_in,
                    (int64_t)1 << hc.n_in, nullptr, targets, loss, grad, status, workspace,
                    workspace_bytes, s, false);
}

}  // extern "C"
