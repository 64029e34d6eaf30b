// Allocation-free variant of the statevector adjoint.
//
// mbqc_sv_adjoint needs a caller-provided device workspace for its period
// checkpoints.  Some callers cannot make that allocation: plugins running
// inside a host framework that owns the GPU memory pool and forbids outside
// cudaMalloc calls, fixed-footprint services that must not grow device memory
// after start-up, and latency-bound loops that cannot afford cudaFree's
// device-wide synchronisation.  This entry point takes only the inputs and
// outputs; its scratch is the fixed array below, part of the library image.
#include <cuda_runtime.h>

#include <mutex>

#include "dispatch.h"
#include "sv_adj.cuh"

namespace mbqc {

// Checkpoint scratch of the allocation-free adjoint: MBQC_NOALLOC_SCRATCH_BYTES
// (16 MiB), held on every GPU that loads the library until the process exits.
static __device__ __align__(256) unsigned char g_noalloc_scratch[MBQC_NOALLOC_SCRATCH_BYTES];

constexpr int kNoAllocMaxDevices = 64;

// Cached device address of the array, per device and per CUDA context: a
// device reset (cudaDeviceReset) or a re-created primary context loads the
// library's module again, possibly at another address, so the cache entry is
// keyed by the context's process-unique id and looked up again when it
// changes.
struct NoallocAddr {
  unsigned long long ctx_id;  // 0 = empty
  void *addr;
};
static NoallocAddr g_noalloc_addr[kNoAllocMaxDevices];
static std::mutex g_noalloc_mu;

// Driver entry points for the current context's id, resolved once through the
// runtime (no link-time dependency on libcuda).
typedef int (*ctx_get_current_fn)(void **ctx);
typedef int (*ctx_get_id_fn)(void *ctx, unsigned long long *id);

static unsigned long long current_ctx_id() {
  static ctx_get_current_fn get_cur = nullptr;
  static ctx_get_id_fn get_id = nullptr;
  static std::once_flag once;
  std::call_once(once, [] {
    void *f = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      get_cur = (ctx_get_current_fn)f;
    f = nullptr;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetId", &f, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      get_id = (ctx_get_id_fn)f;
  });
  if (!get_cur || !get_id) return 0;
  void *ctx = nullptr;
  if (get_cur(&ctx) != 0 || !ctx) return 0;
  unsigned long long id = 0;
  if (get_id(ctx, &id) != 0) return 0;
  return id;
}

// Device address of the scratch array on the current device.  The array's
// name is only a host-side stand-in, so the address is looked up with the
// device current (cudaGetSymbolAddress) on the first call in each context
// and cached; without a context id (driver entry points unavailable) it is
// looked up on every call.
static int noalloc_scratch(void **out) {
  int dev = 0;
  int rc = cuda_check(cudaGetDevice(&dev), "cudaGetDevice");
  if (rc) return rc;
  if (dev < 0 || dev >= kNoAllocMaxDevices)
    return fail(MBQC_E_UNSUPPORTED, "adjoint_noalloc: device %d beyond %d", dev, kNoAllocMaxDevices);
  std::lock_guard<std::mutex> lock(g_noalloc_mu);
  const unsigned long long id = current_ctx_id();
  if (id != 0 && g_noalloc_addr[dev].ctx_id == id) {
    *out = g_noalloc_addr[dev].addr;
    return MBQC_OK;
  }
  void *p = nullptr;
  rc = cuda_check(cudaGetSymbolAddress(&p, g_noalloc_scratch), "cudaGetSymbolAddress(scratch)");
  if (rc) return rc;
  // the lookup makes the device's context current if it was not yet
  g_noalloc_addr[dev] = NoallocAddr{id != 0 ? id : current_ctx_id(), p};
  *out = p;
  return MBQC_OK;
}

typedef int (*noalloc_launcher)(const SvAdjArgs &, const AdjLaunch &, cudaStream_t);

static noalloc_launcher noalloc_pick(int w) {
  switch (w) {
    case 1: return launch_sv_adj_f32_w1;
    case 2: return launch_sv_adj_f32_w2;
    case 3: return launch_sv_adj_f32_w3;
    case 4: return launch_sv_adj_f32_w4;
    case 5: return launch_sv_adj_f32_w5;
    case 6: return launch_sv_adj_f32_w6;
    case 7: return launch_sv_adj_f32_w7;
    case 8: return launch_sv_adj_f32_w8;
    default: return nullptr;
  }
}

}  // namespace mbqc

using namespace mbqc;

extern "C" int mbqc_sv_adjoint_noalloc(const mbqc_plan *plan, int64_t batch, const double *angles,
                                       int64_t angle_stride, const float *psi_in, int64_t in_stride,
                                       const float *grad_out, double *grad_angles, int32_t *status,
                                       mbqc_stream_t stream) {
  if (!plan) return fail(MBQC_E_INVALID, "adjoint_noalloc: null plan");
  if (batch < 0) return fail(MBQC_E_INVALID, "adjoint_noalloc: negative batch");
  if (batch == 0) return MBQC_OK;
  const DevCircuit &hc = host_circuit(plan, 0);
  if (!psi_in || !grad_out || !grad_angles) return fail(MBQC_E_INVALID, "adjoint_noalloc: null buffer");
  if (!hc.sv_planes_ok) return fail(MBQC_E_UNSUPPORTED, "adjoint_noalloc: statevector steps in XY, X or Y only");
  if (hc.n_angles > 0 && (!angles || angle_stride < hc.n_angles))
    return fail(MBQC_E_INVALID, "adjoint_noalloc: bad angle array");
  if (hc.map_off < 0 || hc.w > kAdjMaxWindow)
    return fail(MBQC_E_UNSUPPORTED, "adjoint_noalloc: window %d > %d", hc.w, kAdjMaxWindow);
  noalloc_launcher fn = noalloc_pick(hc.w);
  if (!fn) return fail(MBQC_E_UNSUPPORTED, "adjoint_noalloc: window %d", hc.w);

  // launch geometry: the checkpoints of every run in flight must fit the array
  const int ll = adj_ll(hc.w, false);
  const int rpw = 32 >> ll;
  const size_t per_warp = AdjSmem::bytes_per_warp(hc.n_steps, hc.n_angles, rpw, 8, 4);
  int wpb = 4;
  while (wpb > 1 && per_warp * wpb > (size_t)200 * 1024) wpb >>= 1;
  if (per_warp * wpb > (size_t)220 * 1024)
    return fail(MBQC_E_UNSUPPORTED, "adjoint_noalloc: %d steps x %d angles exceed shared memory",
                hc.n_steps, hc.n_angles);
  // Shared memory binds first: a circuit whose step tables fit needs at most
  // ~2.9 MB of checkpoints per warp of runs (window 8: <= 11,264 steps, one
  // run per warp), so the array only limits how many runs are in flight; the
  // size check below is a defensive guard.
  const int periods = (hc.n_steps + hc.w - 1) / hc.w;
  const size_t slot_bytes = (size_t)periods * ((size_t)1 << hc.w) * sizeof(float2);
  while (wpb > 1 && slot_bytes * rpw * wpb > (size_t)MBQC_NOALLOC_SCRATCH_BYTES) wpb >>= 1;
  const size_t block_bytes = slot_bytes * rpw * wpb;
  if (block_bytes > (size_t)MBQC_NOALLOC_SCRATCH_BYTES)
    return fail(MBQC_E_UNSUPPORTED,
                "adjoint_noalloc: one warp of runs needs %zu bytes of checkpoints (%d periods of "
                "2^%d amplitudes x %d runs), more than the fixed %zu-byte scratch; use "
                "mbqc_sv_adjoint with a workspace",
                block_bytes, periods, hc.w, rpw, (size_t)MBQC_NOALLOC_SCRATCH_BYTES);
  const int threads = 32 * wpb;
  const size_t smem = per_warp * wpb;
  int occ = 0;
  AdjLaunch q{0, threads, smem, true, &occ};
  SvAdjArgs none{};
  int rc = fn(none, q, nullptr);
  if (rc) return rc;
  if (occ < 1) return fail(MBQC_E_UNSUPPORTED, "adjoint_noalloc: kernel does not fit on an SM");
  const int64_t need = (batch + (int64_t)rpw * wpb - 1) / ((int64_t)rpw * wpb);
  int64_t blocks = (int64_t)sm_count() * occ;
  const int64_t cap = (int64_t)((size_t)MBQC_NOALLOC_SCRATCH_BYTES / block_bytes);
  if (cap < blocks) blocks = cap;
  if (need < blocks) blocks = need;
  if (blocks < 1) blocks = 1;

  void *scratch = nullptr;
  rc = noalloc_scratch(&scratch);
  if (rc) return rc;

  const PlanView v = view_of(plan);
  SvAdjArgs a{};
  a.steps = v.d_steps + hc.step_off;
  a.map = v.d_map + hc.map_off;
  a.M = hc.n_steps;
  a.W = hc.w;
  a.n_in = hc.n_in;
  a.n_out = hc.n_out;
  a.n_angles = hc.n_angles;
  a.B = batch;
  a.J = 0;
  a.angles = angles;
  a.astride = angle_stride;
  a.psi_in = psi_in;
  a.istride = in_stride;
  a.grad_out = grad_out;
  a.grad = grad_angles;
  a.status = status;
  a.ckpt = scratch;
  a.n_slots = blocks * wpb * rpw;
  AdjLaunch l{(int)blocks, threads, smem, false, nullptr};
  return fn(a, l, (cudaStream_t)stream);
}
