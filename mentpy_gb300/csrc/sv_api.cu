// Statevector entry points of the C ABI and small auxiliary kernels.
#include <cuda_runtime.h>

#include <new>

#include "dispatch.h"
#include "sv_reg.cuh"

namespace mbqc {

static int sm_count_cached() { return sm_count(); }

// Default log2(lanes per run): the fewest lanes (most work per thread, fewest
// shuffles) that still give every SM a few warps.
static int default_ll(int w, int64_t batch) {
  const int lo = w - 5 > 0 ? w - 5 : 0;
  const int hi = w < 5 ? w : 5;
  const int64_t want_threads = (int64_t)sm_count_cached() * 32 * 8;
  for (int ll = lo; ll <= hi; ++ll)
    if (batch * ((int64_t)1 << ll) >= want_threads) return ll;
  return hi;
}

typedef int (*sv_launcher)(int, const SvArgs &, int, int, cudaStream_t);
typedef int (*sv_gen_launcher)(const SvArgs &, int, int, cudaStream_t);

static sv_gen_launcher pick_gen(int w, bool f64) {
#define MBQC_CASE(W) \
  case W:            \
    return f64 ? launch_sv_reg_gen_f64_w##W : launch_sv_reg_gen_f32_w##W;
  switch (w) {
    MBQC_CASE(1)
    MBQC_CASE(2)
    MBQC_CASE(3)
    MBQC_CASE(4)
    MBQC_CASE(5)
    MBQC_CASE(6)
    MBQC_CASE(7)
    MBQC_CASE(8)
    MBQC_CASE(9)
    MBQC_CASE(10)
    default:
      return nullptr;
  }
#undef MBQC_CASE
}

static sv_launcher pick(int w, bool f64) {
#define MBQC_CASE(W) \
  case W:            \
    return f64 ? launch_sv_reg_f64_w##W : launch_sv_reg_f32_w##W;
  switch (w) {
    MBQC_CASE(1)
    MBQC_CASE(2)
    MBQC_CASE(3)
    MBQC_CASE(4)
    MBQC_CASE(5)
    MBQC_CASE(6)
    MBQC_CASE(7)
    MBQC_CASE(8)
    MBQC_CASE(9)
    MBQC_CASE(10)
    default:
      return nullptr;
  }
#undef MBQC_CASE
}

}  // namespace mbqc

// A statevector batch with its checks done, its kernel parameter block built
// and its kernel and launch geometry chosen: launching it is one kernel launch.
struct mbqc_sv_call {
  mbqc::SvArgs a;
  int ll, blocks, threads;
  mbqc::sv_launcher fn;
  mbqc::sv_gen_launcher gfn;
  bool empty;
};

namespace mbqc {

static int sv_exec(const mbqc_sv_call &c, cudaStream_t stream) {
  if (c.empty) return MBQC_OK;
  if (c.gfn) return c.gfn(c.a, c.blocks, c.threads, stream);
  return c.fn(c.ll, c.a, c.blocks, c.threads, stream);
}

static int sv_build(const mbqc_plan *plan, int64_t batch, const double *angles, int64_t astride,
                    const void *psi_in, int64_t istride, void *psi_out, uint32_t flags, int variant,
                    double *logprob, int32_t *status, bool f64, mbqc_sv_call &c) {
  c.empty = true;
  c.fn = nullptr;
  c.gfn = nullptr;
  if (!plan) return fail(MBQC_E_INVALID, "sv_forward: null plan");
  if (batch < 0) return fail(MBQC_E_INVALID, "sv_forward: negative batch");
  if (batch == 0) return MBQC_OK;
  const DevCircuit &hc = host_circuit(plan, 0);
  if (!psi_in || !psi_out) return fail(MBQC_E_INVALID, "sv_forward: null state buffer");
  if (hc.n_angles > 0 && !angles) return fail(MBQC_E_INVALID, "sv_forward: null angles");
  if (hc.n_angles > 0 && astride < hc.n_angles)
    return fail(MBQC_E_INVALID, "sv_forward: angle stride %lld < %d angles", (long long)astride,
                hc.n_angles);
  if (istride != 0 && istride < ((int64_t)1 << hc.n_in))
    return fail(MBQC_E_INVALID, "sv_forward: input stride too small");
  const bool gen = !hc.sv_planes_ok;  // XZ / YZ steps
  if (gen && !hc.sv_xz_ok)
    return fail(MBQC_E_UNSUPPORTED, "sv_forward: the statevector kernels measure in the XY, X, Y, XZ and YZ planes");
  if (hc.w > kSvRegMaxWindow)
    return fail(MBQC_E_UNSUPPORTED, "sv_forward: window %d needs the streamed kernel", hc.w);
  const PlanView v = view_of(plan);
  SvArgs &a = c.a;
  a.steps = v.d_steps + hc.step_off;
  a.map = v.d_map + hc.map_off;
  a.M = hc.n_steps;
  a.n_in = hc.n_in;
  a.n_out = hc.n_out;
  a.lp_const = hc.lp_const;
  if (hc.w <= kParamMapLog) {
    const int2 *hm = host_map(plan, 0);
    for (int i = 0; i < (1 << hc.w); ++i) a.p_map[i] = hm[i];
  }
  a.steps_in_params = hc.n_steps <= kParamSteps ? 1 : 0;
  if (a.steps_in_params) {
    const DevStep *hs = host_steps(plan, 0);
    for (int k = 0; k < hc.n_steps; ++k) {
      a.p_mask[k] = hs[k].mask;
      a.p_aidx[k] = (int16_t)hs[k].aidx;
      a.p_plane[k] = (int8_t)hs[k].plane;
      a.p_fixed[k] = hs[k].fixed;
    }
  }
  a.A = hc.n_angles;
  a.items = nullptr;
  a.B = batch;
  a.angles = angles;
  a.astride = astride;
  a.psi_in = psi_in;
  a.istride = istride;
  a.psi_out = psi_out;
  a.flags = flags;
  a.logprob = logprob;
  a.status = status;
  const int ll = f64 ? sv_f64_ll(hc.w) : (gen ? sv_gen_ll(hc.w) : (variant >= 0 ? variant : default_ll(hc.w, batch)));
  if (hc.item_off >= 0 && ll >= 0 && ll <= 5 && hc.n_steps <= sv_chunk(hc.w, ll, f64 ? 16 : 8))
    a.items = v.d_items + hc.item_off;
  a.kc = (ll >= 0 && ll <= 5) ? sv_kc(hc.w, ll, f64 ? 16 : 8, hc.n_steps) : hc.w;
  const int64_t rpw = 32 >> ll;
  const int64_t warps = (batch + rpw - 1) / rpw;
  const int wpb = warps >= (int64_t)8 * sm_count_cached() ? kSvWarps : 1;
  const int64_t blocks = (warps + wpb - 1) / wpb;
  if (blocks > 0x7fffffff) return fail(MBQC_E_INVALID, "sv_forward: batch too large");
  c.ll = ll;
  c.blocks = (int)blocks;
  c.threads = 32 * wpb;
  if (gen) {
    c.gfn = pick_gen(hc.w, f64);
    if (!c.gfn) return fail(MBQC_E_UNSUPPORTED, "sv_forward: window %d", hc.w);
  } else {
    c.fn = pick(hc.w, f64);
    if (!c.fn) return fail(MBQC_E_UNSUPPORTED, "sv_forward: window %d", hc.w);
  }
  c.empty = false;
  return MBQC_OK;
}

static int sv_forward_impl(const mbqc_plan *plan, int64_t batch, const double *angles,
                           int64_t astride, const void *psi_in, int64_t istride, void *psi_out,
                           uint32_t flags, int variant, double *logprob, int32_t *status,
                           cudaStream_t stream, bool f64) {
  mbqc_sv_call c;
  int rc = sv_build(plan, batch, angles, astride, psi_in, istride, psi_out, flags, variant, logprob, status, f64, c);
  if (rc) return rc;
  return sv_exec(c, stream);
}

__global__ void outer_kernel(int64_t batch, int n, const float2 *__restrict__ psi,
                             float2 *__restrict__ rho) {
  const int64_t d = (int64_t)1 << n;
  const int64_t total = batch * d * d;
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < total;
       e += (int64_t)gridDim.x * blockDim.x) {
    const int64_t b = e / (d * d);
    const int64_t rem = e - b * d * d;
    const int64_t i = rem / d, j = rem - i * d;
    const float2 x = psi[b * d + i], y = psi[b * d + j];
    rho[e] = make_float2(x.x * y.x + x.y * y.y, x.y * y.x - x.x * y.y);
  }
}

// FP32 FMA throughput probe: 8 independent FMA chains per thread.
__global__ void fma_probe_kernel(int64_t iters, float seed, float *out) {
  float a0 = seed + threadIdx.x, a1 = a0 + 1.f, a2 = a0 + 2.f, a3 = a0 + 3.f;
  float a4 = a0 + 4.f, a5 = a0 + 5.f, a6 = a0 + 6.f, a7 = a0 + 7.f;
  const float m = 0.999999f, c = 1e-7f;
  for (int64_t i = 0; i < iters; ++i) {
#pragma unroll
    for (int u = 0; u < 16; ++u) {
      a0 = fmaf(a0, m, c); a1 = fmaf(a1, m, c); a2 = fmaf(a2, m, c); a3 = fmaf(a3, m, c);
      a4 = fmaf(a4, m, c); a5 = fmaf(a5, m, c); a6 = fmaf(a6, m, c); a7 = fmaf(a7, m, c);
    }
  }
  const float s = a0 + a1 + a2 + a3 + a4 + a5 + a6 + a7;
  if (s == 12345.678f) out[0] = s;  // keeps the chains live
}

// Shared-memory bandwidth probe: every thread streams 16-byte loads and
// stores over its block's buffer (consecutive threads on consecutive 16
// bytes: conflict free), four independent accesses in flight.
__global__ void __launch_bounds__(512) smem_probe_kernel(int64_t iters, float seed, float *out) {
  __shared__ float4 buf[2048];  // 32 KB
  const int t = threadIdx.x;
  for (int i = t; i < 2048; i += blockDim.x) buf[i] = make_float4(seed, seed, seed, seed);
  __syncthreads();
  const float m = 0.999999f;
  const uint32_t base = (uint32_t)__cvta_generic_to_shared(&buf[t]);
  for (int64_t i = 0; i < iters; ++i) {
#pragma unroll
    for (int u = 0; u < 4; ++u) {  // explicit shared loads and stores: the compiler may not keep them in registers
      const uint32_t a = base + 512u * 16u * (uint32_t)u;
      float x, y, z, w;
      asm volatile("ld.shared.v4.f32 {%0, %1, %2, %3}, [%4];" : "=f"(x), "=f"(y), "=f"(z), "=f"(w) : "r"(a) : "memory");
      asm volatile("st.shared.v4.f32 [%0], {%1, %2, %3, %4};" ::"r"(a), "f"(x * m), "f"(y * m), "f"(z * m), "f"(w * m)
                   : "memory");
    }
  }
  __syncthreads();
  if (buf[t].x == 12345.678f) out[0] = buf[t].y;  // keeps the traffic live
}

}  // namespace mbqc

using namespace mbqc;

extern "C" {

int mbqc_probe_smem_bw(int64_t iters, float *sink, double *gbs, mbqc_stream_t stream) {
  if (iters <= 0 || !sink || !gbs) return fail(MBQC_E_INVALID, "probe: bad arguments");
  const int blocks = sm_count_cached() * 4, threads = 512;
  cudaStream_t s = (cudaStream_t)stream;
  cudaEvent_t e0, e1;
  int rc = cuda_check(cudaEventCreate(&e0), "event");
  if (rc) return rc;
  rc = cuda_check(cudaEventCreate(&e1), "event");
  if (rc) { cudaEventDestroy(e0); return rc; }
  smem_probe_kernel<<<blocks, threads, 0, s>>>(iters / 4 + 1, 1.0f, sink);  // warm-up
  cudaEventRecord(e0, s);
  smem_probe_kernel<<<blocks, threads, 0, s>>>(iters, 1.0f, sink);
  cudaEventRecord(e1, s);
  rc = check_launch("smem_probe_kernel");
  if (!rc) rc = cuda_check(cudaEventSynchronize(e1), "probe sync");
  float ms = 0.f;
  if (!rc) rc = cuda_check(cudaEventElapsedTime(&ms, e0, e1), "probe time");
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (rc) return rc;
  const double bytes = (double)blocks * threads * iters * 4 * 32;  // 16 B load + 16 B store per access
  *gbs = bytes / (ms * 1e-3) / 1e9;
  return MBQC_OK;
}

int mbqc_sv_forward(const mbqc_plan *plan, int64_t batch, const double *angles,
                    int64_t angle_stride, const float *psi_in, int64_t in_stride, float *psi_out,
                    uint32_t flags, int32_t variant, double *logprob, int32_t *status,
                    mbqc_stream_t stream) {
  return sv_forward_impl(plan, batch, angles, angle_stride, psi_in, in_stride, psi_out, flags,
                         variant, logprob, status, (cudaStream_t)stream, false);
}

int mbqc_sv_forward_f64(const mbqc_plan *plan, int64_t batch, const double *angles,
                        int64_t angle_stride, const double *psi_in, int64_t in_stride,
                        double *psi_out, uint32_t flags, double *logprob, int32_t *status,
                        mbqc_stream_t stream) {
  return sv_forward_impl(plan, batch, angles, angle_stride, psi_in, in_stride, psi_out, flags, -1,
                         logprob, status, (cudaStream_t)stream, true);
}

int mbqc_sv_call_create(const mbqc_plan *plan, int64_t batch, const double *angles, int64_t angle_stride,
                        const void *psi_in, int64_t in_stride, void *psi_out, uint32_t flags, int32_t variant,
                        double *logprob, int32_t *status, int32_t f64, mbqc_sv_call **call) {
  if (!call) return fail(MBQC_E_INVALID, "sv_call_create: null result pointer");
  *call = nullptr;
  mbqc_sv_call *c = new (std::nothrow) mbqc_sv_call;
  if (!c) return fail(MBQC_E_NOMEM, "sv_call_create: out of host memory");
  const int rc = sv_build(plan, batch, angles, angle_stride, psi_in, in_stride, psi_out, flags,
                          f64 ? -1 : variant, logprob, status, f64 != 0, *c);
  if (rc) {
    delete c;
    return rc;
  }
  *call = c;
  return MBQC_OK;
}

int mbqc_sv_call_launch(const mbqc_sv_call *call, mbqc_stream_t stream) {
  if (!call) return fail(MBQC_E_INVALID, "sv_call_launch: null call");
  return sv_exec(*call, (cudaStream_t)stream);
}

void mbqc_sv_call_destroy(mbqc_sv_call *call) { delete call; }

int mbqc_outer(int64_t batch, int32_t n_qubits, const float *psi, float *rho, mbqc_stream_t stream) {
  if (batch < 0 || n_qubits < 0 || n_qubits > 15) return fail(MBQC_E_INVALID, "outer: bad sizes");
  if (batch == 0) return MBQC_OK;
  if (!psi || !rho) return fail(MBQC_E_INVALID, "outer: null buffer");
  const int64_t total = batch << (2 * n_qubits);
  int64_t blocks = (total + 255) / 256;
  const int64_t cap = (int64_t)sm_count_cached() * 16;
  if (blocks > cap) blocks = cap;
  outer_kernel<<<(int)blocks, 256, 0, (cudaStream_t)stream>>>(
      batch, n_qubits, reinterpret_cast<const float2 *>(psi), reinterpret_cast<float2 *>(rho));
  return check_launch("outer_kernel");
}

int mbqc_probe_fp32_fma(int64_t iters, float *sink, double *tflops, mbqc_stream_t stream) {
  if (iters <= 0 || !sink || !tflops) return fail(MBQC_E_INVALID, "probe: bad arguments");
  const int blocks = sm_count_cached() * 8, threads = 256;
  cudaStream_t s = (cudaStream_t)stream;
  cudaEvent_t e0, e1;
  int rc = cuda_check(cudaEventCreate(&e0), "event");
  if (rc) return rc;
  rc = cuda_check(cudaEventCreate(&e1), "event");
  if (rc) { cudaEventDestroy(e0); return rc; }
  fma_probe_kernel<<<blocks, threads, 0, s>>>(iters / 4 + 1, 1.0f, sink);  // warm-up
  cudaEventRecord(e0, s);
  fma_probe_kernel<<<blocks, threads, 0, s>>>(iters, 1.0f, sink);
  cudaEventRecord(e1, s);
  rc = check_launch("fma_probe_kernel");
  if (!rc) rc = cuda_check(cudaEventSynchronize(e1), "probe sync");
  float ms = 0.f;
  if (!rc) rc = cuda_check(cudaEventElapsedTime(&ms, e0, e1), "probe time");
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (rc) return rc;
  const double fmas = (double)blocks * threads * iters * 16 * 8;
  *tflops = 2.0 * fmas / (ms * 1e-3) / 1e12;
  return MBQC_OK;
}

}  // extern "C"
