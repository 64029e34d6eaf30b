// Statevector sweep with sampled outcomes and flow byproduct corrections.
//
// The semantics of mentpy's PennyLane backend (pennylane_simulator.py:133-152):
// node i is measured in the XY plane at its angle; on outcome 1 an X acts on
// flow(i) and a Z on every neighbour of flow(i) measured after i.  Here the
// corrections are a Pauli frame: a pending X on a node flips the sign of its
// measurement angle, a pending Z adds pi (the same projections as applying
// the gates first); the frame left on the outputs is applied to the final
// state.  With a causal flow the output state does not depend on the drawn
// outcomes (up to a global phase).
//
// A group of threads owns one run: a warp for windows <= 10 (four runs per
// block), the whole block for windows 11..20 (256, 512 or 1024 threads).  The
// window sits in shared memory up to w = 14 (128 KB) and in a caller
// workspace (one 2^w slot per block, the block looping over runs) from 15.
// Batches smaller than the GPU at w >= 15 share each run among a cluster of
// 2 or 4 blocks, each taking a 1/CS slice of every pass: the group sums are
// then summed over the cluster in rank order (the same bits in every thread
// of every block, so all draw the same outcome), each block keeps its own
// copy of the frame (the same updates), and a cluster barrier ends every
// step (the next pass reads pairs the other blocks wrote).
// The input placement and the output gather use the plan's index map up to
// w = 16 and the plan's bit tables above.  The frame is a bitset over all
// steps in shared memory (two bits a step), so the number of steps is
// bounded only by that space.  Each step
// makes one pass to reduce S = sum conj(psi0) psi1 and T = sum |psi0|^2 +
// |psi1|^2 over the pairs of the measured bit (the branch weights are
// T +- 2 Re(c S)), draws the outcome (SplitMix64 of seed, run, step), and one
// pass to apply the branch, renormalised.  The step coefficients are made 32
// steps at a time, one per lane, and broadcast by shuffle.
#include <cuda_runtime.h>

#include "cluster_sum.cuh"
#include "dispatch.h"

namespace mbqc {

constexpr int kSampledSmemMaxWindow = 14;
constexpr int kSampledMaxWindow = 20;
constexpr int kSampledMaxSteps = 1 << 20;  // the step index takes 20 bits of the draw's counter

struct SampledArgs {
  const DevStep *steps;
  const int2 *map;        // index map, or nullptr above its window limit (bit tables below)
  int8_t in_bits[32];
  int8_t out_bits[32];
  uint32_t init_cz[32];
  uint32_t out_mask;
  int64_t B;
  const double *angles;
  int64_t astride;
  const float2 *psi_in;
  int64_t istride;
  float2 *psi_out;
  int M, n_in, n_out;
  uint64_t seed;
  const int32_t *x_step;  // [M] step receiving this step's X, or -1
  const int32_t *z_off;   // [M + 1] range of z_idx per step
  const int32_t *z_idx;   // steps receiving a Z
  const uint32_t *x_out;  // [M] output-index bits receiving an X
  const uint32_t *z_out;  // [M] output-index bits receiving a Z
  int8_t *outcomes;       // [B, ostride]
  int64_t ostride;
  int32_t *status;
  float2 *ws;             // [runs in flight][2^w] (windows above the shared-memory limit)
  int group_bytes;        // shared memory of one run's group
};

template <int W>
struct SampledCfg {
  static constexpr bool kWs = W > kSampledSmemMaxWindow;
  static constexpr int TPR = W <= 10 ? 32 : (W <= 12 ? 256 : (W <= 14 ? 512 : 1024));
  static constexpr int kBlock = TPR == 32 ? 128 : TPR;
};

__device__ __forceinline__ uint64_t sm64(uint64_t z) {
  z += 0x9e3779b97f4a7c15ull;
  z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
  z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
  return z ^ (z >> 31);
}

__device__ __forceinline__ uint32_t insert_bit(uint32_t r, int p, uint32_t b) {
  return ((r >> p) << (p + 1)) | (b << p) | (r & ((1u << p) - 1u));
}

template <int TPR>
__device__ __forceinline__ void group_barrier() {
  if constexpr (TPR == 32)
    __syncwarp();
  else
    __syncthreads();
}

// Sum of three per-thread values over the group, the same bits in every
// thread (a butterfly, then the warps' partials in a fixed order).
template <int TPR>
__device__ __forceinline__ void group_sum3(float &a, float &b, float &c, float *red) {
#pragma unroll
  for (int o = 16; o >= 1; o >>= 1) {
    a += __shfl_xor_sync(0xffffffffu, a, o);
    b += __shfl_xor_sync(0xffffffffu, b, o);
    c += __shfl_xor_sync(0xffffffffu, c, o);
  }
  if constexpr (TPR > 32) {
    constexpr int NW = TPR / 32;
    const int warp = threadIdx.x >> 5;
    if ((threadIdx.x & 31) == 0) {
      red[3 * warp] = a;
      red[3 * warp + 1] = b;
      red[3 * warp + 2] = c;
    }
    __syncthreads();
    a = b = c = 0.f;
#pragma unroll
    for (int w = 0; w < NW; ++w) {
      a += red[3 * w];
      b += red[3 * w + 1];
      c += red[3 * w + 2];
    }
  }
}

// the end of a step or a run: the group's barrier, or the cluster's
template <int TPR, int CS>
__device__ __forceinline__ void sampled_barrier() {
  if constexpr (CS > 1)
    run_barrier<CS>();
  else
    group_barrier<TPR>();
}

template <int W, int CS>
__global__ void __launch_bounds__(SampledCfg<W>::kBlock) sv_sampled(SampledArgs a) {
  using Cfg = SampledCfg<W>;
  constexpr int D = 1 << W, TPR = Cfg::TPR;
  static_assert(CS == 1 || (Cfg::kWs && TPR > 32), "clusters share a run only with the window in the workspace");
  constexpr int QS = D / 2 / CS, DS = D / CS;  // this block's pairs / window entries of a pass
  __shared__ float cred[8];
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int lane = threadIdx.x & 31;
  const int tid = TPR == 32 ? lane : (int)threadIdx.x;
  const int G = blockDim.x / TPR, g = threadIdx.x / TPR;
  const int M = a.M, FW = (M + 31) >> 5;
  int crank = 0, cid = blockIdx.x, ncl = gridDim.x, cpar = 0;
  if constexpr (CS > 1) {
    crank = (int)cooperative_groups::this_cluster().block_rank();
    cid = blockIdx.x / CS;
    ncl = gridDim.x / CS;
  }
  const int q_lo = crank * QS, i_lo = crank * DS;
  unsigned char *base = smem_raw + (size_t)g * a.group_bytes;
  float2 *s = Cfg::kWs ? a.ws + (size_t)cid * D : reinterpret_cast<float2 *>(base);
  uint32_t *fx = reinterpret_cast<uint32_t *>(base + (Cfg::kWs ? 0 : (size_t)D * sizeof(float2)));
  uint32_t *fz = fx + FW;
  float *red = reinterpret_cast<float *>(fz + FW);

  // G == 1 whenever TPR > 32, so the block-wide barriers see the same trip count
  for (int64_t run = (int64_t)cid * G + g; run < a.B; run += (int64_t)ncl * G) {
    for (int i = tid; i < 2 * FW; i += TPR) fx[i] = 0u;
    const float2 *in = a.psi_in + (a.istride ? run * a.istride : 0);
    for (int i = i_lo + tid; i < i_lo + DS; i += TPR) {
      if (a.map) {
        const int2 m = a.map[i];
        s[i] = flip_sign(in[m.x & 0x7fffffff], (uint32_t)m.x & 0x80000000u);
      } else {
        s[i] = flip_sign(in[gather_bits((uint32_t)i, a.in_bits, a.n_in)],
                         init_parity((uint32_t)i, a.init_cz, W) << 31);
      }
    }
    sampled_barrier<TPR, CS>();

    uint32_t xo = 0, zo = 0;  // pending X / Z on the outputs
    int32_t code = MBQC_RUN_OK;
    float2 creg = make_float2(0.f, 0.f);
    uint32_t mreg = 0u;
    for (int k = 0; k < M; ++k) {
      if ((k & 31) == 0 && k + lane < M) {  // coefficients of steps k .. k+31, one per lane
        const DevStep st = a.steps[k + lane];
        const double th = st.aidx >= 0 ? a.angles[run * a.astride + st.aidx] : st.fixed;
        float2 ph;
        sv_coef(st.plane, th, false, creg, ph);
        mreg = st.mask;
      }
      float2 c = make_float2(__shfl_sync(0xffffffffu, creg.x, k & 31), __shfl_sync(0xffffffffu, creg.y, k & 31));
      const uint32_t mask = __shfl_sync(0xffffffffu, mreg, k & 31);
      const bool dead = (mask & kDead) != 0u;
      const int p = k % W;
      const uint32_t bit = 1u << (k & 31);
      if (fx[k >> 5] & bit) c.y = -c.y;                         // X: angle -> -angle
      if (fz[k >> 5] & bit) c = make_float2(-c.x, -c.y);       // Z: angle -> angle + pi
      // branch weights
      float sr = 0.f, si = 0.f, t = 0.f;
      for (int q = q_lo + tid; q < q_lo + QS; q += TPR) {
        const uint32_t i0 = insert_bit((uint32_t)q, p, 0u), i1 = i0 | (1u << p);
        const float2 u = s[i0], v = s[i1];
        sr += u.x * v.x + u.y * v.y;
        si += u.x * v.y - u.y * v.x;
        t += u.x * u.x + u.y * u.y + v.x * v.x + v.y * v.y;
      }
      group_sum3<TPR>(sr, si, t, red);
      if constexpr (CS > 1) {
        float v3[3] = {sr, si, t};
        cluster_sum<CS, 3>(v3, cred, cpar);
        sr = v3[0];
        si = v3[1];
        t = v3[2];
      }
      const float re = c.x * sr - c.y * si;  // Re(c S)
      const float n0 = t + 2.f * re, n1 = t - 2.f * re;
      const uint64_t h = sm64(a.seed ^ sm64(((uint64_t)run << 20) ^ (uint64_t)k));
      const float u01 = (float)(h >> 40) * 5.9604644775390625e-08f;
      const int m = (u01 * (n0 + n1) >= n0) ? 1 : 0;
      const float nm = m ? n1 : n0;
      if (!(nm > 0.f) || isnan(nm) || isinf(nm)) {  // the same value in every thread of the group
        code = isnan(nm) ? MBQC_RUN_NAN : MBQC_RUN_ZERO_NORM;
        break;
      }
      const float gn = rsqrtf(dead ? nm : 2.f * nm);
      const float2 ce = m ? make_float2(-c.x, -c.y) : c;
      for (int q = q_lo + tid; q < q_lo + QS; q += TPR) {
        const uint32_t i0 = insert_bit((uint32_t)q, p, 0u), i1 = i0 | (1u << p);
        const float2 u = s[i0], v = s[i1];
        const float2 phi =
            make_float2(gn * (u.x + ce.x * v.x - ce.y * v.y), gn * (u.y + ce.x * v.y + ce.y * v.x));
        s[i0] = phi;
        s[i1] = dead ? make_float2(0.f, 0.f) : flip_sign(phi, (uint32_t)(__popc(i1 & mask) & 1u) << 31);
      }
      if (m) {  // byproducts of outcome 1 go to later steps only (checked on the host; skipped here otherwise)
        if (tid == 0) {
          const int xt = a.x_step[k];
          if (xt > k && xt < M) atomicXor(&fx[xt >> 5], 1u << (xt & 31));
        }
        const int z0 = a.z_off[k], z1 = a.z_off[k + 1];
        for (int j = z0 + tid; j < z1; j += TPR) {
          const int zt = a.z_idx[j];
          if (zt > k && zt < M) atomicXor(&fz[zt >> 5], 1u << (zt & 31));
        }
        xo ^= a.x_out[k];
        zo ^= a.z_out[k];
      }
      if (tid == 0 && crank == 0 && a.outcomes) a.outcomes[run * a.ostride + k] = (int8_t)m;
      sampled_barrier<TPR, CS>();
    }
    const int dout = 1 << a.n_out;
    float2 *out = a.psi_out + run * dout;
    for (int i = i_lo + tid; i < i_lo + DS; i += TPR) {
      const int y = a.map ? a.map[i].y
                          : (((uint32_t)i & ~a.out_mask) ? -1 : gather_bits((uint32_t)i, a.out_bits, a.n_out));
      if (y < 0) continue;
      const uint32_t yy = (uint32_t)y ^ xo;  // X on the outputs permutes the index
      const float2 v = code == MBQC_RUN_OK ? s[i] : make_float2(NAN, NAN);
      out[yy] = flip_sign(v, (uint32_t)(__popc(yy & zo) & 1u) << 31);  // then Z signs
    }
    if (tid == 0 && crank == 0 && a.status) a.status[run] = code;
    sampled_barrier<TPR, CS>();  // the next run overwrites the window and the frame
  }
}

static int64_t sampled_slots(int64_t batch) { return batch < sm_count() ? batch : (int64_t)sm_count(); }

static size_t sampled_ws_bytes(int w, int64_t batch) {
  return w > kSampledSmemMaxWindow ? (size_t)sampled_slots(batch) * ((size_t)1 << w) * sizeof(float2) : 0;
}

// runs x CS blocks in clusters of CS (runs <= the workspace slots)
template <int W, int CS>
static int sampled_cluster_launch(const SampledArgs &a, int runs, size_t smem, cudaStream_t s) {
  if constexpr (SampledCfg<W>::kWs && SampledCfg<W>::TPR > 32) {
    auto k = sv_sampled<W, CS>;
    int rc = cuda_check(cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem),
                        "sampled smem attribute");
    if (rc) return rc;
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned)(runs * CS));
    cfg.blockDim = dim3(SampledCfg<W>::TPR);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = s;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeClusterDimension;
    at[0].val.clusterDim.x = CS;
    at[0].val.clusterDim.y = 1;
    at[0].val.clusterDim.z = 1;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    rc = cuda_check(cudaLaunchKernelEx(&cfg, k, a), "sv_sampled cluster launch");
    if (rc) return rc;
    return check_launch("sv_sampled");
  } else {
    return fail(MBQC_E_UNSUPPORTED, "sv_forward_sampled: window %d has no cluster form", W);
  }
}

template <int W>
static int launch_sampled(SampledArgs a, size_t ws_bytes, cudaStream_t s) {
  using Cfg = SampledCfg<W>;
  const int fw = (a.M + 31) >> 5;
  size_t gb = (Cfg::kWs ? 0 : ((size_t)1 << W) * sizeof(float2)) + (size_t)8 * fw +
              (Cfg::TPR > 32 ? (size_t)12 * (Cfg::TPR / 32) : 0);
  gb = (gb + 15) & ~(size_t)15;
  int dev = 0, optin = 0;
  int rc = cuda_check(cudaGetDevice(&dev), "cudaGetDevice");
  if (rc) return rc;
  rc = cuda_check(cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev), "smem limit");
  if (rc) return rc;
  int G = Cfg::TPR == 32 ? Cfg::kBlock / 32 : 1;
  while (G > 1 && (size_t)G * gb > (size_t)optin) G >>= 1;
  if ((size_t)G * gb > (size_t)optin)
    return fail(MBQC_E_UNSUPPORTED, "sv_forward_sampled: window %d with %d steps needs %zu bytes of shared memory",
                W, a.M, gb);
  a.group_bytes = (int)gb;
  int64_t blocks = (a.B + G - 1) / G;
  int cs = 1;  // blocks per run (a cluster when > 1)
  if (Cfg::kWs) {
    const size_t slot = ((size_t)1 << W) * sizeof(float2);
    if (!a.ws || ws_bytes < slot)
      return fail(MBQC_E_INVALID, "sv_forward_sampled: window %d needs a workspace (mbqc_sv_sampled_workspace)", W);
    const int64_t slots = (int64_t)(ws_bytes / slot);
    if (blocks > slots) blocks = slots;
    // a batch smaller than the GPU: more SMs per run, each run still in one slot
    const int64_t sms = sm_count();
    cs = a.B * 4 <= sms ? 4 : (a.B * 2 <= sms ? 2 : 1);
  }
  if (blocks > 0x7fffffff / 4) blocks = 0x7fffffff / 4;  // the blocks loop over the remaining runs
  if (cs == 4) return sampled_cluster_launch<W, 4>(a, (int)blocks, G * gb, s);
  if (cs == 2) return sampled_cluster_launch<W, 2>(a, (int)blocks, G * gb, s);
  auto k = sv_sampled<W, 1>;
  rc = cuda_check(cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)(G * gb)),
                  "sampled smem attribute");
  if (rc) return rc;
  k<<<(int)blocks, G * Cfg::TPR, G * gb, s>>>(a);
  return check_launch("sv_sampled");
}

}  // namespace mbqc

using namespace mbqc;

extern "C" int mbqc_sv_sampled_workspace(const mbqc_plan *plan, int64_t batch, size_t *bytes) {
  if (!plan || !bytes) return fail(MBQC_E_INVALID, "sv_sampled_workspace: null argument");
  if (batch < 0) return fail(MBQC_E_INVALID, "sv_sampled_workspace: negative batch");
  *bytes = sampled_ws_bytes(host_circuit(plan, 0).w, batch);
  return MBQC_OK;
}

extern "C" int mbqc_sv_forward_sampled(const mbqc_plan *plan, int64_t batch, const double *angles,
                                       int64_t angle_stride, const float *psi_in, int64_t in_stride,
                                       float *psi_out, uint64_t seed, const mbqc_byproducts *corr,
                                       int8_t *outcomes, int64_t outcome_stride, int32_t *status,
                                       void *workspace, size_t workspace_bytes, mbqc_stream_t stream) {
  if (!plan) return fail(MBQC_E_INVALID, "sv_forward_sampled: null plan");
  if (batch < 0) return fail(MBQC_E_INVALID, "sv_forward_sampled: negative batch");
  if (batch == 0) return MBQC_OK;
  const DevCircuit &hc = host_circuit(plan, 0);
  if (!psi_in || !psi_out || !corr) return fail(MBQC_E_INVALID, "sv_forward_sampled: null buffer");
  if (!hc.sv_planes_ok) return fail(MBQC_E_UNSUPPORTED, "sv_forward_sampled: steps in XY, X or Y only");
  if (hc.w > kSampledMaxWindow)
    return fail(MBQC_E_UNSUPPORTED, "sv_forward_sampled: window %d > %d", hc.w, kSampledMaxWindow);
  if (hc.n_steps > kSampledMaxSteps)
    return fail(MBQC_E_UNSUPPORTED, "sv_forward_sampled: %d steps > %d", hc.n_steps, kSampledMaxSteps);
  if (hc.n_out > 32) return fail(MBQC_E_UNSUPPORTED, "sv_forward_sampled: %d outputs > 32", hc.n_out);
  if (hc.n_steps > 0 && (!corr->x_step || !corr->z_off || !corr->z_idx || !corr->x_out || !corr->z_out))
    return fail(MBQC_E_INVALID, "sv_forward_sampled: byproduct tables");
  if (hc.n_angles > 0 && (!angles || angle_stride < hc.n_angles))
    return fail(MBQC_E_INVALID, "sv_forward_sampled: bad angle array");
  if (in_stride != 0 && in_stride < ((int64_t)1 << hc.n_in))
    return fail(MBQC_E_INVALID, "sv_forward_sampled: input stride too small");
  if (outcomes && outcome_stride < hc.n_steps) return fail(MBQC_E_INVALID, "sv_forward_sampled: outcome stride");
  const PlanView v = view_of(plan);
  SampledArgs a;
  a.steps = v.d_steps + hc.step_off;
  a.map = hc.map_off >= 0 ? v.d_map + hc.map_off : nullptr;
  for (int i = 0; i < 32; ++i) {
    a.in_bits[i] = hc.in_bits[i];
    a.out_bits[i] = hc.out_bits[i];
    a.init_cz[i] = hc.init_cz[i];
  }
  a.out_mask = hc.out_mask;
  a.B = batch;
  a.angles = angles;
  a.astride = angle_stride;
  a.psi_in = reinterpret_cast<const float2 *>(psi_in);
  a.istride = in_stride;
  a.psi_out = reinterpret_cast<float2 *>(psi_out);
  a.M = hc.n_steps;
  a.n_in = hc.n_in;
  a.n_out = hc.n_out;
  a.seed = seed;
  a.x_step = corr->x_step;
  a.z_off = corr->z_off;
  a.z_idx = corr->z_idx;
  a.x_out = corr->x_out;
  a.z_out = corr->z_out;
  a.outcomes = outcomes;
  a.ostride = outcome_stride;
  a.status = status;
  a.ws = reinterpret_cast<float2 *>(workspace);
  a.group_bytes = 0;
  cudaStream_t s = (cudaStream_t)stream;
  const size_t wb = workspace_bytes;
  switch (hc.w) {
    case 1: return launch_sampled<1>(a, wb, s);
    case 2: return launch_sampled<2>(a, wb, s);
    case 3: return launch_sampled<3>(a, wb, s);
    case 4: return launch_sampled<4>(a, wb, s);
    case 5: return launch_sampled<5>(a, wb, s);
    case 6: return launch_sampled<6>(a, wb, s);
    case 7: return launch_sampled<7>(a, wb, s);
    case 8: return launch_sampled<8>(a, wb, s);
    case 9: return launch_sampled<9>(a, wb, s);
    case 10: return launch_sampled<10>(a, wb, s);
    case 11: return launch_sampled<11>(a, wb, s);
    case 12: return launch_sampled<12>(a, wb, s);
    case 13: return launch_sampled<13>(a, wb, s);
    case 14: return launch_sampled<14>(a, wb, s);
    case 15: return launch_sampled<15>(a, wb, s);
    case 16: return launch_sampled<16>(a, wb, s);
    case 17: return launch_sampled<17>(a, wb, s);
    case 18: return launch_sampled<18>(a, wb, s);
    case 19: return launch_sampled<19>(a, wb, s);
    default: return launch_sampled<20>(a, wb, s);
  }
}
