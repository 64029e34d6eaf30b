// Adjoint gradient of the statevector sweep for windows 9..20, and for plans
// with XZ / YZ steps at any window up to 20: a block per run.
//
// The chain is the one of sv_adj.cuh: per step k the window is scaled by an
// exact power of two alpha_k (its norm then lies in [1, 4)), measured and
// expanded,
//   psi_k = E_k C_k(alpha_k u_{k-1}),  C_k: phi[r] = v[r, 0] + c_k v[r, 1],
// and the output is z = u_M / |u_M|.  Backward, with lambda_M = dL/du_M:
//   mu[r]              = lambda_k[r, 0] + s_k(r) lambda_k[r, 1]
//   dL/dtheta_k        = alpha_k Im(c_k sum_r conj(mu[r]) u_{k-1}[r, 1])
//   lambda_{k-1}[r, 0] = alpha_k mu[r],  lambda_{k-1}[r, 1] = alpha_k conj(c_k) mu[r].
//
// The window does not fit in registers here, so the block keeps it in shared
// memory (w <= 14) or in its workspace slot (w >= 15), one pair of the
// measured bit per thread and pass.  The forward pass writes the pre-step
// half-state u_{k-1}[., 1] of every step to the slot's history (2^(w-1)
// complex64 per step) and the backward pass reads it back: one forward, one
// backward, no recompute.  The grid is persistent (a workspace slot per
// block); the slot count is capped so the workspace stays within
// kWideAdjMaxWorkspace.  Block sums (norms, <z|g>, the gradient terms) are a
// butterfly per warp, then the warps' partials in a fixed order, so every
// thread holds the same bits.  The input placement and the output gather are
// computed from the plan's bit tables (no index map, which stops at w = 16).
//
// GEN (plans with XZ / YZ steps): the step is phi = amp v[., 0] + c v[., 1]
// with both coefficients depending on theta (sv_coef_gen: amp = C + S and
// c = C - S (XZ) or -i (C - S) (YZ), C, S = cos, sin of half the reduced
// angle), so d amp / dtheta = (C - S) / 2 and dc / dtheta = -amp / 2 (XZ) or
// i amp / 2 (YZ); an XY step keeps amp = 1 and dc = -i c.  Backward:
//   dL/dtheta_k = alpha_k Re(damp sum conj(mu) u[., 0] + dc sum conj(mu) u[., 1])
//   lambda_{k-1}[r, 0] = alpha_k amp mu[r],  lambda_{k-1}[r, 1] = alpha_k conj(c) mu[r]
// and the history keeps both halves of every pre-step state.
//
// CS > 1 (windows >= 15, batches smaller than the GPU): a cluster of CS blocks
// shares one run, each block taking a 1/CS slice of every pass; the block
// sums are then summed over the cluster (each block's partials read through
// distributed shared memory, in rank order, so every thread still holds the
// same bits) and the cluster barrier that does it also orders the window's
// global writes between the blocks.  Every block of a cluster runs the same
// loops, so every barrier is reached by all of them.
#include <cuda_runtime.h>

#include <type_traits>

#include "cluster_sum.cuh"
#include "dispatch.h"
#include "sv_adj.cuh"

namespace mbqc {

template <int W>
struct WideAdjCfg {
  static constexpr int D = 1 << W;
  static constexpr int TPR = W <= 9 ? 128 : (W == 10 ? 256 : (W == 11 ? 512 : 1024));
  static constexpr int NW = TPR / 32;
  static constexpr bool kWs = W > 14;  // the window itself in the workspace slot
};

// pairs per thread whose loads are issued together in a pass: 4 took the
// 64-run grid 16 x 10 adjoint (w = 17) from 7.85 to 5.84 ms (2: 6.52 ms; 8
// spills ~650 bytes a thread under the 64 registers of a 1,024-thread
// block).  GEN keeps both history halves per pair, so it takes 2.
template <bool GEN>
constexpr int kWideBatch = GEN ? 2 : 4;

__device__ __forceinline__ uint32_t wide_insert_bit(uint32_t r, int p) {
  return ((r >> p) << (p + 1)) | (r & ((1u << p) - 1u));
}

__host__ __device__ inline size_t wide_al(size_t b) { return (b + 15) & ~(size_t)15; }

// shared memory of one block: [window (w <= 14)] [coef M] [mask M] [aidx M] [expo M] [red 2 x NW x 4]
// [general-plane derivative table M (GEN)]
__host__ __device__ inline size_t wide_smem_bytes(int w, int M, bool gen) {
  const int tpr = w <= 9 ? 128 : (w == 10 ? 256 : (w == 11 ? 512 : 1024));
  return (w > 14 ? 0 : wide_al(((size_t)1 << w) * 8)) + wide_al((size_t)M * 8) + 3 * wide_al((size_t)M * 4) +
         wide_al((size_t)2 * (tpr / 32) * 4 * sizeof(float)) + (gen ? wide_al((size_t)M * 16) : 0);
}

// Sum of NV per-thread values over the block; the same bits in every thread.
// red is double-buffered: a fast thread's next call cannot overwrite partials
// a slow thread is still reading (it waits at the next barrier first).
template <int NW, int NV>
__device__ __forceinline__ void block_sum(float (&v)[NV], float *red, int &par) {
#pragma unroll
  for (int j = 0; j < NV; ++j)
#pragma unroll
    for (int o = 16; o >= 1; o >>= 1) v[j] += __shfl_xor_sync(0xffffffffu, v[j], o);
  float *r = red + par * (NW * 4);
  if ((threadIdx.x & 31) == 0) {
#pragma unroll
    for (int j = 0; j < NV; ++j) r[(threadIdx.x >> 5) * 4 + j] = v[j];
  }
  __syncthreads();
#pragma unroll
  for (int j = 0; j < NV; ++j) {
    float s = 0.f;
#pragma unroll
    for (int w = 0; w < NW; ++w) s += r[w * 4 + j];
    v[j] = s;
  }
  par ^= 1;
}


template <int W, bool GEN, int CS>
__global__ void __launch_bounds__(WideAdjCfg<W>::TPR) sv_adj_wide(SvAdjArgs A, WideAdjGeom G) {
  using Cfg = WideAdjCfg<W>;
  constexpr int D = Cfg::D, TPR = Cfg::TPR, NW = Cfg::NW, H2 = D / 2;
  constexpr int HS = GEN ? D : H2;  // history entries per step (both halves for GEN)
  static_assert(CS == 1 || Cfg::kWs, "clusters share a run only with the window in the workspace");
  constexpr int QS = H2 / CS, DS = D / CS;  // this block's pairs / window entries of a pass
  // a pass gives each thread NIT pairs (q = q_lo + tid + n TPR), taken U at a
  // time: the U pairs' loads are all issued before the first write-back (the
  // window sits in the workspace above w = 14, and a load after a store to
  // it cannot be hoisted by the compiler), so a thread keeps 2U window loads
  // (3U in the backward pass, with the history) in flight instead of two;
  // each thread still sums its pairs in q order
  constexpr int NIT = QS >= TPR ? QS / TPR : 1;
  constexpr int U = NIT < kWideBatch<GEN> ? NIT : kWideBatch<GEN>;
  static_assert((QS < TPR || QS % TPR == 0) && NIT % U == 0, "pairs per thread");
  using HistT = typename std::conditional<GEN, float4, float2>::type;
  const bool live = QS >= TPR || threadIdx.x < (unsigned)QS;  // small windows: fewer pairs than threads
  __shared__ float cred[8];
  extern __shared__ __align__(16) unsigned char smem[];
  const int tid = threadIdx.x;
  const int M = A.M, NA = A.n_angles;
  size_t off = Cfg::kWs ? 0 : wide_al((size_t)D * 8);
  float2 *s_coef = reinterpret_cast<float2 *>(smem + off);
  off += wide_al((size_t)M * 8);
  uint32_t *s_mask = reinterpret_cast<uint32_t *>(smem + off);
  off += wide_al((size_t)M * 4);
  int32_t *s_aidx = reinterpret_cast<int32_t *>(smem + off);
  off += wide_al((size_t)M * 4);
  int32_t *s_expo = reinterpret_cast<int32_t *>(smem + off);
  off += wide_al((size_t)M * 4);
  float *red = reinterpret_cast<float *>(smem + off);
  off += wide_al((size_t)2 * NW * 4 * sizeof(float));
  float4 *s_gen = reinterpret_cast<float4 *>(smem + off);  // [M] (amp, damp, dc) for GEN

  int crank = 0, cid = blockIdx.x, ncl = gridDim.x, cpar = 0;
  if constexpr (CS > 1) {
    crank = (int)cooperative_groups::this_cluster().block_rank();
    cid = blockIdx.x / CS;
    ncl = gridDim.x / CS;
  }
  const int q_lo = crank * QS, i_lo = crank * DS;
  float2 *slot = reinterpret_cast<float2 *>(A.ckpt) + (size_t)cid * G.slot_elems;
  float2 *s = Cfg::kWs ? slot : reinterpret_cast<float2 *>(smem);
  float2 *hist = slot + (Cfg::kWs ? D : 0);

  for (int k = tid; k < M; k += TPR) {
    const DevStep st = A.steps[k];
    s_mask[k] = st.mask;
    s_aidx[k] = st.aidx;
  }
  const bool fid = A.J > 0;
  const int n_in = A.n_in, n_out = A.n_out;
  const int64_t dout = (int64_t)1 << n_out;
  int par = 0;

  for (int64_t run = cid; run < A.B; run += ncl) {
    const int64_t vrow = fid ? run / A.J : run;
    const int64_t irow = fid ? run % A.J : (A.istride ? run : 0);
    for (int k = tid; k < M; k += TPR) {
      const DevStep st = A.steps[k];
      const double th = st.aidx >= 0 ? A.angles[vrow * A.astride + st.aidx] : st.fixed;
      float2 c, ph;
      if constexpr (GEN) {
        float amp;
        sv_coef_gen(st.plane, th, false, c, amp, ph);
        float damp = 0.f;
        float2 dc = make_float2(c.y, -c.x);  // XY: -i c
        if (st.plane == MBQC_PLANE_XZ) {
          damp = 0.5f * c.x;  // (C - S) / 2
          dc = make_float2(-0.5f * amp, 0.f);
        } else if (st.plane == MBQC_PLANE_YZ) {
          damp = -0.5f * c.y;  // c = -i (C - S)
          dc = make_float2(0.f, 0.5f * amp);
        }
        s_gen[k] = make_float4(amp, damp, dc.x, dc.y);
      } else {
        sv_coef(st.plane, th, false, c, ph);
      }
      s_coef[k] = c;
    }
    // ---- initial window: input on its bits, |+> elsewhere, the CZ layer's signs
    const float2 *in = reinterpret_cast<const float2 *>(A.psi_in) +
                       irow * (fid ? ((int64_t)1 << n_in) : A.istride);
    float nv[1] = {0.f};
    for (int i = i_lo + tid; i < i_lo + DS; i += TPR) {
      const float2 v = flip_sign(in[gather_bits((uint32_t)i, G.in_bits, n_in)],
                                 init_parity((uint32_t)i, G.init_cz, W) << 31);
      s[i] = v;
      nv[0] += v.x * v.x + v.y * v.y;
    }
    block_sum<NW, 1>(nv, red, par);
    cluster_sum<CS, 1>(nv, cred, cpar);
    float nrm = nv[0];

    // ---- forward, keeping every step's pre-step half-state
    for (int k = 0; k < M; ++k) {
      const int e = renorm_exponent<float>(nrm);
      if (tid == 0) s_expo[k] = e;
      const float al = RealBits<float>::pow2(-e);
      const float2 c = s_coef[k];
      const float amp = GEN ? s_gen[k].x : 1.f;
      const uint32_t mask = s_mask[k];
      const bool dead = (mask & kDead) != 0u;
      const int p = k % W;
      float2 *hk = hist + (size_t)k * HS;
      float acc[1] = {0.f};
      if (live) {
        for (int b = 0; b < NIT; b += U) {
          float2 u0[U], u1[U];  // U pairs loaded before any is written back
#pragma unroll
          for (int j = 0; j < U; ++j) {
            const uint32_t i0 = wide_insert_bit((uint32_t)(q_lo + tid + (b + j) * TPR), p);
            u0[j] = s[i0];
            u1[j] = s[i0 | (1u << p)];
          }
#pragma unroll
          for (int j = 0; j < U; ++j) {
            const int q = q_lo + tid + (b + j) * TPR;
            const uint32_t i0 = wide_insert_bit((uint32_t)q, p), i1 = i0 | (1u << p);
            if constexpr (GEN)
              reinterpret_cast<float4 *>(hk)[q] = make_float4(u0[j].x, u0[j].y, u1[j].x, u1[j].y);
            else
              hk[q] = u1[j];
            const float2 phi = make_float2(al * (amp * u0[j].x + c.x * u1[j].x - c.y * u1[j].y),
                                           al * (amp * u0[j].y + c.x * u1[j].y + c.y * u1[j].x));
            s[i0] = phi;
            s[i1] = dead ? make_float2(0.f, 0.f) : flip_sign(phi, (uint32_t)(__popc(i1 & mask) & 1u) << 31);
            acc[0] += phi.x * phi.x + phi.y * phi.y;
          }
        }
      }
      block_sum<NW, 1>(acc, red, par);
      cluster_sum<CS, 1>(acc, cred, cpar);
      nrm = dead ? acc[0] : 2.f * acc[0];
    }

    // ---- output and the seed lambda_M = dL/du_M
    const bool ok = RealBits<float>::finite_pos(nrm);
    float inv = 0.f;
    if (ok) {
      const float y = rsqrtf(nrm);
      inv = y * (1.5f - 0.5f * nrm * y * y);  // one Newton step
    }
    if (!ok) {
      if (!fid)
        for (int ai = tid; ai < NA && crank == 0; ai += TPR) A.grad[run * NA + ai] = NAN;
      if (tid == 0 && crank == 0 && A.status) A.status[run] = isnan(nrm) ? MBQC_RUN_NAN : MBQC_RUN_ZERO_NORM;
      run_barrier<CS>();  // the next run overwrites the coefficients
      continue;
    }
    float loss_term = 0.f;
    if (fid) {
      const float2 *tg = reinterpret_cast<const float2 *>(A.targets) + irow * dout;
      float pv[2] = {0.f, 0.f};  // <t|u_M>
      for (int i = i_lo + tid; i < i_lo + DS; i += TPR) {
        if ((uint32_t)i & ~G.out_mask) continue;
        const float2 t = tg[gather_bits((uint32_t)i, G.out_bits, n_out)], a = s[i];
        pv[0] += t.x * a.x + t.y * a.y;
        pv[1] += t.x * a.y - t.y * a.x;
      }
      block_sum<NW, 2>(pv, red, par);
      cluster_sum<CS, 2>(pv, cred, cpar);
      const float ar = pv[0] * inv, ai = pv[1] * inv;
      const float F = ar * ar + ai * ai;
      const float wJ = 1.f / (float)A.J;
      loss_term = (1.f - F) * wJ;
      // lambda = (2/J)(F z - a t) / |u_M|
      const float k2 = 2.f * wJ * inv, fz = F * inv;
      for (int i = i_lo + tid; i < i_lo + DS; i += TPR) {
        float2 l = make_float2(0.f, 0.f);
        if (!((uint32_t)i & ~G.out_mask)) {
          const float2 t = tg[gather_bits((uint32_t)i, G.out_bits, n_out)], a = s[i];
          l = make_float2(k2 * (fz * a.x - (ar * t.x - ai * t.y)), k2 * (fz * a.y - (ar * t.y + ai * t.x)));
        }
        s[i] = l;
      }
    } else {
      const float2 *go = reinterpret_cast<const float2 *>(A.grad_out) + run * dout;
      float zv[1] = {0.f};  // Re <u_M|g>
      for (int i = i_lo + tid; i < i_lo + DS; i += TPR) {
        if ((uint32_t)i & ~G.out_mask) continue;
        const float2 g = go[gather_bits((uint32_t)i, G.out_bits, n_out)], a = s[i];
        zv[0] += a.x * g.x + a.y * g.y;
      }
      block_sum<NW, 1>(zv, red, par);
      cluster_sum<CS, 1>(zv, cred, cpar);
      const float zgi = zv[0] * inv * inv;
      for (int i = i_lo + tid; i < i_lo + DS; i += TPR) {
        float2 l = make_float2(0.f, 0.f);
        if (!((uint32_t)i & ~G.out_mask)) {
          const float2 g = go[gather_bits((uint32_t)i, G.out_bits, n_out)], a = s[i];
          l = make_float2(inv * (g.x - zgi * a.x), inv * (g.y - zgi * a.y));
        }
        s[i] = l;
      }
    }
    run_barrier<CS>();

    // ---- backward
    for (int k = M - 1; k >= 0; --k) {
      const float al = RealBits<float>::pow2(-s_expo[k]);
      const float2 c = s_coef[k];
      const float amp = GEN ? s_gen[k].x : 1.f;
      const uint32_t mask = s_mask[k];
      const bool dead = (mask & kDead) != 0u;
      const int p = k % W;
      const float2 *hk = hist + (size_t)k * HS;
      float t[GEN ? 4 : 2] = {};  // sum conj(mu) u[., 1] (and sum conj(mu) u[., 0])
      if (live) {
        for (int b = 0; b < NIT; b += U) {
          // U pairs and their history entries loaded before any is written back
          float2 l0[U], l1[U];
          HistT hh[U];
#pragma unroll
          for (int j = 0; j < U; ++j) {
            const int q = q_lo + tid + (b + j) * TPR;
            const uint32_t i0 = wide_insert_bit((uint32_t)q, p);
            l0[j] = s[i0];
            l1[j] = dead ? make_float2(0.f, 0.f) : s[i0 | (1u << p)];
            hh[j] = reinterpret_cast<const HistT *>(hk)[q];
          }
#pragma unroll
          for (int j = 0; j < U; ++j) {
            const int q = q_lo + tid + (b + j) * TPR;
            const uint32_t i0 = wide_insert_bit((uint32_t)q, p), i1 = i0 | (1u << p);
            float2 mu = l0[j];
            if (!dead) {
              const float2 m1 = flip_sign(l1[j], (uint32_t)(__popc(i1 & mask) & 1u) << 31);
              mu.x += m1.x;
              mu.y += m1.y;
            }
            float2 h;
            if constexpr (GEN) {
              h = make_float2(hh[j].z, hh[j].w);
              t[2] += mu.x * hh[j].x + mu.y * hh[j].y;
              t[3] += mu.x * hh[j].y - mu.y * hh[j].x;
            } else {
              h = make_float2(hh[j].x, hh[j].y);
            }
            t[0] += mu.x * h.x + mu.y * h.y;
            t[1] += mu.x * h.y - mu.y * h.x;
            s[i0] = make_float2(al * amp * mu.x, al * amp * mu.y);
            s[i1] = make_float2(al * (c.x * mu.x + c.y * mu.y), al * (c.x * mu.y - c.y * mu.x));  // conj(c) mu
          }
        }
      }
      block_sum<NW, GEN ? 4 : 2>(t, red, par);
      cluster_sum<CS, GEN ? 4 : 2>(t, cred, cpar);
      const int ai = s_aidx[k];
      if (tid == 0 && crank == 0 && ai >= 0) {
        double g;
        if constexpr (GEN) {  // alpha Re(damp t0 + dc t1)
          const float4 gd = s_gen[k];
          g = (double)al * ((double)gd.y * t[2] + (double)gd.z * t[0] - (double)gd.w * t[1]);
        } else {
          g = (double)al * ((double)c.x * t[1] + (double)c.y * t[0]);  // alpha Im(c t)
        }
        if (fid)
          atomicAdd(&A.grad[vrow * NA + ai], g);
        else
          A.grad[run * NA + ai] = g;
      }
    }
    if (tid == 0 && crank == 0) {
      if (fid) atomicAdd(&A.loss[vrow], (double)loss_term);
      if (A.status) A.status[run] = MBQC_RUN_OK;
    }
    run_barrier<CS>();  // the next run overwrites the window, the coefficients and the exponents
  }
}

template <int W, bool GEN, int CS>
static int wide_launch(const SvAdjArgs &a, const WideAdjGeom &g, const AdjLaunch &l, cudaStream_t s) {
  auto k = sv_adj_wide<W, GEN, CS>;
  if (cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)l.smem) != cudaSuccess)
    return fail(MBQC_E_UNSUPPORTED, "adjoint: %zu bytes of shared memory per block", l.smem);
  if (l.query) {
    int occ = 0;
    int rc = cuda_check(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k, WideAdjCfg<W>::TPR, l.smem),
                        "occupancy");
    if (rc) return rc;
    *l.occ = occ;
    return MBQC_OK;
  }
  if constexpr (CS == 1) {
    k<<<l.blocks, WideAdjCfg<W>::TPR, l.smem, s>>>(a, g);
  } else {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(l.blocks * CS);
    cfg.blockDim = dim3(WideAdjCfg<W>::TPR);
    cfg.dynamicSmemBytes = l.smem;
    cfg.stream = s;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeClusterDimension;
    at[0].val.clusterDim.x = CS;
    at[0].val.clusterDim.y = 1;
    at[0].val.clusterDim.z = 1;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    const int rc = cuda_check(cudaLaunchKernelEx(&cfg, k, a, g), "sv_adj_wide cluster launch");
    if (rc) return rc;
  }
  return check_launch("sv_adj_wide");
}

template <int W>
static int wide_pick(const SvAdjArgs &a, const WideAdjGeom &g, const AdjLaunch &l, cudaStream_t s, bool gen) {
  if (gen) return wide_launch<W, true, 1>(a, g, l, s);
  if constexpr (W >= 9) {
    if constexpr (WideAdjCfg<W>::kWs) {
      if (g.cluster == 4) return wide_launch<W, false, 4>(a, g, l, s);
      if (g.cluster == 2) return wide_launch<W, false, 2>(a, g, l, s);
    }
    return wide_launch<W, false, 1>(a, g, l, s);
  }
  return fail(MBQC_E_UNSUPPORTED, "adjoint: window %d takes the register kernel", W);
}

int wide_adj_threads(int w) { return w <= 9 ? 128 : (w == 10 ? 256 : (w == 11 ? 512 : 1024)); }
size_t wide_adj_smem(int w, int M, bool gen) { return wide_smem_bytes(w, M, gen); }

int launch_sv_adj_wide(const SvAdjArgs &a, const WideAdjGeom &g, const AdjLaunch &l, cudaStream_t s, bool gen) {
  switch (a.W) {
    case 1: return wide_pick<1>(a, g, l, s, gen);
    case 2: return wide_pick<2>(a, g, l, s, gen);
    case 3: return wide_pick<3>(a, g, l, s, gen);
    case 4: return wide_pick<4>(a, g, l, s, gen);
    case 5: return wide_pick<5>(a, g, l, s, gen);
    case 6: return wide_pick<6>(a, g, l, s, gen);
    case 7: return wide_pick<7>(a, g, l, s, gen);
    case 8: return wide_pick<8>(a, g, l, s, gen);
    case 9: return wide_pick<9>(a, g, l, s, gen);
    case 10: return wide_pick<10>(a, g, l, s, gen);
    case 11: return wide_pick<11>(a, g, l, s, gen);
    case 12: return wide_pick<12>(a, g, l, s, gen);
    case 13: return wide_pick<13>(a, g, l, s, gen);
    case 14: return wide_pick<14>(a, g, l, s, gen);
    case 15: return wide_pick<15>(a, g, l, s, gen);
    case 16: return wide_pick<16>(a, g, l, s, gen);
    case 17: return wide_pick<17>(a, g, l, s, gen);
    case 18: return wide_pick<18>(a, g, l, s, gen);
    case 19: return wide_pick<19>(a, g, l, s, gen);
    case 20: return wide_pick<20>(a, g, l, s, gen);
    default: return fail(MBQC_E_UNSUPPORTED, "adjoint: window %d", a.W);
  }
}

}  // namespace mbqc
