// Adjoint of the (noisy) density-matrix sweep through the channel, windows <= 10
// (the matrix in shared memory up to 7, in a workspace slot per block above).
//
// With the outcomes held fixed, every step is linear up to its 1/prob_k
// normalisation, so rho_out = K(rho_in) / Tr K(rho_in) for a linear map K.
// For a loss with dL = Re sum conj(Gamma) d rho_out the seed is
//   Lambda_M = Gamma - Re<Gamma|rho_out> I          (on the output subspace)
// followed by the adjoint of the output depolarising channel (a Pauli channel
// is self-adjoint).  Step k (functional G_k, c_k = 1/prob_k, bit p):
//   mu[r,r']         = E^dagger(Lambda_k): sum_{b,b'} s_b(r) s_b'(r') Lambda_k[(b,r),(b',r')] / 2
//                      (or Lambda_k[(0,r),(0,r')] when no qubit entered)
//   dL/dtheta_k     += c_k Re sum_{r,r'} conj(mu[r,r']) sum_{x,x'} dG_{xx'} rho_{k-1}[(x,r),(x',r')]
//   Lambda_{k-1}     = c_k conj(G_{xx'}) mu[r,r']   on the same 2x2 block
// dG = (1 - 4q/3) dF for outcome 0 and its negative for outcome 1, with
// dF = d(P0^T)/dtheta = (d n . sigma)^T / 2.  The pre-step states rho_{k-1}
// are kept in a workspace indexed by in-flight slot (persistent grid).
#pragma once

#include "dm.cuh"

namespace mbqc {

struct DmAdjArgs {
  DmArgs f;                  // forward arguments (rho_out may be NULL)
  const float2 *grad_out;    // Gamma [row, gstride_out]
  int64_t gout_stride;
  double *grad;              // [row, grad_stride] dL/dangles
  int64_t grad_stride;
  float2 *hist;              // [slots][maxm][4^W]
  float2 *rho_ws;            // [slots][4^W]: the matrix itself for windows > kDmAdjSmemMaxWindow
  int64_t n_slots;
};

// Windows up to 7 keep rho in shared memory (128 KB at 7); 8..10 keep it in
// the workspace, one 1024-thread block per run slot.
constexpr int kDmAdjSmemMaxWindow = 7;
constexpr int kDmAdjMaxWindow = 10;

// d n / d theta of the outcome-0 Bloch vector
__device__ __forceinline__ void dbloch(int plane, double theta, float &dx, float &dy, float &dz) {
  float s = 0.f, c = 1.f;
  dx = dy = dz = 0.f;
  if (plane == MBQC_PLANE_XY || plane == MBQC_PLANE_XZ || plane == MBQC_PLANE_YZ)
    sincos_reduced(reduce_angle(theta), s, c);
  switch (plane) {
    case MBQC_PLANE_XY: dx = -s; dy = c; break;
    case MBQC_PLANE_XZ: dx = -s; dz = c; break;
    case MBQC_PLANE_YZ: dy = -s; dz = c; break;
    default: break;  // X, Y: fixed
  }
}

template <int W> struct DmAdjCfg {
  static constexpr bool kWs = W > kDmAdjSmemMaxWindow;
  static constexpr int TPR = kWs ? 1024 : DmCfg<W>::TPR;
  static constexpr int GROUPS = kWs ? 1 : DmCfg<W>::GROUPS;
  static constexpr int BLOCK = TPR * GROUPS;
  static constexpr int NRED = TPR / 32 > 8 ? TPR / 32 : 8;  // reduction scratch entries
};

template <int W> struct DmAdjSmem {
  // [rho/Lambda] | F | dF | mask | prob | outcome | reduction, per group
  static __host__ __device__ size_t group_bytes(int maxm) {
    size_t b = DmAdjCfg<W>::kWs ? 0 : (size_t)DmCfg<W>::N * sizeof(float2);
    b += (size_t)maxm * (2 * sizeof(float4) + sizeof(uint32_t) + sizeof(float2) + sizeof(int32_t));
    b += DmAdjCfg<W>::NRED * sizeof(float2);
    return (b + 15) & ~(size_t)15;
  }
  static __host__ __device__ size_t bytes(int maxm) { return DmAdjCfg<W>::GROUPS * group_bytes(maxm); }
};

template <int W>
__global__ void __launch_bounds__(DmAdjCfg<W>::BLOCK) dm_adj_smem(DmAdjArgs A) {
  using Cfg = DmCfg<W>;
  constexpr int D = Cfg::D, TPR = DmAdjCfg<W>::TPR, NB = Cfg::NB, H = D / 2;
  constexpr int GROUPS = DmAdjCfg<W>::GROUPS;
  extern __shared__ __align__(16) unsigned char smem[];
  const int group = threadIdx.x / TPR, tid = threadIdx.x % TPR;
  const int maxm = A.f.maxm;
  unsigned char *gb = smem + (size_t)group * DmAdjSmem<W>::group_bytes(maxm);
  const int64_t slot = (int64_t)blockIdx.x * GROUPS + group;
  float2 *rho = DmAdjCfg<W>::kWs ? A.rho_ws + slot * (int64_t)Cfg::N : reinterpret_cast<float2 *>(gb);
  float4 *sF = reinterpret_cast<float4 *>(gb + (DmAdjCfg<W>::kWs ? 0 : (size_t)Cfg::N * sizeof(float2)));
  float4 *sdF = sF + maxm;
  float2 *sProb = reinterpret_cast<float2 *>(sdF + maxm);  // prob_k as a (hi, lo) pair
  uint32_t *sMask = reinterpret_cast<uint32_t *>(sProb + maxm);
  int32_t *sOut = reinterpret_cast<int32_t *>(sMask + maxm);
  float2 *sRed = reinterpret_cast<float2 *>(sOut + maxm);  // DmAdjCfg<W>::NRED entries

  float2 *hist = A.hist + slot * (int64_t)maxm * Cfg::N;
  const DmArgs &F0 = A.f;
  const float qn = f64_to_f32_rn(F0.noise);
  const float a_n = 1.f - (4.f / 3.f) * qn, b_n = (2.f / 3.f) * qn;

  for (int64_t b = slot; b < F0.B; b += (int64_t)gridDim.x * GROUPS) {
    const int ci = F0.run_circuit ? F0.run_circuit[b] : 0;
    const int64_t run = F0.run_circuit ? (int64_t)ci : b;
    const DevCircuit &C = F0.circ[ci];
    const int M = C.n_steps;
    if (C.w != W || M > maxm || C.map_off < 0) {
      if (tid == 0 && F0.status) F0.status[run] = MBQC_RUN_NAN;
      continue;
    }
    const DevStep *steps = F0.steps + C.step_off;
    const int2 *map = F0.maps + C.map_off;
    const double *ang = F0.angles + run * F0.astride;
    group_sync(TPR, group);  // previous run of this group is done with shared memory
    for (int k = tid; k < M; k += TPR) {
      const DevStep st = steps[k];
      const double th = st.aidx >= 0 ? ang[st.aidx] : st.fixed;
      float nx, ny, nz, dx, dy, dz;
      bloch(st.plane, th, nx, ny, nz);
      dbloch(st.plane, th, dx, dy, dz);
      sF[k] = make_float4(a_n * 0.5f * (1.f + nz) + b_n, a_n * 0.5f * (1.f - nz) + b_n, a_n * 0.5f * nx,
                          a_n * 0.5f * ny);
      sdF[k] = make_float4(a_n * 0.5f * dz, -a_n * 0.5f * dz, a_n * 0.5f * dx, a_n * 0.5f * dy);
      sMask[k] = st.mask;
    }
    {
      const float2 *in = F0.psi_in + (F0.istride ? run * F0.istride : 0);
      const float pad = exp2f(-0.5f * (float)(C.w - C.n_in));
      for (int e = tid; e < Cfg::N; e += TPR) {
        const int i = e >> W, j = e & (D - 1);
        const int2 mi = __ldg(&map[i]), mj = __ldg(&map[j]);
        float2 u = in[mi.x & 0x7fffffff], v = in[mj.x & 0x7fffffff];
        u = flip_sign(u, ((uint32_t)(mi.x ^ mj.x)) & 0x80000000u);
        rho[e] = make_float2(pad * pad * (u.x * v.x + u.y * v.y), pad * pad * (u.y * v.x - u.x * v.y));
      }
    }
    group_sync(TPR, group);

    // ---------------------------------------------------------- forward
    int32_t st_code = MBQC_RUN_OK;
    for (int k = 0; k < M; ++k) {
      const int p = k % W;
      const float4 Fk = sF[k];
      const uint32_t mask = sMask[k];
      float part = 0.f;
      for (int r = tid; r < H; r += TPR) {
        const uint32_t r0 = ins_bit(r, p, 0), r1 = ins_bit(r, p, 1);
        const float2 q00 = rho[r0 * D + r0], q11 = rho[r1 * D + r1], q01 = rho[r0 * D + r1];
        part += Fk.x * q00.x + Fk.y * q11.x + 2.f * (Fk.z * q01.x - Fk.w * q01.y);
      }
      float2 prob = group_sum2<TPR>(part, sRed, tid, group);
      float4 G = Fk;
      int outcome = 0;
      if (!pair_ge(prob, 1e-4)) {
        const float tr_noise = a_n + 2.f * b_n;
        G = make_float4(tr_noise - Fk.x, tr_noise - Fk.y, -Fk.z, -Fk.w);
        float part1 = 0.f;
        for (int r = tid; r < H; r += TPR) {
          const uint32_t r0 = ins_bit(r, p, 0), r1 = ins_bit(r, p, 1);
          const float2 q00 = rho[r0 * D + r0], q11 = rho[r1 * D + r1], q01 = rho[r0 * D + r1];
          part1 += G.x * q00.x + G.y * q11.x + 2.f * (G.z * q01.x - G.w * q01.y);
        }
        prob = group_sum2<TPR>(part1, sRed, tid, group);
        outcome = 1;
      }
      if (tid == 0) {
        sProb[k] = prob;
        sOut[k] = outcome;
        if (F0.outcomes) F0.outcomes[run * F0.ostride + k] = (int8_t)outcome;
      }
      if (!(prob.x > 0.f) || isnan(prob.x) || isinf(prob.x)) {
        st_code = MBQC_RUN_NAN;
        break;
      }
      float inv = 1.f / prob.x;
      inv = fmaf(-inv * inv, prob.y, inv);
      group_sync(TPR, group);
      const bool dead = (mask & kDead) != 0u;
      const float half = dead ? inv : 0.5f * inv;
      float2 *hk = hist + (int64_t)k * Cfg::N;
      for (int e = tid; e < NB; e += TPR) {
        const uint32_t r = (uint32_t)e >> (W - 1), c = (uint32_t)e & (H - 1);
        const uint32_t r0 = ins_bit(r, p, 0), r1 = ins_bit(r, p, 1);
        const uint32_t c0 = ins_bit(c, p, 0), c1 = ins_bit(c, p, 1);
        const float2 x00 = rho[r0 * D + c0], x01 = rho[r0 * D + c1];
        const float2 x10 = rho[r1 * D + c0], x11 = rho[r1 * D + c1];
        hk[r0 * D + c0] = x00;
        hk[r0 * D + c1] = x01;
        hk[r1 * D + c0] = x10;
        hk[r1 * D + c1] = x11;
        const float sr = G.x * x00.x + G.y * x11.x + G.z * (x01.x + x10.x) - G.w * (x01.y - x10.y);
        const float si = G.x * x00.y + G.y * x11.y + G.z * (x01.y + x10.y) + G.w * (x01.x - x10.x);
        const float2 s = make_float2(sr * half, si * half);
        if (dead) {
          rho[r0 * D + c0] = s;
          rho[r0 * D + c1] = make_float2(0.f, 0.f);
          rho[r1 * D + c0] = make_float2(0.f, 0.f);
          rho[r1 * D + c1] = make_float2(0.f, 0.f);
        } else {
          const uint32_t pr = (__popc(r1 & mask) & 1u) << 31, pc = (__popc(c1 & mask) & 1u) << 31;
          rho[r0 * D + c0] = s;
          rho[r0 * D + c1] = flip_sign(s, pc);
          rho[r1 * D + c0] = flip_sign(s, pr);
          rho[r1 * D + c1] = flip_sign(s, pr ^ pc);
        }
      }
      group_sync(TPR, group);
    }
    if (st_code != MBQC_RUN_OK) {
      if (tid == 0 && F0.status) F0.status[run] = st_code;
      if (A.grad)
        for (int ai = tid; ai < C.n_angles; ai += TPR) A.grad[run * A.grad_stride + ai] = NAN;
      continue;
    }
    // output noise on each output qubit
    auto depolarise = [&](int p) {
      for (int e = tid; e < NB; e += TPR) {
        const uint32_t r = (uint32_t)e >> (W - 1), c = (uint32_t)e & (H - 1);
        const uint32_t r0 = ins_bit(r, p, 0), r1 = ins_bit(r, p, 1);
        const uint32_t c0 = ins_bit(c, p, 0), c1 = ins_bit(c, p, 1);
        const float2 x00 = rho[r0 * D + c0], x01 = rho[r0 * D + c1];
        const float2 x10 = rho[r1 * D + c0], x11 = rho[r1 * D + c1];
        const float2 tr = make_float2(x00.x + x11.x, x00.y + x11.y);
        rho[r0 * D + c0] = make_float2(a_n * x00.x + b_n * tr.x, a_n * x00.y + b_n * tr.y);
        rho[r1 * D + c1] = make_float2(a_n * x11.x + b_n * tr.x, a_n * x11.y + b_n * tr.y);
        rho[r0 * D + c1] = make_float2(a_n * x01.x, a_n * x01.y);
        rho[r1 * D + c0] = make_float2(a_n * x10.x, a_n * x10.y);
      }
      group_sync(TPR, group);
    };
    if (F0.noise != 0.0)
      for (int j = 0; j < C.n_out; ++j) depolarise(C.out_bits[j]);
    // output, and Re<Gamma|rho_out>
    const int dout = 1 << C.n_out;
    const float2 *gam = A.grad_out + run * A.gout_stride;
    float zpart = 0.f;
    for (int e = tid; e < Cfg::N; e += TPR) {
      const int i = e >> W, j = e & (D - 1);
      const int yi = __ldg(&map[i]).y, yj = __ldg(&map[j]).y;
      if (yi >= 0 && yj >= 0) {
        const float2 x = rho[e], g = gam[yi * dout + yj];
        zpart += g.x * x.x + g.y * x.y;
        if (F0.rho_out) F0.rho_out[run * F0.out_stride + yi * dout + yj] = x;
      }
    }
    const float2 zp = group_sum2<TPR>(zpart, sRed, tid, group);
    const float z = zp.x + zp.y;
    // seed Lambda = Gamma - z I on the output subspace
    for (int e = tid; e < Cfg::N; e += TPR) {
      const int i = e >> W, j = e & (D - 1);
      const int yi = __ldg(&map[i]).y, yj = __ldg(&map[j]).y;
      float2 l = make_float2(0.f, 0.f);
      if (yi >= 0 && yj >= 0) {
        l = gam[yi * dout + yj];
        if (yi == yj) l.x -= z;
      }
      rho[e] = l;
    }
    group_sync(TPR, group);
    if (F0.noise != 0.0)
      for (int j = C.n_out - 1; j >= 0; --j) depolarise(C.out_bits[j]);

    // ---------------------------------------------------------- backward
    for (int k = M - 1; k >= 0; --k) {
      const int p = k % W;
      const uint32_t mask = sMask[k];
      const bool dead = (mask & kDead) != 0u;
      const float2 pk = sProb[k];
      float ck = 1.f / pk.x;
      ck = fmaf(-ck * ck, pk.y, ck);
      float4 G = sF[k], dG = sdF[k];
      if (sOut[k]) {
        const float tr_noise = a_n + 2.f * b_n;
        G = make_float4(tr_noise - G.x, tr_noise - G.y, -G.z, -G.w);
        dG = make_float4(-dG.x, -dG.y, -dG.z, -dG.w);
      }
      const float2 *hk = hist + (int64_t)k * Cfg::N;
      float gpart = 0.f;
      for (int e = tid; e < NB; e += TPR) {
        const uint32_t r = (uint32_t)e >> (W - 1), c = (uint32_t)e & (H - 1);
        const uint32_t r0 = ins_bit(r, p, 0), r1 = ins_bit(r, p, 1);
        const uint32_t c0 = ins_bit(c, p, 0), c1 = ins_bit(c, p, 1);
        float2 mu;
        if (dead) {
          mu = rho[r0 * D + c0];
        } else {
          const uint32_t pr = (__popc(r1 & mask) & 1u) << 31, pc = (__popc(c1 & mask) & 1u) << 31;
          const float2 l00 = rho[r0 * D + c0], l01 = flip_sign(rho[r0 * D + c1], pc);
          const float2 l10 = flip_sign(rho[r1 * D + c0], pr), l11 = flip_sign(rho[r1 * D + c1], pr ^ pc);
          mu = make_float2(0.5f * (l00.x + l01.x + l10.x + l11.x), 0.5f * (l00.y + l01.y + l10.y + l11.y));
        }
        const float2 x00 = hk[r0 * D + c0], x01 = hk[r0 * D + c1];
        const float2 x10 = hk[r1 * D + c0], x11 = hk[r1 * D + c1];
        // dsigma = dG00 x00 + dG11 x11 + dG01 x01 + conj(dG01) x10
        const float dr = dG.x * x00.x + dG.y * x11.x + dG.z * (x01.x + x10.x) - dG.w * (x01.y - x10.y);
        const float di = dG.x * x00.y + dG.y * x11.y + dG.z * (x01.y + x10.y) + dG.w * (x01.x - x10.x);
        gpart += mu.x * dr + mu.y * di;  // Re(conj(mu) dsigma)
        // Lambda_{k-1} = ck conj(G_xx') mu
        const float2 m = make_float2(ck * mu.x, ck * mu.y);
        rho[r0 * D + c0] = make_float2(G.x * m.x, G.x * m.y);
        rho[r1 * D + c1] = make_float2(G.y * m.x, G.y * m.y);
        rho[r0 * D + c1] = make_float2(G.z * m.x + G.w * m.y, G.z * m.y - G.w * m.x);  // conj(G01) mu
        rho[r1 * D + c0] = make_float2(G.z * m.x - G.w * m.y, G.z * m.y + G.w * m.x);  // G01 mu
      }
      const float2 gk2 = group_sum2<TPR>(gpart, sRed, tid, group);
      const float gk = gk2.x + gk2.y;
      const int ai = steps[k].aidx;
      if (tid == 0 && ai >= 0 && A.grad) A.grad[run * A.grad_stride + ai] = (double)(ck * gk);
      group_sync(TPR, group);
    }
    if (tid == 0 && F0.status) F0.status[run] = MBQC_RUN_OK;
    // angles never reached by a step keep a zero gradient
    for (int ai = tid; ai < C.n_angles; ai += TPR) {
      bool used = false;
      for (int k = 0; k < M && !used; ++k) used = steps[k].aidx == ai;
      if (!used && A.grad) A.grad[run * A.grad_stride + ai] = 0.0;
    }
  }
}

}  // namespace mbqc
