// Density-matrix sweep with the window's density matrix in factored form.
//
// After step k the window bit p = k mod w holds the entering qubit: |+><+|
// with CZs to its partners m_k (or |0><0| when no qubit enters, the window
// shrinking), so the full 2^w x 2^w matrix is
//     rho[x, y] = f[x_p, y_p] s(x) s(y) R[x \ p, y \ p],
//     f = 1/2 [[1, 1], [1, 1]] (|+>) or [[1, 0], [0, 0]] (|0>),
//     s(x) = (-1)^{x_p parity(x & m_k)},
// and only R, the (w-1)-qubit matrix over the other bits, is stored: a
// quarter of the memory and of the shared-memory traffic per step of the
// full matrix (w = 7: 32 KB instead of 128 KB per run), one more window
// (w = 8) within one SM's shared memory.
//
// Step k+1 measures q = (k+1) mod w with the step functional G (outcome
// projector transposed, depolarising noise folded in, as dm.cuh):
//     new[(u,a'), (v,b')] = f[a',b'] (-1)^{a' pi(u) + b' pi(v)} T_{a'b'}(u, v),
//     T_{a'b'}(u, v) = sum_{a,b} G[a,b] (-1)^{(a' a + b' b) m_q} R[(u,a), (v,b)],
// where (u, a) is the index with bit q = a (u: the bits other than p, q),
// (u, a') the index with bit p = a', pi(u) = parity(u & m_k) and m_q = bit q
// of m_k.  new / prob is the next R, stored over the bits other than q: bit
// p takes over the storage position that bit q had, so the pass is in place
// over the 2x2 blocks of that position, like the full-matrix kernel's pass
// (np_simulator_dm.py:307-346 + state_ops.py:77-119 for the measurement and
// trace, np_simulator_dm.py:151-216 for the |+> and CZs).  Step 0 forms R
// from the initial pure window state directly.
#pragma once

#include "dm.cuh"

namespace mbqc {

// Windows up to 8 keep R in shared memory; windows 9..11 (R of 512 KB to
// 8 MB) keep it in a device workspace, one 1024-thread block per run.
constexpr int kDmFactSmemMaxWindow = 8;
constexpr int kDmFactMaxWindow = 11;

template <int W> struct DmFactCfg {
  static_assert(W >= 2 && W <= kDmFactMaxWindow, "factored density matrix: windows 2..11");
  static constexpr int D = 1 << (W - 1);  // side of R
  static constexpr int N = D * D;         // entries of R
  static constexpr int H = D / 2;         // block index range per side
  static constexpr int NB = N / 4;        // 2x2 blocks per step
  static constexpr int DW = 1 << W;       // amplitudes of the initial window
  static constexpr bool kSmemR = W <= kDmFactSmemMaxWindow;
  // threads per run: ~8 blocks each, one warp at least, a block at most
  // (1024 threads for a workspace-resident R)
  static constexpr int TPR = !kSmemR ? 1024 : (NB / 8 < 32 ? 32 : (NB / 8 > 256 ? 256 : NB / 8));
};

// Per-step word of the factored pass (staged once per run):
//   aux bits 0-3: storage position of the measured bit in R
//       bit 4: m_q (the previous entering qubit has a CZ to the measured one)
//       bit 5: the previous step's slot is |0> (no qubit entered)
//       bit 6: Z-basis step
//   sgn: the previous entering qubit's CZ partners other than the measured
//        bit, as storage positions of R
constexpr uint32_t kFactMq = 1u << 4, kFactDead = 1u << 5, kFactZ = 1u << 6;

// bytes of one run's shared-memory slice (16-byte aligned): R (when it is
// shared-memory resident), the initial window, the step tables, the
// reduction scratch (one entry per warp of the group) and the position table
template <int W> __host__ __device__ constexpr size_t dm_fact_slice_bytes(int maxm) {
  return ((DmFactCfg<W>::kSmemR ? (size_t)DmFactCfg<W>::N * 8 : 0) + (size_t)DmFactCfg<W>::DW * 8 +
          (size_t)maxm * 24 + 64 * 8 + 16 + 15) &
         ~(size_t)15;
}

// Column swizzle of R's rows (float2 index within a row): columns 16..31 of
// every 32 are stored with bits 1..3 flipped.  In a pass over storage
// position 1, 2 or 3 the eight threads of a 16-byte access phase touch the
// even (or odd) float4 slots of 16 consecutive ones, which without the
// swizzle fall on four banks twice (a two-way conflict on every access);
// flipping the slot's low three bits in the upper half of each 16 makes the
// eight slots distinct modulo 8.  Positions 0, 4, 5 touch 8 consecutive
// slots and stay conflict free.  A column pair (c, c + 1), c even, stays one
// float4.
__device__ __forceinline__ uint32_t rsw(uint32_t col) { return col ^ (((col >> 4) & 1u) * 14u); }

// group_sum2 with a double-buffered scratch: one barrier a call.  ``par``
// alternates between calls; a buffer is written again only two calls later,
// after a barrier that every reader of its previous contents has passed.
template <int TPR>
__device__ __forceinline__ float2 group_sum2_db(float v, float2 *scratch, int tid, int group, int &par) {
  float hi = v, lo = 0.f;
#pragma unroll
  for (int o = 16; o >= 1; o >>= 1) {
    const float oh = __shfl_xor_sync(0xffffffffu, hi, o);
    const float ol = __shfl_xor_sync(0xffffffffu, lo, o);
    two_sum_acc(hi, lo, oh, ol);
  }
  if constexpr (TPR != 32) {
    constexpr int NW = TPR / 32;
    float2 *buf = scratch + par * 32;
    par ^= 1;
    if ((tid & 31) == 0) buf[tid >> 5] = make_float2(hi, lo);
    group_sync(TPR, group);
    float2 p = buf[0];
    hi = p.x;
    lo = p.y;
#pragma unroll
    for (int i = 1; i < NW; ++i) {
      p = buf[i];
      two_sum_acc(hi, lo, p.x, p.y);
    }
  }
  const float s = hi + lo;  // renormalise
  return make_float2(s, lo - (s - hi));
}

// One run of the factored sweep by a group of TPR threads.  ``base`` is the
// group's slice of shared memory; every thread of the group calls this with
// the same slot.
template <int W, int TPR>
__device__ __forceinline__ void dm_fact_run(const DmArgs &A, int64_t slot, int tid, int group,
                                            unsigned char *base, float2 *R_ws = nullptr) {
  using Cfg = DmFactCfg<W>;
  constexpr int D = Cfg::D, N = Cfg::N, H = Cfg::H, NB = Cfg::NB, DW = Cfg::DW;
  float2 *R = Cfg::kSmemR ? reinterpret_cast<float2 *>(base) : R_ws;
  float2 *psi = reinterpret_cast<float2 *>(base) + (Cfg::kSmemR ? N : 0);
  float4 *sF = reinterpret_cast<float4 *>(psi + DW);
  uint2 *sSt = reinterpret_cast<uint2 *>(sF + A.maxm);
  float2 *sRed = reinterpret_cast<float2 *>(sSt + A.maxm);  // 2 x 32 entries (one per warp of the group)
  int8_t *sPos = reinterpret_cast<int8_t *>(sRed + 64);     // [W] storage position of each window bit
  int red_par = 0;

  const int ci = A.run_circuit ? A.run_circuit[slot] : 0;
  const int64_t run = A.run_circuit ? (int64_t)ci : slot;
  const DevCircuit &C = A.circ[ci];
  const int M = C.n_steps;
  const DevStep *steps = A.steps + C.step_off;
  if (C.w != W || M > A.maxm || M < 1 || C.map_off < 0 || !(steps[M - 1].mask & kDead)) {
    if (tid == 0 && A.status) A.status[run] = MBQC_RUN_NAN;  // the host routes such plans elsewhere
    return;
  }
  const int2 *map = A.maps + C.map_off;
  const double *ang = A.angles + run * A.astride;
  const float qn = f64_to_f32_rn(A.noise);
  const float a_n = 1.f - (4.f / 3.f) * qn, b_n = (2.f / 3.f) * qn;

  // ---- stage the step functionals (noise folded in) and the position table
  for (int k = tid; k < M; k += TPR) {
    const DevStep st = steps[k];
    const double th = st.aidx >= 0 ? ang[st.aidx] : st.fixed;
    float nx, ny, nz;
    bloch(st.plane, th, nx, ny, nz);
    sF[k] = make_float4(a_n * 0.5f * (1.f + nz) + b_n, a_n * 0.5f * (1.f - nz) + b_n, a_n * 0.5f * nx,
                        a_n * 0.5f * ny);
  }
  if (tid == 0) {
    int8_t pos_of[W];
    pos_of[0] = -1;  // after step 0 bit 0 is the fresh slot; bit b > 0 is stored at position b - 1
#pragma unroll
    for (int b = 1; b < W; ++b) pos_of[b] = (int8_t)(b - 1);
    int p = 0;
    uint32_t pmask = steps[0].mask;
    sSt[0] = make_uint2(steps[0].plane == MBQC_PLANE_Z ? kFactZ : 0u, 0u);
    for (int k = 1; k < M; ++k) {
      const int q = k % W;
      const int pos = pos_of[q];
      const bool dead = (pmask & kDead) != 0u;
      uint32_t aux = (uint32_t)pos, sgn = 0u;
      if (dead) {
        aux |= kFactDead;
      } else {
        if ((pmask >> q) & 1u) aux |= kFactMq;
#pragma unroll
        for (int b = 0; b < W; ++b)
          if (b != p && b != q && ((pmask >> b) & 1u)) sgn |= 1u << pos_of[b];
      }
      const DevStep st = steps[k];
      if (st.plane == MBQC_PLANE_Z) aux |= kFactZ;
      sSt[k] = make_uint2(aux, sgn);
      pos_of[p] = (int8_t)pos;
      pos_of[q] = -1;
      p = q;
      pmask = st.mask;
    }
#pragma unroll
    for (int b = 0; b < W; ++b) sPos[b] = pos_of[b];
  }
  // ---- the initial window |psi_0> (input, |+> padding, initial CZ signs)
  {
    const float2 *in = A.psi_in + (A.istride ? run * A.istride : 0);
    const float pad = exp2f(-0.5f * (float)(W - C.n_in));
    for (int i = tid; i < DW; i += TPR) {
      const int2 mi = __ldg(&map[i]);
      const float2 u = flip_sign(in[mi.x & 0x7fffffff], (uint32_t)mi.x & 0x80000000u);
      psi[i] = make_float2(pad * u.x, pad * u.y);
    }
  }
  group_sync(TPR, group);

  int32_t st_code = MBQC_RUN_OK;
  const float tr_noise = a_n + 2.f * b_n;  // functional of I after noise folding
  for (int k = 0; k < M; ++k) {
    const float4 F = sF[k];
    const uint2 ss = sSt[k];
    const bool zstep = (ss.x & kFactZ) != 0u;
    const int pos = (int)(ss.x & 15u);
    const bool mq = (ss.x & kFactMq) != 0u, pdead = (ss.x & kFactDead) != 0u;
    // 1. outcome probability: trace of the contraction (diagonal blocks)
    //    step 0: from |psi_0> over bit 0; later: from R over position pos
    //    (with a |+> slot entangled to the measured qubit, the coherences of
    //    the measured qubit drop out of the trace)
    float p_re = 0.f, p_off = 0.f, t_re = 0.f;  // sums of G00 x00 + G11 x11, of 2 Re(G01 x01), of the trace
    if (k == 0) {
      for (int r = tid; r < DW / 2; r += TPR) {
        const float2 u0 = psi[2 * r], u1 = psi[2 * r + 1];
        const float q00 = u0.x * u0.x + u0.y * u0.y, q11 = u1.x * u1.x + u1.y * u1.y;
        p_re += F.x * q00 + F.y * q11;
        // x01 = psi0 conj(psi1)
        p_off += 2.f * (F.z * (u0.x * u1.x + u0.y * u1.y) - F.w * (u0.y * u1.x - u0.x * u1.y));
        t_re += q00 + q11;
      }
    } else {
      for (int r = tid; r < H; r += TPR) {
        const uint32_t i0 = ins_bit(r, pos, 0), i1 = ins_bit(r, pos, 1);
        const float2 q00 = R[i0 * D + rsw(i0)], q11 = R[i1 * D + rsw(i1)], q01 = R[i0 * D + rsw(i1)];
        p_re += F.x * q00.x + F.y * q11.x;
        p_off += 2.f * (F.z * q01.x - F.w * q01.y);
        t_re += q00.x + q11.x;
      }
    }
    const bool drop_coh = k > 0 && !pdead && mq;
    float2 prob = group_sum2_db<TPR>(drop_coh ? p_re : p_re + p_off, sRed, tid, group, red_par);
    float4 G = F;
    int outcome = 0;
    bool take1 = false;
    bool unprojected = false;
    if (zstep) {
      const float2 tot = group_sum2_db<TPR>(t_re, sRed, tid, group, red_par);
      if (A.flags & MBQC_F_DM_EXPECTATION) {
        if (tid == 0 && A.probs)
          A.probs[run * A.ostride + k] = 1.0 - ((double)prob.x + (double)prob.y) / ((double)tot.x + (double)tot.y);
        G = make_float4(1.f, 1.f, 0.f, 0.f);
        prob = make_float2(1.f, 0.f);
        outcome = 2;
        unprojected = true;
      } else {
        take1 = !(draw_uniform(A.seed, run, k) * tot.x < prob.x);
      }
    } else {
      take1 = !pair_ge(prob, 1e-4);  // prob0 < 1e-4 (or NaN): outcome 1 (np_simulator_dm.py:335-338)
    }
    if (take1) {  // outcome 1 with P1 = I - P0
      G = make_float4(tr_noise - F.x, tr_noise - F.y, -F.z, -F.w);
      // prob1 = trace - prob0 term by term: the same sums with G
      const float p1 = drop_coh ? (tr_noise * t_re - p_re) : (tr_noise * t_re - p_re - p_off);
      const float2 prob1 = group_sum2_db<TPR>(p1, sRed, tid, group, red_par);
      if (tid == 0 && A.probs) A.probs[run * A.ostride + k] = (double)prob.x + (double)prob.y;
      prob = prob1;
      outcome = 1;
    } else if (tid == 0 && A.probs && !unprojected) {
      A.probs[run * A.ostride + k] = (double)prob.x + (double)prob.y;
    }
    if (tid == 0 && A.outcomes) A.outcomes[run * A.ostride + k] = (int8_t)outcome;
    if (!(prob.x > 0.f) || isnan(prob.x) || isinf(prob.x)) {  // the reference's NaN check
      st_code = MBQC_RUN_NAN;
      break;
    }
    float inv = __frcp_rn(prob.x);        // correctly rounded 1/hi
    inv = fmaf(-inv * inv, prob.y, inv);  // 1/(hi + lo) to first order in lo
    // G01 as the coefficient of x01; x10 takes its conjugate
    const float g00 = G.x, g11 = G.y, gr = G.z, gi = G.w;
    if (k == 0) {
      // R = (1/prob) sum_{a,b} G[a,b] psi(x', a) conj(psi(y', b)) over bits 1..w-1
      for (int e = tid; e < N; e += TPR) {
        const int x = e / D, y = e % D;
        const float2 u0 = psi[2 * x], u1 = psi[2 * x + 1], v0 = psi[2 * y], v1 = psi[2 * y + 1];
        // x_ab = psi(x,a) conj(psi(y,b))
        const float2 x00 = make_float2(u0.x * v0.x + u0.y * v0.y, u0.y * v0.x - u0.x * v0.y);
        const float2 x11 = make_float2(u1.x * v1.x + u1.y * v1.y, u1.y * v1.x - u1.x * v1.y);
        const float2 x01 = make_float2(u0.x * v1.x + u0.y * v1.y, u0.y * v1.x - u0.x * v1.y);
        const float2 x10 = make_float2(u1.x * v0.x + u1.y * v0.y, u1.y * v0.x - u1.x * v0.y);
        const float sr = g00 * x00.x + g11 * x11.x + gr * (x01.x + x10.x) - gi * (x01.y - x10.y);
        const float si = g00 * x00.y + g11 * x11.y + gr * (x01.y + x10.y) + gi * (x01.x - x10.x);
        R[x * D + rsw((uint32_t)y)] = make_float2(sr * inv, si * inv);
      }
      group_sync(TPR, group);
      continue;
    }
    // every thread has read the diagonal before it changes: the barrier of the
    // probability sum above follows each thread's reads (a warp-sized group
    // syncs here)
    if constexpr (TPR == 32) group_sync(TPR, group);
    // 2. one in-place pass over the 2x2 blocks of position pos, the scale
    //    folded into the functional.  16-byte shared-memory accesses: at pos
    //    0 a block's two columns are adjacent (one float4 per row); at pos > 0
    //    a unit is the two blocks of columns c0 and c0 + 1 (one float4 per
    //    row and column half).  A thread keeps one column (pair) for the
    //    whole pass and walks rows, so its column index, signs and the
    //    row-independent address parts are computed once; all loads of U
    //    units before their stores (distinct units never alias).
    const uint32_t sgn = ss.y;
    const float half = pdead ? inv : 0.5f * inv;
    const float hA = g00 * half, hB = g11 * half, hR = gr * half, hI = gi * half;
    // outputs of one block from its entries x_ab (a: row half, b: column half)
    auto combine = [&](float2 x00, float2 x01, float2 x10, float2 x11, uint32_t pr, uint32_t pc, float2 &o00,
                       float2 &o01, float2 &o10, float2 &o11) {
      // sA = G00 x00 + G11 x11, dA = G00 x00 - G11 x11 (a == b terms)
      const float px = hA * x00.x, py = hA * x00.y;
      const float2 sA = make_float2(fmaf(hB, x11.x, px), fmaf(hB, x11.y, py));
      // sB = G01 x01 + conj(G01) x10 (a != b terms), dB = conj(G01) x10 - G01 x01
      const float2 u = make_float2(x01.x + x10.x, x01.y + x10.y), v = make_float2(x01.x - x10.x, x01.y - x10.y);
      const float2 sB = make_float2(fmaf(hR, u.x, -hI * v.y), fmaf(hR, u.y, hI * v.x));
      o00 = make_float2(sA.x + sB.x, sA.y + sB.y);
      if (pdead) {
        o01 = o10 = o11 = make_float2(0.f, 0.f);
      } else if (!mq) {
        o01 = flip_sign(o00, pc);
        o10 = flip_sign(o00, pr);
        o11 = flip_sign(o00, pr ^ pc);
      } else {
        // signs (-1)^{a' a + b' b} on the terms: T01 = dA + dB, T10 = dA - dB, T11 = sA - sB
        const float2 dA = make_float2(fmaf(-hB, x11.x, px), fmaf(-hB, x11.y, py));
        const float2 dB = make_float2(fmaf(hI, u.y, -hR * v.x), fmaf(-hI, u.x, -hR * v.y));
        o01 = flip_sign(make_float2(dA.x + dB.x, dA.y + dB.y), pc);
        o10 = flip_sign(make_float2(dA.x - dB.x, dA.y - dB.y), pr);
        o11 = flip_sign(make_float2(sA.x - sB.x, sA.y - sB.y), pr ^ pc);
      }
    };
    float4 *R4 = reinterpret_cast<float4 *>(R);
    if (pos == 0) {
      // H columns of blocks; thread tid: column tid % H, rows tid / H + j * (TPR / H)
      constexpr int CPT = H < TPR ? H : TPR;  // threads per row of blocks
      constexpr int RSTEP = TPR / CPT, NJ = (H + RSTEP - 1) / RSTEP;
      constexpr int U = NJ >= 4 ? 4 : NJ;
      const uint32_t c = (uint32_t)(tid % CPT), r_first = (uint32_t)(tid / CPT);
      for (int cc = (int)c; cc < H; cc += CPT) {  // one iteration unless H > TPR
        const uint32_t pc = (__popc((2u * (uint32_t)cc) & sgn) & 1u) << 31;
        const uint32_t ccs = rsw(2u * (uint32_t)cc) >> 1;  // the column pair's float4 slot in its row
        for (int j0 = 0; j0 < NJ; j0 += U) {
          float4 top[U], bot[U];
          uint32_t at[U], pr[U];
#pragma unroll
          for (int uu = 0; uu < U; ++uu) {
            const uint32_t r = r_first + (uint32_t)(j0 + uu) * RSTEP;
            if (r < (uint32_t)H) {
              at[uu] = r * D + ccs;  // float4 index of (row 2r, columns 2c, 2c + 1)
              pr[uu] = (__popc((2u * r) & sgn) & 1u) << 31;
              top[uu] = R4[at[uu]];
              bot[uu] = R4[at[uu] + D / 2];
            }
          }
#pragma unroll
          for (int uu = 0; uu < U; ++uu) {
            const uint32_t r = r_first + (uint32_t)(j0 + uu) * RSTEP;
            if (r < (uint32_t)H) {
              float2 o00, o01, o10, o11;
              combine(make_float2(top[uu].x, top[uu].y), make_float2(top[uu].z, top[uu].w),
                      make_float2(bot[uu].x, bot[uu].y), make_float2(bot[uu].z, bot[uu].w), pr[uu], pc, o00, o01,
                      o10, o11);
              R4[at[uu]] = make_float4(o00.x, o00.y, o01.x, o01.y);
              R4[at[uu] + D / 2] = make_float4(o10.x, o10.y, o11.x, o11.y);
            }
          }
        }
      }
    } else if constexpr (W >= 3) {  // window 2 has position 0 only
      // H/2 column pairs; thread tid: pair tid % HU, rows tid / HU + j * (TPR / HU)
      constexpr int HU = H / 2;
      constexpr int CPT = HU < TPR ? HU : TPR;
      constexpr int RSTEP = TPR / CPT, NJ = (H + RSTEP - 1) / RSTEP;
      constexpr int U = NJ >= 2 ? 2 : NJ;
      const uint32_t rs = ((uint32_t)D << pos) >> 1;  // row step in float4
      const uint32_t r_first = (uint32_t)(tid / CPT);
      for (int cp = tid % CPT; cp < HU; cp += CPT) {  // one iteration unless HU > TPR
        const uint32_t c0 = ins_bit(2u * (uint32_t)cp, pos, 0);  // even
        const uint32_t pc0 = (__popc(c0 & sgn) & 1u) << 31, pc1 = (__popc((c0 + 1u) & sgn) & 1u) << 31;
        // float4 slots of the column pairs (c0, c0 + 1) and (c0 + 2^pos, c0 + 2^pos + 1) in a row
        const uint32_t s0 = rsw(c0) >> 1, s1 = rsw(c0 | (1u << pos)) >> 1;
        for (int j0 = 0; j0 < NJ; j0 += U) {
          float4 q00[U], q01[U], q10[U], q11[U];
          uint32_t at[U], pr[U];
#pragma unroll
          for (int uu = 0; uu < U; ++uu) {
            const uint32_t r = r_first + (uint32_t)(j0 + uu) * RSTEP;
            if (r < (uint32_t)H) {
              const uint32_t r0 = ins_bit(r, pos, 0);
              at[uu] = (r0 * D) >> 1;  // float4 index of row r0
              pr[uu] = (__popc(r0 & sgn) & 1u) << 31;
              q00[uu] = R4[at[uu] + s0];
              q01[uu] = R4[at[uu] + s1];
              q10[uu] = R4[at[uu] + rs + s0];
              q11[uu] = R4[at[uu] + rs + s1];
            }
          }
#pragma unroll
          for (int uu = 0; uu < U; ++uu) {
            const uint32_t r = r_first + (uint32_t)(j0 + uu) * RSTEP;
            if (r < (uint32_t)H) {
              float2 a00, a01, a10, a11, b00, b01, b10, b11;
              combine(make_float2(q00[uu].x, q00[uu].y), make_float2(q01[uu].x, q01[uu].y),
                      make_float2(q10[uu].x, q10[uu].y), make_float2(q11[uu].x, q11[uu].y), pr[uu], pc0, a00, a01,
                      a10, a11);
              combine(make_float2(q00[uu].z, q00[uu].w), make_float2(q01[uu].z, q01[uu].w),
                      make_float2(q10[uu].z, q10[uu].w), make_float2(q11[uu].z, q11[uu].w), pr[uu], pc1, b00, b01,
                      b10, b11);
              R4[at[uu] + s0] = make_float4(a00.x, a00.y, b00.x, b00.y);
              R4[at[uu] + s1] = make_float4(a01.x, a01.y, b01.x, b01.y);
              R4[at[uu] + rs + s0] = make_float4(a10.x, a10.y, b10.x, b10.y);
              R4[at[uu] + rs + s1] = make_float4(a11.x, a11.y, b11.x, b11.y);
            }
          }
        }
      }
    }
    group_sync(TPR, group);
  }

  // ---- output noise (each output qubit once, on its storage position)
  if (st_code == MBQC_RUN_OK && qn != 0.f) {
    for (int j = 0; j < C.n_out; ++j) {
      const int pos = sPos[C.out_bits[j]];
      for (int e = tid; e < NB; e += TPR) {
        const uint32_t r = (uint32_t)e / H, c = (uint32_t)e % H;
        const uint32_t r0 = ins_bit(r, pos, 0), r1 = ins_bit(r, pos, 1);
        const uint32_t c0 = ins_bit(c, pos, 0), c1 = ins_bit(c, pos, 1);
        const uint32_t c0s = rsw(c0), c1s = rsw(c1);
        const float2 x00 = R[r0 * D + c0s], x01 = R[r0 * D + c1s];
        const float2 x10 = R[r1 * D + c0s], x11 = R[r1 * D + c1s];
        const float2 tr = make_float2(x00.x + x11.x, x00.y + x11.y);
        R[r0 * D + c0s] = make_float2(a_n * x00.x + b_n * tr.x, a_n * x00.y + b_n * tr.y);
        R[r1 * D + c1s] = make_float2(a_n * x11.x + b_n * tr.x, a_n * x11.y + b_n * tr.y);
        R[r0 * D + c1s] = make_float2(a_n * x01.x, a_n * x01.y);
        R[r1 * D + c0s] = make_float2(a_n * x10.x, a_n * x10.y);
      }
      group_sync(TPR, group);
    }
  }
  // ---- gather the outputs in the reference order: output qubit j (the
  // most significant first) sits at storage position sPos[out_bits[j]]; the
  // other stored bits are |0> slots of the shrunk window
  const int n_out = C.n_out, dout = 1 << n_out;
  int *ridx = reinterpret_cast<int *>(psi);  // psi is no longer needed
  for (int y = tid; y < dout; y += TPR) {
    int ri = 0;
    for (int j = 0; j < n_out; ++j) ri |= ((y >> (n_out - 1 - j)) & 1) << sPos[C.out_bits[j]];
    ridx[y] = ri;
  }
  group_sync(TPR, group);
  float2 *out = A.rho_out + run * A.out_stride;
  for (int e = tid; e < dout * dout; e += TPR) {
    const int yi = e >> n_out, yj = e & (dout - 1);
    out[e] = st_code == MBQC_RUN_OK ? R[ridx[yi] * D + rsw((uint32_t)ridx[yj])] : make_float2(NAN, NAN);
  }
  if (tid == 0 && A.status) A.status[run] = st_code;
  group_sync(TPR, group);  // the slice is reused by the caller's next run
}

// Windows 9..11: one 1024-thread block per run, R in the workspace (one
// slice of N complex64 per resident block), blocks looping over the runs.
template <int W>
__global__ void __launch_bounds__(1024) dm_fwd_fact_ws(DmArgs A, float2 *ws) {
  extern __shared__ __align__(16) unsigned char smem_w[];
  float2 *R = ws + (size_t)blockIdx.x * DmFactCfg<W>::N;
  for (int64_t slot = blockIdx.x; slot < A.B; slot += gridDim.x)
    dm_fact_run<W, 1024>(A, slot, threadIdx.x, 0, smem_w, R);
}

// One run per group of TPR threads, 256 / TPR runs per block.
template <int W, int TPR>
__global__ void __launch_bounds__(256, 3) dm_fwd_fact(DmArgs A) {
  extern __shared__ __align__(16) unsigned char smem_f[];
  const int group = threadIdx.x / TPR, tid = threadIdx.x % TPR;
  const int64_t slot = (int64_t)blockIdx.x * (256 / TPR) + group;
  if (slot >= A.B) return;  // whole group leaves together
  dm_fact_run<W, TPR>(A, slot, tid, group, smem_f + (size_t)group * dm_fact_slice_bytes<W>(A.maxm));
}

}  // namespace mbqc
