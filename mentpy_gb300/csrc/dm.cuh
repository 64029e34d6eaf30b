// Density-matrix sweep, windows w <= 7, rho resident in shared memory.
//
// One group of TPR threads owns one run; rho (2^w x 2^w complex64, row-major)
// lives in the group's slice of shared memory.  Step k on window bit p, with
// the outcome-0 projector P0 = (I + n.sigma)/2 of the step's plane and angle
// (ment.py:218-260):
//   1. prob0 = Re Tr(P0 rho) = sum_r sum_{x,x'} F_{xx'} rho[(x,r),(x',r)],
//      F_{xx'} = P0[x', x]; FP32 per thread, FP64 across the group.  As the
//      reference (np_simulator_dm.py:335-338): outcome 1 iff prob0 < 1e-4,
//      then the same with P1 = I - P0.
//   2. one in-place pass over the 4^(w-1) 2x2 blocks (r, r') on bit p:
//        sigma = sum_{x,x'} F_{xx'} rho[(x,r),(x',r')] / prob
//      (= Tr_p(P rho P)/prob, np_simulator_dm.py:341-344 + state_ops.py:77-119)
//      and the entering |+><+| with its CZ signs:
//        rho'[(b,r),(b',r')] = sigma s_b(r) s_b'(r') / 2
//      or rho'[(0,r),(0,r')] = sigma when no qubit enters.
// Depolarising noise of strength q on the measured qubit just before it is
// measured folds into the functional: F -> (1 - 4q/3) F + (2q/3) I.  Output
// qubits are depolarised once after the sweep.
#pragma once

#include "common.cuh"

namespace mbqc {

struct DmArgs {
  const DevCircuit *circ;     // plan table
  const DevStep *steps;
  const int2 *maps;           // all index maps (circuit map_off into it)
  const int32_t *run_circuit; // [B] circuit of each run, NULL = circuit 0
  int64_t B;
  const double *angles;
  int64_t astride;
  const float2 *psi_in;       // pure input states
  int64_t istride;            // 0 = broadcast row 0
  float2 *rho_out;            // [B, out_stride]
  int64_t out_stride;         // complex elements per run (>= 4^n_out)
  double noise;               // depolarising strength, 0 = none
  int8_t *outcomes;           // [B, ostride] or NULL
  int64_t ostride;
  double *probs;              // [B, ostride] prob0 per step, or NULL
  int32_t *status;
  int maxm;                   // staged steps per run (>= every circuit's n_steps)
  uint32_t flags;             // MBQC_F_DM_EXPECTATION: Z steps are not projected
  uint64_t seed;              // outcome draws of Z steps in sample mode
};

// Staged step mask bit: the step measures in the Z basis (the reference
// draws its outcome, or in expectation mode records prob1 / (prob0 + prob1)
// and does not project, np_simulator_dm.py:327-344).
constexpr uint32_t kZStep = 1u << 30;

// SplitMix64 (Steele, Lea and Flood 2014) as a counter-based generator: a
// uniform float in [0, 1) for (seed, run, step), the same on every thread.
__device__ __forceinline__ uint64_t splitmix64(uint64_t z) {
  z += 0x9e3779b97f4a7c15ull;
  z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
  z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
  return z ^ (z >> 31);
}
__device__ __forceinline__ float draw_uniform(uint64_t seed, int64_t run, int step) {
  const uint64_t h = splitmix64(seed ^ splitmix64(((uint64_t)run << 20) ^ (uint64_t)step));
  return (float)(h >> 40) * 5.9604644775390625e-08f;  // 24 bits / 2^24
}

template <int W> struct DmCfg {
  static constexpr int D = 1 << W;
  static constexpr int N = D * D;                 // entries of rho
  static constexpr int NB = N / 4;                // 2x2 blocks per step
  static constexpr int TPR = NB / 8 < 32 ? 32 : (NB / 8 > 256 ? 256 : NB / 8);
  static constexpr int GROUPS = 256 / TPR;        // runs per 256-thread block
};

// bytes before the reduction scratch (8-byte aligned)
template <int W> __host__ __device__ constexpr size_t dm_smem_head(int maxm) {
  return (((size_t)DmCfg<W>::GROUPS *
               ((size_t)DmCfg<W>::N * sizeof(float2) + (size_t)maxm * (sizeof(float4) + sizeof(uint32_t))) +
           7) &
          ~(size_t)7);
}

__device__ __forceinline__ void group_sync(int tpr, int group) {
  if (tpr == 32) {
    __syncwarp();
  } else if (tpr == (int)blockDim.x) {
    __syncthreads();
  } else {
    asm volatile("bar.sync %0, %1;" ::"r"(group + 1), "r"(tpr) : "memory");
  }
}

// sum of one double over the group (all threads get the result)
template <int TPR>
__device__ __forceinline__ double group_sum(double v, double *scratch, int tid, int group) {
#pragma unroll
  for (int o = 16; o >= 1; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  if constexpr (TPR == 32) {
    return v;
  } else {
    constexpr int NW = TPR / 32;
    group_sync(TPR, group);
    if ((tid & 31) == 0) scratch[tid >> 5] = v;
    group_sync(TPR, group);
    double s = 0.0;
#pragma unroll
    for (int i = 0; i < NW; ++i) s += scratch[i];
    return s;
  }
}

// Sum of one float over the group as an unevaluated pair hi + lo (error-free
// two-sum at every addition: ~48-bit significand, FP64-level accuracy, on
// the FP32 pipe -- GB300's FP64 pipe runs at a small fraction of the FP32
// rate and a per-step FP64 reduction sits on every run's critical path).  All
// threads get the same bits (xor butterfly, then the same serial order over
// the group's warps).
template <int TPR>
__device__ __forceinline__ float2 group_sum2(float v, float2 *scratch, int tid, int group) {
  float hi = v, lo = 0.f;
#pragma unroll
  for (int o = 16; o >= 1; o >>= 1) {
    const float oh = __shfl_xor_sync(0xffffffffu, hi, o);
    const float ol = __shfl_xor_sync(0xffffffffu, lo, o);
    two_sum_acc(hi, lo, oh, ol);
  }
  if constexpr (TPR != 32) {
    constexpr int NW = TPR / 32;
    group_sync(TPR, group);
    if ((tid & 31) == 0) scratch[tid >> 5] = make_float2(hi, lo);
    group_sync(TPR, group);
    float2 p = scratch[0];
    hi = p.x;
    lo = p.y;
#pragma unroll
    for (int i = 1; i < NW; ++i) {
      p = scratch[i];
      two_sum_acc(hi, lo, p.x, p.y);
    }
  }
  const float s = hi + lo;  // renormalise
  return make_float2(s, lo - (s - hi));
}

// hi + lo >= t for a pair from group_sum2: decided in float unless hi is
// within 1e-6 (relative) of t, where the pair is compared in FP64
__device__ __forceinline__ bool pair_ge(float2 p, double t) {
  const float tf = (float)t;
  if (fabsf(p.x - tf) > 1e-6f * tf) return p.x > tf;
  return (double)p.x + (double)p.y >= t;
}

__device__ __forceinline__ uint32_t ins_bit(uint32_t r, int p, uint32_t b) {
  return ((r >> p) << (p + 1)) | (b << p) | (r & ((1u << p) - 1u));
}

// Bloch vector of the outcome-0 projector of a step
__device__ __forceinline__ void bloch(int plane, double theta, float &nx, float &ny, float &nz) {
  float s = 0.f, c = 1.f;
  if (plane == MBQC_PLANE_XY || plane == MBQC_PLANE_XZ || plane == MBQC_PLANE_YZ)
    sincos_reduced(reduce_angle(theta), s, c);
  nx = ny = nz = 0.f;
  switch (plane) {
    case MBQC_PLANE_XY: nx = c; ny = s; break;
    case MBQC_PLANE_X: nx = 1.f; break;
    case MBQC_PLANE_Y: ny = 1.f; break;
    case MBQC_PLANE_XZ: nx = c; nz = s; break;
    case MBQC_PLANE_Z: nz = 1.f; break;
    default: ny = c; nz = s; break;  // YZ
  }
}

template <int W>
__global__ void __launch_bounds__(256) dm_fwd_smem(DmArgs A) {
  using Cfg = DmCfg<W>;
  constexpr int D = Cfg::D, TPR = Cfg::TPR, NB = Cfg::NB, H = D / 2;
  extern __shared__ __align__(16) unsigned char smem[];
  const int group = threadIdx.x / TPR, tid = threadIdx.x % TPR;
  // carve-up: [GROUPS][N] rho | [GROUPS][maxm] F | [GROUPS][maxm] masks | [GROUPS][8] reduction
  float2 *rho = reinterpret_cast<float2 *>(smem) + (size_t)group * Cfg::N;
  float4 *sF = reinterpret_cast<float4 *>(smem + (size_t)Cfg::GROUPS * Cfg::N * sizeof(float2)) +
               (size_t)group * A.maxm;
  uint32_t *sMask = reinterpret_cast<uint32_t *>(smem + (size_t)Cfg::GROUPS * Cfg::N * sizeof(float2) +
                                                 (size_t)Cfg::GROUPS * A.maxm * sizeof(float4)) +
                    (size_t)group * A.maxm;
  float2 *sRed = reinterpret_cast<float2 *>(smem + dm_smem_head<W>(A.maxm)) + (size_t)group * 8;

  const int64_t slot = (int64_t)blockIdx.x * Cfg::GROUPS + group;
  if (slot >= A.B) return;  // whole group leaves together
  // with a circuit list, slot b simulates circuit run_circuit[b] and every
  // per-run array is indexed by that circuit
  const int ci = A.run_circuit ? A.run_circuit[slot] : 0;
  const int64_t run = A.run_circuit ? (int64_t)ci : slot;
  const DevCircuit &C = A.circ[ci];
  const int M = C.n_steps;
  if (C.w != W || M > A.maxm || C.map_off < 0) {  // launch grouped runs of another window
    if (tid == 0 && A.status) A.status[run] = MBQC_RUN_NAN;
    return;
  }
  const DevStep *steps = A.steps + C.step_off;
  const int2 *map = A.maps + C.map_off;
  const double *ang = A.angles + run * A.astride;
  const float qn = f64_to_f32_rn(A.noise);
  const float a_n = 1.f - (4.f / 3.f) * qn, b_n = (2.f / 3.f) * qn;

  // ---- stage the run's step functionals F = P0^T (noise folded in)
  for (int k = tid; k < M; k += TPR) {
    const DevStep st = steps[k];
    const double th = st.aidx >= 0 ? ang[st.aidx] : st.fixed;
    float nx, ny, nz;
    bloch(st.plane, th, nx, ny, nz);
    // F00 = (1+nz)/2, F11 = (1-nz)/2, F01 = P0[1][0] = (nx + i ny)/2
    sF[k] = make_float4(a_n * 0.5f * (1.f + nz) + b_n, a_n * 0.5f * (1.f - nz) + b_n, a_n * 0.5f * nx,
                        a_n * 0.5f * ny);
    sMask[k] = st.mask | (st.plane == MBQC_PLANE_Z ? kZStep : 0u);
  }
  // ---- rho_0 = |psi_0><psi_0| (input, |+> padding, initial CZ signs)
  {
    const float2 *in = A.psi_in + (A.istride ? run * A.istride : 0);
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

  int32_t st_code = MBQC_RUN_OK;
  for (int k = 0; k < M; ++k) {
    const int p = k % W;
    const float4 F = sF[k];
    const uint32_t mask = sMask[k];
    const bool zstep = (mask & kZStep) != 0u;
    // 1. outcome probabilities from the diagonal blocks
    float part = 0.f, part_t = 0.f;
    for (int r = tid; r < H; r += TPR) {
      const uint32_t r0 = ins_bit(r, p, 0), r1 = ins_bit(r, p, 1);
      const float2 q00 = rho[r0 * D + r0], q11 = rho[r1 * D + r1], q01 = rho[r0 * D + r1];
      // F01 rho01 + F10 rho10 = 2 Re(F01 rho01) for Hermitian rho
      part += F.x * q00.x + F.y * q11.x + 2.f * (F.z * q01.x - F.w * q01.y);
      part_t += q00.x + q11.x;
    }
    float2 prob = group_sum2<TPR>(part, sRed, tid, group);
    float4 G = F;
    int outcome = 0;
    bool take1;
    bool unprojected = false;
    if (zstep) {
      const float2 tot = group_sum2<TPR>(part_t, sRed, tid, group);
      if (A.flags & MBQC_F_DM_EXPECTATION) {
        // no projection: the qubit is traced out (identity functional), the
        // recorded outcome is prob1 / (prob0 + prob1)
        if (tid == 0 && A.probs)
          A.probs[run * A.ostride + k] =
              1.0 - ((double)prob.x + (double)prob.y) / ((double)tot.x + (double)tot.y);
        G = make_float4(1.f, 1.f, 0.f, 0.f);
        prob = make_float2(1.f, 0.f);  // no renormalisation
        outcome = 2;
        unprojected = true;
        take1 = false;
      } else {
        take1 = !(draw_uniform(A.seed, run, k) * tot.x < prob.x);
      }
    } else {
      take1 = !pair_ge(prob, 1e-4);  // prob0 < 1e-4 (or NaN): outcome 1
    }
    if (take1) {  // outcome 1 with P1 = I - P0
      const float tr_noise = a_n + 2.f * b_n;  // functional of I after noise folding
      G = make_float4(tr_noise - F.x, tr_noise - F.y, -F.z, -F.w);
      float part1 = 0.f;
      for (int r = tid; r < H; r += TPR) {
        const uint32_t r0 = ins_bit(r, p, 0), r1 = ins_bit(r, p, 1);
        const float2 q00 = rho[r0 * D + r0], q11 = rho[r1 * D + r1], q01 = rho[r0 * D + r1];
        part1 += G.x * q00.x + G.y * q11.x + 2.f * (G.z * q01.x - G.w * q01.y);
      }
      const float2 prob1 = group_sum2<TPR>(part1, sRed, tid, group);
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
    float inv = 1.f / prob.x;
    inv = fmaf(-inv * inv, prob.y, inv);  // 1/(hi + lo) to first order in lo
    group_sync(TPR, group);  // every thread has read the diagonal before it changes
    // 2. contraction + expansion, one pass over the 2x2 blocks
    const bool dead = (mask & kDead) != 0u;
    const float half = dead ? inv : 0.5f * inv;
    // U blocks per thread at a time: all loads before any store (distinct
    // blocks never alias), so shared-memory latency overlaps
    constexpr int ITER = (NB + TPR - 1) / TPR;
    constexpr int U = ITER >= 4 ? 4 : ITER;
    for (int it = 0; it < ITER; it += U) {
      uint32_t a00[U], a01[U], a10[U], a11[U];
      float2 x00[U], x01[U], x10[U], x11[U];
      uint32_t pr[U], pc[U];
#pragma unroll
      for (int u = 0; u < U; ++u) {
        const int e = tid + (it + u) * TPR;
        if (e < NB) {
          const uint32_t r = (uint32_t)e >> (W - 1), c = (uint32_t)e & (H - 1);
          const uint32_t r0 = ins_bit(r, p, 0), r1 = ins_bit(r, p, 1);
          const uint32_t c0 = ins_bit(c, p, 0), c1 = ins_bit(c, p, 1);
          a00[u] = r0 * D + c0;
          a01[u] = r0 * D + c1;
          a10[u] = r1 * D + c0;
          a11[u] = r1 * D + c1;
          pr[u] = (__popc(r1 & mask) & 1u) << 31;
          pc[u] = (__popc(c1 & mask) & 1u) << 31;
          x00[u] = rho[a00[u]];
          x01[u] = rho[a01[u]];
          x10[u] = rho[a10[u]];
          x11[u] = rho[a11[u]];
        }
      }
#pragma unroll
      for (int u = 0; u < U; ++u) {
        const int e = tid + (it + u) * TPR;
        if (e < NB) {
          // sigma = G00 x00 + G11 x11 + G01 x01 + conj(G01) x10
          float sr = G.x * x00[u].x + G.y * x11[u].x + G.z * (x01[u].x + x10[u].x) - G.w * (x01[u].y - x10[u].y);
          float si = G.x * x00[u].y + G.y * x11[u].y + G.z * (x01[u].y + x10[u].y) + G.w * (x01[u].x - x10[u].x);
          const float2 s = make_float2(sr * half, si * half);
          if (dead) {
            rho[a00[u]] = s;
            rho[a01[u]] = make_float2(0.f, 0.f);
            rho[a10[u]] = make_float2(0.f, 0.f);
            rho[a11[u]] = make_float2(0.f, 0.f);
          } else {
            rho[a00[u]] = s;
            rho[a01[u]] = flip_sign(s, pc[u]);
            rho[a10[u]] = flip_sign(s, pr[u]);
            rho[a11[u]] = flip_sign(s, pr[u] ^ pc[u]);
          }
        }
      }
    }
    group_sync(TPR, group);
  }

  // ---- output noise (each output qubit once), gather in the reference order
  if (st_code == MBQC_RUN_OK && qn != 0.f) {
    for (int j = 0; j < C.n_out; ++j) {
      const int p = C.out_bits[j];
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
    }
  }
  float2 *out = A.rho_out + run * A.out_stride;
  const int dout = 1 << C.n_out;
  for (int e = tid; e < Cfg::N; e += TPR) {
    const int i = e >> W, j = e & (D - 1);
    const int yi = __ldg(&map[i]).y, yj = __ldg(&map[j]).y;
    if (yi >= 0 && yj >= 0)
      out[yi * dout + yj] = st_code == MBQC_RUN_OK ? rho[e] : make_float2(NAN, NAN);
  }
  if (tid == 0 && A.status) A.status[run] = st_code;
}

template <int W> __host__ __device__ constexpr size_t dm_smem_bytes(int maxm) {
  return dm_smem_head<W>(maxm) + (size_t)DmCfg<W>::GROUPS * 8 * sizeof(double);
}

}  // namespace mbqc
