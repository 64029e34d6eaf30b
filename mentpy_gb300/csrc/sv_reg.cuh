// Register-resident statevector sweep for windows w <= 10.
//
// A run owns L = 2^LL consecutive lanes of a warp; each lane keeps
// R = 2^(W-LL) amplitudes in registers.  Index bit b of the 2^W window is
//   b <  RB = W-LL : a register bit (slot j of the lane's array),
//   b >= RB        : lane bit b-RB of the run's lane index.
// The plan measures bit (k mod W) at step k, so one unrolled "period" of W
// steps has compile-time bit positions and register indices; plan data
// (CZ masks, angles) stay runtime.
//
// Step k on bit p with coefficient c = e^{-i theta_k} (unnormalised
// <+_theta| contraction, np_simulator_sv.py:322-358 + state_ops.py:42-74):
//     phi[r]      = psi[r, p=0] + c * psi[r, p=1]
//     psi[r, p=0] = phi[r]
//     psi[r, p=1] = (-1)^{parity(idx & mask_k)} phi[r]   (|+> and its CZs,
//                                                         np_simulator_sv.py:207-223)
// or psi[r, p=1] = 0 when no qubit enters (the window shrinks).
// A register bit pairs two slots of one lane; a lane bit pairs two lanes and
// is done as a butterfly: each lane forms its own term c_a * psi and adds the
// partner's term with one xor-shuffle.
//
// The norm is not renormalised every step: every period the run's squared
// norm is all-reduced and an exact power-of-two scale is applied one period
// later (no rounding, no dependency stall).  The exact exponents make the
// all-zero-branch log-probability a by-product.  The final norm is reduced
// across lanes in FP64.
#pragma once

#include <utility>

#include "common.cuh"

namespace mbqc {

struct SvArgs {
  const DevCircuit *circ;
  const DevStep *steps;
  const int2 *map;        // [2^w]: .x = input index | sign<<31, .y = output index or -1
  int64_t B;
  const double *angles;
  int64_t astride;
  const void *psi_in;
  int64_t istride;
  void *psi_out;
  uint32_t flags;
  double *logprob;
  int32_t *status;
};

template <typename T> struct RealBits;
template <> struct RealBits<float> {
  __device__ static int expo(float s) { return (int)((__float_as_uint(s) >> 23) & 0xffu) - 127; }
  __device__ static float pow2(int e) { return __uint_as_float((uint32_t)(127 + e) << 23); }
  __device__ static bool finite_pos(float s) { return s > 0.f && s < 3.0e38f; }
};
template <> struct RealBits<double> {
  __device__ static int expo(double s) {
    return (int)((__double_as_longlong(s) >> 52) & 0x7ff) - 1023;
  }
  __device__ static double pow2(int e) {
    return __longlong_as_double((long long)(1023 + e) << 52);
  }
  __device__ static bool finite_pos(double s) { return s > 0.0 && s < 1.0e300; }
};

template <typename T, int W, int LL> struct SvRegCfg {
  static constexpr int L = 1 << LL;
  static constexpr int RB = W - LL;
  static constexpr int R = 1 << RB;
  static constexpr int RPW = 32 / L;  // runs per warp
  static constexpr int PC = (40 / W) > 0 ? (40 / W) : 1;
  static constexpr int KC = PC * W;  // steps staged per chunk
  static_assert(LL >= 0 && LL <= 5 && RB >= 0 && RB <= 5, "register layout");
};

constexpr int kSvWarps = 4;  // warps per block (max)

// ---------------------------------------------------------------- steps
template <typename T, int R, int BIT>
__device__ __forceinline__ void reg_step(cplx<T> (&a)[R], cplx<T> c, uint32_t ts, bool dead) {
  if (dead) {
#pragma unroll
    for (int j = 0; j < R; ++j) {
      if (j & (1 << BIT)) continue;
      const int jh = j | (1 << BIT);
      const cplx<T> x0 = a[j], x1 = a[jh];
      a[j] = mk<T>(x0.x + c.x * x1.x - c.y * x1.y, x0.y + c.x * x1.y + c.y * x1.x);
      a[jh] = mk<T>(T(0), T(0));
    }
  } else {
#pragma unroll
    for (int j = 0; j < R; ++j) {
      if (j & (1 << BIT)) continue;
      const int jh = j | (1 << BIT);
      const cplx<T> x0 = a[j], x1 = a[jh];
      const cplx<T> phi = mk<T>(x0.x + c.x * x1.x - c.y * x1.y, x0.y + c.x * x1.y + c.y * x1.x);
      a[j] = phi;
      a[jh] = flip_sign(phi, (ts << (31 - jh)) & 0x80000000u);
    }
  }
}

template <typename T, int R, int Q>
__device__ __forceinline__ void lane_step(cplx<T> (&a)[R], cplx<T> c, uint32_t ts, bool dead, int li) {
  const bool hi = (li >> Q) & 1;
  const cplx<T> cm = hi ? c : mk<T>(T(1), T(0));
  const uint32_t tl = hi ? ts : 0u;
#pragma unroll
  for (int j = 0; j < R; ++j) {
    const cplx<T> m = a[j];
    const cplx<T> term = mk<T>(cm.x * m.x - cm.y * m.y, cm.x * m.y + cm.y * m.x);
    const cplx<T> phi = mk<T>(term.x + __shfl_xor_sync(0xffffffffu, term.x, 1 << Q),
                              term.y + __shfl_xor_sync(0xffffffffu, term.y, 1 << Q));
    if (dead)
      a[j] = hi ? mk<T>(T(0), T(0)) : phi;
    else
      a[j] = flip_sign(phi, (tl << (31 - j)) & 0x80000000u);
  }
}

template <typename T, int W, int LL, int BIT>
__device__ __forceinline__ void one_step(cplx<T> (&a)[SvRegCfg<T, W, LL>::R], const cplx<T> *coef,
                                         const uint32_t *smask, const uint32_t *streg, int kk,
                                         int li) {
  using Cfg = SvRegCfg<T, W, LL>;
  const uint32_t mask = smask[kk];
  const uint32_t lp = __popc(((uint32_t)li << Cfg::RB) & mask) & 1u;
  const uint32_t ts = streg[kk] ^ (0u - lp);
  const bool dead = (mask & kDead) != 0u;
  const cplx<T> c = coef[kk];
  if constexpr (BIT < Cfg::RB)
    reg_step<T, Cfg::R, BIT>(a, c, ts, dead);
  else
    lane_step<T, Cfg::R, BIT - Cfg::RB>(a, c, ts, dead, li);
}

template <typename T, int W, int LL, int... BITS>
__device__ __forceinline__ void run_period(std::integer_sequence<int, BITS...>,
                                           cplx<T> (&a)[SvRegCfg<T, W, LL>::R], const cplx<T> *coef,
                                           const uint32_t *smask, const uint32_t *streg, int p0,
                                           int kend, int li) {
  ((p0 + BITS < kend ? one_step<T, W, LL, BITS>(a, coef, smask, streg, p0 + BITS, li) : void()),
   ...);
}

// --------------------------------------------------------------- kernel
template <typename T, int W, int LL>
__global__ void __launch_bounds__(32 * kSvWarps) sv_fwd_reg(SvArgs args) {
  using Cfg = SvRegCfg<T, W, LL>;
  constexpr int L = Cfg::L, RB = Cfg::RB, R = Cfg::R, RPW = Cfg::RPW, KC = Cfg::KC;
  using CT = cplx<T>;

  __shared__ CT s_coef[kSvWarps][RPW][KC];
  __shared__ uint32_t s_mask[kSvWarps][KC];
  __shared__ uint32_t s_treg[kSvWarps][KC];

  const int lane = threadIdx.x & 31;
  const int wid = threadIdx.x >> 5;
  const int sub = lane >> LL;
  const int li = lane & (L - 1);
  const int64_t wrun0 = ((int64_t)blockIdx.x * (blockDim.x >> 5) + wid) * RPW;
  const int64_t run = wrun0 + sub;
  const bool valid = run < args.B;
  const int64_t runc = valid ? run : args.B - 1;

  const DevCircuit &C = args.circ[0];
  const int M = C.n_steps;
  const int n_out = C.n_out;

  // ---- initial window: input amplitudes, |+> padding, initial CZ signs
  CT a[R];
  {
    const CT *in = reinterpret_cast<const CT *>(args.psi_in) + (args.istride ? runc * args.istride : 0);
#pragma unroll
    for (int j = 0; j < R; ++j) {
      const int idx = (li << RB) | j;
      const int2 mp = __ldg(&args.map[idx]);
      const CT v = in[mp.x & 0x7fffffff];
      a[j] = flip_sign(v, (uint32_t)mp.x & 0x80000000u);
    }
  }

  const bool want_phase = (args.flags & MBQC_F_REF_PHASE) != 0u;
  CT phase = mk<T>(T(1), T(0));  // product of this lane's step phases
  int e_applied = 0, pending = 0;
  for (int base = 0; base < M; base += KC) {
    __syncwarp();
    // stage this chunk: each run's lanes compute that run's coefficients
    for (int kk = li; kk < KC; kk += L) {
      const int k = base + kk;
      if (k < M) {
        const DevStep st = args.steps[C.step_off + k];
        const double th = st.aidx >= 0 ? args.angles[runc * args.astride + st.aidx] : st.fixed;
        CT c, ph;
        sv_coef(st.plane, th, want_phase, c, ph);
        s_coef[wid][sub][kk] = c;
        if (want_phase) phase = cmul(phase, ph);
      }
    }
    for (int kk = lane; kk < KC; kk += 32) {
      const int k = base + kk;
      if (k < M) {
        const uint32_t m = args.steps[C.step_off + k].mask;
        s_mask[wid][kk] = m;
        s_treg[wid][kk] = parity_table(m & ((1u << RB) - 1u), RB);
      }
    }
    __syncwarp();
    const int kend = min(KC, M - base);
    for (int p0 = 0; p0 < kend; p0 += W) {
      run_period<T, W, LL>(std::make_integer_sequence<int, W>{}, a, s_coef[wid][sub], s_mask[wid],
                           s_treg[wid], p0, kend, li);
      // period end: all-reduce the squared norm, apply last period's scale
      T s = T(0);
#pragma unroll
      for (int j = 0; j < R; ++j) s += a[j].x * a[j].x + a[j].y * a[j].y;
#pragma unroll
      for (int o = 1; o < L; o <<= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
      if (pending != 0) {
        const T g = RealBits<T>::pow2(-pending);
#pragma unroll
        for (int j = 0; j < R; ++j) a[j] = mk<T>(a[j].x * g, a[j].y * g);
      }
      e_applied += pending;
      int f = RealBits<T>::finite_pos(s) ? (RealBits<T>::expo(s) >> 1) : pending;
      int np = f - pending;
      pending = np > 100 ? 100 : (np < -100 ? -100 : np);
    }
  }

  // ---- epilogue: norm (pairwise within the lane, FP64 across lanes)
  T part[R];
#pragma unroll
  for (int j = 0; j < R; ++j) part[j] = a[j].x * a[j].x + a[j].y * a[j].y;
#pragma unroll
  for (int h = R / 2; h >= 1; h >>= 1)
#pragma unroll
    for (int j = 0; j < h; ++j) part[j] += part[j + h];
  double n2 = (double)part[0];
#pragma unroll
  for (int o = 1; o < L; o <<= 1) n2 += __shfl_xor_sync(0xffffffffu, n2, o);
  if (want_phase) {
#pragma unroll
    for (int o = 1; o < L; o <<= 1) {
      CT q;
      q.x = __shfl_xor_sync(0xffffffffu, phase.x, o);
      q.y = __shfl_xor_sync(0xffffffffu, phase.y, o);
      phase = cmul(phase, q);
    }
  }

  const bool ok = (n2 > 0.0) && (n2 < 1.0e300);
  T inv;
  if constexpr (sizeof(T) == 4) {
    const float nf = (float)n2;
    float y = rsqrtf(nf);
    y = y * (1.5f - 0.5f * nf * y * y);  // one Newton step
    inv = ok ? y : T(NAN);
  } else {
    inv = ok ? 1.0 / sqrt(n2) : T(NAN);
  }
  const CT sc = mk<T>(phase.x * inv, phase.y * inv);

  if (valid) {
    CT *out = reinterpret_cast<CT *>(args.psi_out) + run * ((int64_t)1 << n_out);
#pragma unroll
    for (int j = 0; j < R; ++j) {
      const int idx = (li << RB) | j;
      const int y = __ldg(&args.map[idx]).y;
      if (y >= 0) out[y] = cmul(a[j], sc);
    }
    if (li == 0) {
      if (args.status)
        args.status[run] = ok ? MBQC_RUN_OK : (isnan(n2) ? MBQC_RUN_NAN : MBQC_RUN_ZERO_NORM);
      if (args.logprob) {
        // ln(n2 / |in|^2) + ln2 * (2 e_applied + lp_const): exact exponents,
        // float logs of the mantissas
        const CT *in = reinterpret_cast<const CT *>(args.psi_in) + (args.istride ? run * args.istride : 0);
        T nin = T(0);
        for (int x = 0; x < (1 << C.n_in); ++x) nin += in[x].x * in[x].x + in[x].y * in[x].y;
        int e1, e2;
        const float m1 = frexpf((float)n2, &e1), m2 = frexpf((float)nin, &e2);
        const double ln2 = 0.6931471805599453;
        args.logprob[run] = (double)(logf(m1) - logf(m2)) +
                            ln2 * (double)(e1 - e2 + 2 * e_applied + C.lp_const);
      }
    }
  }
}

}  // namespace mbqc
