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

// Steps of circuits up to this length travel in the kernel parameters
// (constant bank): no dependent global load before the first angle load.
constexpr int kParamSteps = 128;

struct SvArgs {
  const DevStep *steps;   // this circuit's step table (used when M > kParamSteps)
  const int2 *map;        // [2^w]: .x = input index | CZ sign << 31, .y = output index or -1
  int64_t B;
  const double *angles;
  int64_t astride;
  const void *psi_in;
  int64_t istride;
  void *psi_out;
  uint32_t flags;
  double *logprob;
  int32_t *status;
  int M, n_in, n_out, lp_const;
  uint32_t out_mask;
  int steps_in_params;
  int8_t in_bits[16];
  int8_t out_bits[16];
  uint32_t init_cz[16];
  uint32_t p_mask[kParamSteps];
  int16_t p_aidx[kParamSteps];
  int8_t p_plane[kParamSteps];
  double p_fixed[kParamSteps];
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
// (x & keep) ^ sign on both components: the sign flip of the entering
// qubit's CZs and, with keep = 0, the zero of a shrinking step -- one LOP per
// component and a single code path (the period body stays small: with few
// warps per SM the unrolled body must fit the instruction caches)
__device__ __forceinline__ float2 keep_flip(float2 z, uint32_t keep, uint32_t s) {
  return make_float2(__uint_as_float((__float_as_uint(z.x) & keep) ^ s),
                     __uint_as_float((__float_as_uint(z.y) & keep) ^ s));
}
__device__ __forceinline__ double2 keep_flip(double2 z, uint32_t keep, uint32_t s) {
  const unsigned long long k = keep ? ~0ull : 0ull, m = (unsigned long long)s << 32;
  return make_double2(__longlong_as_double((__double_as_longlong(z.x) & k) ^ m),
                      __longlong_as_double((__double_as_longlong(z.y) & k) ^ m));
}

template <typename T, int R, int BIT>
__device__ __forceinline__ void reg_step(cplx<T> (&a)[R], cplx<T> c, uint32_t ts, bool dead) {
  const uint32_t keep = dead ? 0u : 0xffffffffu;
  const uint32_t tsk = dead ? 0u : ts;
#pragma unroll
  for (int j = 0; j < R; ++j) {
    if (j & (1 << BIT)) continue;
    const int jh = j | (1 << BIT);
    const cplx<T> x0 = a[j], x1 = a[jh];
    const cplx<T> phi = mk<T>(x0.x + c.x * x1.x - c.y * x1.y, x0.y + c.x * x1.y + c.y * x1.x);
    a[j] = phi;
    a[jh] = keep_flip(phi, keep, (tsk << (31 - jh)) & 0x80000000u);
  }
}

template <typename T, int R, int Q>
__device__ __forceinline__ void lane_step(cplx<T> (&a)[R], cplx<T> c, uint32_t ts, bool dead, int li) {
  const bool hi = (li >> Q) & 1;
  const cplx<T> cm = hi ? c : mk<T>(T(1), T(0));
  const uint32_t tl = (hi && !dead) ? ts : 0u;
  const uint32_t keep = (hi && dead) ? 0u : 0xffffffffu;
#pragma unroll
  for (int j = 0; j < R; ++j) {
    const cplx<T> m = a[j];
    const cplx<T> term = mk<T>(cm.x * m.x - cm.y * m.y, cm.x * m.y + cm.y * m.x);
    const cplx<T> phi = mk<T>(term.x + __shfl_xor_sync(0xffffffffu, term.x, 1 << Q),
                              term.y + __shfl_xor_sync(0xffffffffu, term.y, 1 << Q));
    a[j] = keep_flip(phi, keep, (tl << (31 - j)) & 0x80000000u);
  }
}

// coefficient of step kk at coef[kk * CS]
template <typename T, int W, int LL, int CS, int BIT>
__device__ __forceinline__ void one_step(cplx<T> (&a)[SvRegCfg<T, W, LL>::R], const cplx<T> *coef,
                                         const uint32_t *smask, const uint32_t *streg, int kk,
                                         int li) {
  using Cfg = SvRegCfg<T, W, LL>;
  const uint32_t mask = smask[kk];
  const uint32_t lp = __popc(((uint32_t)li << Cfg::RB) & mask) & 1u;
  const uint32_t ts = streg[kk] ^ (0u - lp);
  const bool dead = (mask & kDead) != 0u;
  const cplx<T> c = coef[kk * CS];
  if constexpr (BIT < Cfg::RB)
    reg_step<T, Cfg::R, BIT>(a, c, ts, dead);
  else
    lane_step<T, Cfg::R, BIT - Cfg::RB>(a, c, ts, dead, li);
}

template <typename T, int W, int LL, int CS, int... BITS>
__device__ __forceinline__ void run_period(std::integer_sequence<int, BITS...>,
                                           cplx<T> (&a)[SvRegCfg<T, W, LL>::R], const cplx<T> *coef,
                                           const uint32_t *smask, const uint32_t *streg, int p0,
                                           int kend, int li) {
  ((p0 + BITS < kend ? one_step<T, W, LL, CS, BITS>(a, coef, smask, streg, p0 + BITS, li) : void()),
   ...);
}

// --------------------------------------------------------------- kernel
template <typename T, int W, int LL>
__global__ void __launch_bounds__(32 * kSvWarps) sv_fwd_reg(const __grid_constant__ SvArgs args) {
  using Cfg = SvRegCfg<T, W, LL>;
  constexpr int L = Cfg::L, RB = Cfg::RB, R = Cfg::R, RPW = Cfg::RPW, KC = Cfg::KC;
  using CT = cplx<T>;

  // [step][run]: at each step the lanes of different runs read consecutive
  // slots (no bank conflicts)
  __shared__ CT s_coef[kSvWarps][KC][RPW];
  __shared__ uint32_t s_mask[kSvWarps][KC];
  __shared__ uint32_t s_treg[kSvWarps][KC];
  // index map of the window, shared by the block: one coalesced copy instead
  // of per-register bit loops (the code executed once per warp stays small,
  // which matters when few warps share an SM's instruction fetches)
  __shared__ int2 s_map[1 << W];
  for (int i = threadIdx.x; i < (1 << W); i += blockDim.x) s_map[i] = __ldg(&args.map[i]);
  __syncthreads();

  const int lane = threadIdx.x & 31;
  const int wid = threadIdx.x >> 5;
  const int sub = lane >> LL;
  const int li = lane & (L - 1);
  const int64_t wrun0 = ((int64_t)blockIdx.x * (blockDim.x >> 5) + wid) * RPW;
  const int64_t run = wrun0 + sub;
  const bool valid = run < args.B;
  const int64_t runc = valid ? run : args.B - 1;

  const int M = args.M;
  const int n_out = args.n_out;
  const bool pstep = args.steps_in_params != 0;

  // ---- initial window: input amplitudes, |+> padding, initial CZ signs
  CT a[R];
  {
    const CT *in = reinterpret_cast<const CT *>(args.psi_in) + (args.istride ? runc * args.istride : 0);
#pragma unroll
    for (int j = 0; j < R; ++j) {
      const int2 mp = s_map[(li << RB) | j];
      a[j] = flip_sign(in[mp.x & 0x7fffffff], (uint32_t)mp.x & 0x80000000u);
    }
  }

  const bool want_phase = (args.flags & MBQC_F_REF_PHASE) != 0u;
  CT phase = mk<T>(T(1), T(0));  // product of this lane's step phases
  int e_applied = 0, pending = 0;
  for (int base = 0; base < M; base += KC) {
    __syncwarp();
    // stage this chunk: each run's lanes compute that run's coefficients.
    // The angle loads of a batch of UB steps are issued together; the
    // coefficient loop is rolled (one sincos site in the code).
    {
      constexpr int ITER = (KC + L - 1) / L;
      constexpr int UB = ITER < 4 ? ITER : 4;
      for (int i0 = 0; i0 < ITER; i0 += UB) {
        double th[UB];
#pragma unroll
        for (int u = 0; u < UB; ++u) {
          const int kk = li + (i0 + u) * L, k = base + kk;
          th[u] = 0.0;
          if (kk < KC && k < M) {
            const int aidx = pstep ? (int)args.p_aidx[k] : args.steps[k].aidx;
            th[u] = aidx >= 0 ? args.angles[runc * args.astride + aidx]
                              : (pstep ? args.p_fixed[k] : args.steps[k].fixed);
          }
        }
#pragma unroll 1
        for (int u = 0; u < UB; ++u) {
          const int kk = li + (i0 + u) * L, k = base + kk;
          if (kk < KC && k < M) {
            const int plane = pstep ? (int)args.p_plane[k] : args.steps[k].plane;
            double t = th[0];
#pragma unroll
            for (int v = 1; v < UB; ++v)
              if (v == u) t = th[v];
            CT c, ph;
            sv_coef(plane, t, want_phase, c, ph);
            s_coef[wid][kk][sub] = c;
            if (want_phase) phase = cmul(phase, ph);
          }
        }
      }
    }
    for (int kk = lane; kk < KC; kk += 32) {
      const int k = base + kk;
      if (k < M) {
        const uint32_t m = pstep ? args.p_mask[k] : args.steps[k].mask;
        s_mask[wid][kk] = m;
        s_treg[wid][kk] = parity_table(m & ((1u << RB) - 1u), RB);
      }
    }
    __syncwarp();
    const int kend = min(KC, M - base);
    for (int p0 = 0; p0 < kend; p0 += W) {
      run_period<T, W, LL, RPW>(std::make_integer_sequence<int, W>{}, a, &s_coef[wid][0][sub], s_mask[wid],
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
      const int y = s_map[(li << RB) | j].y;
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
        for (int x = 0; x < (1 << args.n_in); ++x) nin += in[x].x * in[x].x + in[x].y * in[x].y;
        int e1, e2;
        const float m1 = frexpf((float)n2, &e1), m2 = frexpf((float)nin, &e2);
        const double ln2 = 0.6931471805599453;
        args.logprob[run] = (double)(logf(m1) - logf(m2)) +
                            ln2 * (double)(e1 - e2 + 2 * e_applied + args.lp_const);
      }
    }
  }
}

}  // namespace mbqc
