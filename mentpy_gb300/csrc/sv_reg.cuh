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
// (constant bank); only warp-uniform indices read them.
constexpr int kParamSteps = 128;
// The index map of windows up to 2^7 amplitudes travels there too: its
// per-lane reads replay in the constant cache, but they need no global
// memory access (after an L2 flush a global table costs a DRAM round trip
// and a TLB walk before the first input gather).
constexpr int kParamMapLog = 7;

struct SvArgs {
  const DevStep *steps;   // this circuit's step table (used when M > kParamSteps)
  const int2 *map;        // [2^w]: .x = input index | CZ sign << 31, .y = output index or -1
  const DevItem *items;   // item table (coefficients staged in item order), or nullptr
  int64_t B;
  const double *angles;
  int64_t astride;
  const void *psi_in;
  int64_t istride;
  void *psi_out;
  uint32_t flags;
  double *logprob;
  int32_t *status;
  int M, n_in, n_out, lp_const, A;
  int steps_in_params;
  int kc;                 // steps staged per chunk: a multiple of w, <= the kernel's KC
  uint32_t p_mask[kParamSteps];
  int16_t p_aidx[kParamSteps];
  int8_t p_plane[kParamSteps];
  double p_fixed[kParamSteps];
  int2 p_map[1 << kParamMapLog];  // the index map when w <= kParamMapLog
};

constexpr int kSvWarps = 4;  // warps per block (max)

// Input/output rows go through shared memory (coalesced row loads and
// stores, index-map gathers on chip) in the complex64 variants with at most
// 16 amplitudes per lane; the others gather from global memory directly.
__host__ __device__ constexpr bool sv_stage_io(int w, int ll, int cplx_bytes) {
  return cplx_bytes == 8 && w - ll <= 4;
}
// Shared-memory bytes of one warp's row staging: its runs' rows of up to 2^w
// amplitudes.
__host__ __device__ constexpr int sv_io_bytes(int w, int ll, int cplx_bytes) {
  return sv_stage_io(w, ll, cplx_bytes) ? (32 >> ll) * (1 << w) * cplx_bytes : 0;
}

// Steps staged per chunk at most: a multiple of w, at most the parameter step
// table, the block's coefficient and row staging within ~44 KB of shared
// memory.  A launch stages min(this, M rounded up to w) steps per chunk, and
// its dynamic shared memory is sized to that (sv_warp_smem per warp), so a
// short circuit leaves room for many blocks per SM.
__host__ __device__ constexpr int sv_chunk(int w, int ll, int cplx_bytes) {
  int k = (45056 - kSvWarps * sv_io_bytes(w, ll, cplx_bytes)) / (kSvWarps * (32 >> ll) * cplx_bytes);
  if (k > kParamSteps) k = kParamSteps;
  const int q = k / w;
  return (q > 0 ? q : 1) * w;
}
__host__ __device__ constexpr int sv_al16(int b) { return (b + 15) & ~15; }
// The warp's angle rows are staged in shared memory (16-byte row loads, one
// round trip) when the circuit is one chunk and the rows take at most 4 KB.
__host__ __device__ constexpr bool sv_stage_ang(int ll, int kc) { return (32 >> ll) * kc * 8 <= 4096; }
// Shared memory of one warp for a chunk of kc steps: coefficients [kc][runs],
// amp [kc][runs] (general planes), CZ masks and register parity tables [kc],
// input/output rows [runs][2^w] (when staged), angle rows [runs][<= kc].
__host__ __device__ constexpr int sv_warp_smem(int w, int ll, int cplx_bytes, int kc, bool gen) {
  return sv_al16(kc * (32 >> ll) * cplx_bytes) + (gen ? sv_al16(kc * (32 >> ll) * cplx_bytes / 2) : 0) +
         2 * sv_al16(kc * 4) + sv_io_bytes(w, ll, cplx_bytes) + (sv_stage_ang(ll, kc) ? (32 >> ll) * kc * 8 : 0);
}
// Steps per chunk for a circuit of M steps.
__host__ __device__ constexpr int sv_kc(int w, int ll, int cplx_bytes, int M) {
  const int kmax = sv_chunk(w, ll, cplx_bytes);
  const int need = ((M > 0 ? M : 1) + w - 1) / w * w;
  return need < kmax ? need : kmax;
}

// uncached loads of one complex amplitude (host-mapped inputs)
__device__ __forceinline__ void ldcv_cplx(const float2 *p, float2 &v) { v = __ldcv(p); }
__device__ __forceinline__ void ldcv_cplx(const double2 *p, double2 &v) { v = __ldcv(p); }

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
  // steps staged per chunk: a multiple of W, at most 128 (the parameter step
  // table), coefficient staging within ~40 KB of shared memory per block
  static constexpr int KC = sv_chunk(W, LL, (int)sizeof(cplx<T>));
  static_assert(LL >= 0 && LL <= 5 && RB >= 0 && RB <= 5, "register layout");
};

// ---------------------------------------------------------------- steps
// (x & keep) ^ sign on both components: the sign flip of the entering
// qubit's CZs and, with keep = 0, the zero of a shrinking step (the FP64
// check mode's path)
__device__ __forceinline__ float2 keep_flip(float2 z, uint32_t keep, uint32_t s) {
  return make_float2(__uint_as_float((__float_as_uint(z.x) & keep) ^ s),
                     __uint_as_float((__float_as_uint(z.y) & keep) ^ s));
}
__device__ __forceinline__ double2 keep_flip(double2 z, uint32_t keep, uint32_t s) {
  const unsigned long long k = keep ? ~0ull : 0ull, m = (unsigned long long)s << 32;
  return make_double2(__longlong_as_double((__double_as_longlong(z.x) & k) ^ m),
                      __longlong_as_double((__double_as_longlong(z.y) & k) ^ m));
}

// float path: the sign alone is one LOP3 per component (z ^ (t & 0x80000000),
// t shifted by a multiply that may issue on the FMA pipe); a shrinking step
// zeroes the upper halves afterwards
__device__ __forceinline__ float2 sign_bit_flip(float2 z, uint32_t t) {
  return make_float2(__uint_as_float(__float_as_uint(z.x) ^ (t & 0x80000000u)),
                     __uint_as_float(__float_as_uint(z.y) ^ (t & 0x80000000u)));
}

template <typename T, int R, int BIT>
__device__ __forceinline__ void reg_step(cplx<T> (&a)[R], cplx<T> c, uint32_t ts, bool dead) {
  if constexpr (sizeof(T) == 4) {
#pragma unroll
    for (int j = 0; j < R; ++j) {
      if (j & (1 << BIT)) continue;
      const int jh = j | (1 << BIT);
      const float2 x0 = a[j], x1 = a[jh];
      const float2 phi = make_float2(x0.x + c.x * x1.x - c.y * x1.y, x0.y + c.x * x1.y + c.y * x1.x);
      a[j] = phi;
      a[jh] = sign_bit_flip(phi, ts * (1u << (31 - jh)));
    }
    if (dead) {
#pragma unroll
      for (int j = 0; j < R; ++j)
        if (j & (1 << BIT)) a[j] = make_float2(0.f, 0.f);
    }
  } else {
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
}

template <typename T, int R, int Q>
__device__ __forceinline__ void lane_step(cplx<T> (&a)[R], cplx<T> c, uint32_t ts, bool dead, int li) {
  const bool hi = (li >> Q) & 1;
  const cplx<T> cm = hi ? c : mk<T>(T(1), T(0));
  if constexpr (sizeof(T) == 4) {
    const uint32_t tl = hi ? ts : 0u;
#pragma unroll
    for (int j = 0; j < R; ++j) {
      const float2 m = a[j];
      const float2 term = make_float2(cm.x * m.x - cm.y * m.y, cm.x * m.y + cm.y * m.x);
      const float2 phi = make_float2(term.x + __shfl_xor_sync(0xffffffffu, term.x, 1 << Q),
                                     term.y + __shfl_xor_sync(0xffffffffu, term.y, 1 << Q));
      a[j] = sign_bit_flip(phi, tl * (1u << (31 - j)));
    }
    if (hi && dead) {
#pragma unroll
      for (int j = 0; j < R; ++j) a[j] = make_float2(0.f, 0.f);
    }
  } else {
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
}

// General-plane steps (XZ, YZ): phi = amp x0 + c x1 with a real amp (1 in
// the XY plane); the same sign and shrink handling as reg_step / lane_step.
template <typename T, int R, int BIT>
__device__ __forceinline__ void reg_step_g(cplx<T> (&a)[R], cplx<T> c, T amp, uint32_t ts, bool dead) {
  const uint32_t keep = dead ? 0u : 0xffffffffu;
  const uint32_t tsk = dead ? 0u : ts;
#pragma unroll
  for (int j = 0; j < R; ++j) {
    if (j & (1 << BIT)) continue;
    const int jh = j | (1 << BIT);
    const cplx<T> x0 = a[j], x1 = a[jh];
    const cplx<T> phi = mk<T>(amp * x0.x + c.x * x1.x - c.y * x1.y, amp * x0.y + c.x * x1.y + c.y * x1.x);
    a[j] = phi;
    a[jh] = keep_flip(phi, keep, (tsk << (31 - jh)) & 0x80000000u);
  }
}

template <typename T, int R, int Q>
__device__ __forceinline__ void lane_step_g(cplx<T> (&a)[R], cplx<T> c, T amp, uint32_t ts, bool dead, int li) {
  const bool hi = (li >> Q) & 1;
  const cplx<T> cm = hi ? c : mk<T>(amp, T(0));
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

// Stage J of the xor butterfly that all-reduces the previous period's squared
// norm over the run's lanes, spread over the steps of the next period so that
// the shuffle latency overlaps the step arithmetic (stage J adds the partner
// value fetched at stage J-1 and fetches the next one).  The xor butterfly
// gives bitwise-identical sums on every lane, so all lanes of a run pick the
// same power-of-two scale.
template <int LL, int J, typename T>
__device__ __forceinline__ void norm_stage(T &x, T &t) {
  if constexpr (J < LL) {
    x += t;
    t = __shfl_xor_sync(0xffffffffu, x, 1 << J);
  }
}

// one period of steps p0 .. min(p0 + W, kend) - 1
template <typename T, int W, int LL, int CS, int... BITS>
__device__ __forceinline__ void run_period(std::integer_sequence<int, BITS...>,
                                           cplx<T> (&a)[SvRegCfg<T, W, LL>::R], const cplx<T> *coef,
                                           const uint32_t *smask, const uint32_t *streg, int p0,
                                           int kend, int li) {
  ((p0 + BITS < kend ? one_step<T, W, LL, CS, BITS>(a, coef, smask, streg, p0 + BITS, li) : void()),
   ...);
}

// Step constants of step kk: CZ sign word of this lane, window-shrink flag
// and coefficient (the parts of one_step that do not depend on the state).
template <typename T, int W, int LL, int CS, bool GEN>
__device__ __forceinline__ void step_consts(const cplx<T> *coef, const T *amps, const uint32_t *smask,
                                            const uint32_t *streg, int kk, int li, uint32_t &ts,
                                            uint32_t &dead, cplx<T> &c, T &amp) {
  using Cfg = SvRegCfg<T, W, LL>;
  const uint32_t mask = smask[kk];
  const uint32_t lp = __popc(((uint32_t)li << Cfg::RB) & mask) & 1u;
  ts = streg[kk] ^ (0u - lp);
  dead = mask & kDead;
  c = coef[kk * CS];
  if constexpr (GEN) amp = amps[kk * CS];
}

template <typename T, int W, int LL, int BIT, bool GEN>
__device__ __forceinline__ void step_apply(cplx<T> (&a)[SvRegCfg<T, W, LL>::R], cplx<T> c, T amp, uint32_t ts,
                                           uint32_t dead, int li) {
  using Cfg = SvRegCfg<T, W, LL>;
  if constexpr (GEN) {
    if constexpr (BIT < Cfg::RB)
      reg_step_g<T, Cfg::R, BIT>(a, c, amp, ts, dead != 0u);
    else
      lane_step_g<T, Cfg::R, BIT - Cfg::RB>(a, c, amp, ts, dead != 0u, li);
  } else {
    if constexpr (BIT < Cfg::RB)
      reg_step<T, Cfg::R, BIT>(a, c, ts, dead != 0u);
    else
      lane_step<T, Cfg::R, BIT - Cfg::RB>(a, c, ts, dead != 0u, li);
  }
}

// The same with the stages of a norm all-reduce interleaved.  The period's
// step constants are read from shared memory up front (slots past kend hold
// stale values of this chunk and are not applied), so the steps' dependency
// chain is the state arithmetic alone.
template <typename T, int W, int LL, int CS, bool GEN, int... BITS>
__device__ __forceinline__ void run_period(std::integer_sequence<int, BITS...>,
                                           cplx<T> (&a)[SvRegCfg<T, W, LL>::R], const cplx<T> *coef,
                                           const T *amps, const uint32_t *smask, const uint32_t *streg, int p0,
                                           int kend, int li, T &x, T &t) {
  uint32_t ts[W], dead[W];
  cplx<T> c[W];
  T amp[W];
  (step_consts<T, W, LL, CS, GEN>(coef, amps, smask, streg, p0 + BITS, li, ts[BITS], dead[BITS], c[BITS],
                                  amp[BITS]),
   ...);
  ((p0 + BITS < kend ? step_apply<T, W, LL, BITS, GEN>(a, c[BITS], amp[BITS], ts[BITS], dead[BITS], li) : void(),
    norm_stage<LL, BITS>(x, t)),
   ...);
}

// squared norm of a lane's amplitudes, summed as a tree (short dependency chain)
template <typename T, int R>
__device__ __forceinline__ T lane_norm2(const cplx<T> (&a)[R]) {
  T p[R];
#pragma unroll
  for (int j = 0; j < R; ++j) p[j] = a[j].x * a[j].x + a[j].y * a[j].y;
#pragma unroll
  for (int h = R / 2; h >= 1; h >>= 1)
#pragma unroll
    for (int j = 0; j < h; ++j) p[j] += p[j + h];
  return p[0];
}

// --------------------------------------------------------------- kernel
// GEN: plans with XZ / YZ steps (coefficient pairs amp, c); the XY, X, Y
// instantiations keep the one-coefficient step.
// Register cap of an instantiation.  The device-input float kernels with at
// most 8 amplitudes a lane are capped at 120 (16 warps per SM instead of 12 at
// their natural ~134, no spills): back-to-back 4096-run steps overlap more,
// 3.13 -> 2.90 us.  The host-mapped instantiations keep their registers
// (capped they lost ~0.4 us per step over the CPU-GPU link).
template <typename T, int W, int LL, bool GEN, bool HOST>
__host__ __device__ constexpr int sv_maxnreg() {
  return (sizeof(T) == 4 && !GEN && !HOST && W - LL <= 3) ? 120 : 255;
}

// HOST: the instantiation for host-mapped inputs (MBQC_F_HOST_INPUTS), which
// stages one-chunk angle rows with 16-byte loads.
template <typename T, int W, int LL, bool GEN = false, bool HOST = false>
__global__ void __maxnreg__((sv_maxnreg<T, W, LL, GEN, HOST>())) sv_fwd_reg(const __grid_constant__ SvArgs args) {
  using Cfg = SvRegCfg<T, W, LL>;
  constexpr int L = Cfg::L, RB = Cfg::RB, R = Cfg::R, RPW = Cfg::RPW, KC = Cfg::KC;
  using CT = cplx<T>;

  constexpr bool kIO = sv_stage_io(W, LL, (int)sizeof(CT));
  static_assert(KC >= W, "chunk");
  const int lane = threadIdx.x & 31;
  const int wid = threadIdx.x >> 5;
  // this warp's slice of the dynamic shared memory (sv_warp_smem):
  // coefficients [kc][run] (at each step the lanes of different runs read
  // consecutive slots: no bank conflicts), amp of general-plane steps, the
  // chunk's CZ masks and register parity tables, and the input and output
  // rows of the warp's runs (coalesced row accesses, index gathers on chip)
  const int kc = args.kc;
  extern __shared__ __align__(16) unsigned char sv_smem[];
  unsigned char *wsm = sv_smem + (size_t)wid * sv_warp_smem(W, LL, (int)sizeof(CT), kc, GEN);
  CT *s_coef = reinterpret_cast<CT *>(wsm);
  wsm += sv_al16(kc * RPW * (int)sizeof(CT));
  T *s_amp = reinterpret_cast<T *>(wsm);
  wsm += GEN ? sv_al16(kc * RPW * (int)sizeof(T)) : 0;
  uint32_t *s_mask = reinterpret_cast<uint32_t *>(wsm);
  wsm += sv_al16(kc * 4);
  uint32_t *s_treg = reinterpret_cast<uint32_t *>(wsm);
  wsm += sv_al16(kc * 4);
  CT *s_io = reinterpret_cast<CT *>(wsm);  // [RPW][2^W]
  wsm += sv_io_bytes(W, LL, (int)sizeof(CT));
  double *s_ang = reinterpret_cast<double *>(wsm);  // [RPW][A] (staged angle rows)
  const int sub = lane >> LL;
  const int li = lane & (L - 1);
  const int64_t wrun0 = ((int64_t)blockIdx.x * (blockDim.x >> 5) + wid) * RPW;
  const int64_t run = wrun0 + sub;
  const bool valid = run < args.B;
  const int64_t runc = valid ? run : args.B - 1;

  const int M = args.M;
  const int n_out = args.n_out;
  const bool pstep = args.steps_in_params != 0;
  // item order (the host passes an item table only when the circuit is one
  // chunk): item i < A is angle i -- a contiguous row load that depends on
  // nothing in the plan -- and items A.. are the fixed-angle steps; otherwise
  // item i of a chunk is step base + i
  const DevItem *items = args.items;
  const bool want_phase = (args.flags & MBQC_F_REF_PHASE) != 0u;
  const bool host_in = (args.flags & MBQC_F_HOST_INPUTS) != 0u;
  const bool inputs_ready = (args.flags & MBQC_F_INPUTS_READY) != 0u;
  const double *arow = args.angles + runc * args.astride;
  auto angle_at = [&](int i) -> double { return host_in ? __ldcv(arow + i) : arow[i]; };

  // coefficient staging, four items per batch: lane li stages items
  // li, li + L, ...; a batch's loads are issued before the previous batch is
  // computed.  All per-lane tables are global loads (per-lane indices into
  // the kernel parameters would serialise in the constant cache).  The plan
  // half of a batch (step, plane, angle index or fixed angle) reads only plan
  // tables; the angle half reads the caller's angles.
  struct Batch {
    double th[4];
    int step[4], plane[4], aidx[4];
  };
  auto load4_plan = [&](int base, int n, int u0, Batch &b) {
#pragma unroll
    for (int u = 0; u < 4; ++u) {
      const int i = li + (u0 + u) * L;
      b.th[u] = 0.0;
      b.step[u] = base + i;
      b.plane[u] = MBQC_PLANE_X;
      b.aidx[u] = -1;
      if (i < n) {
        if (items) {
          const DevItem it = items[i];
          b.step[u] = it.step;
          b.plane[u] = it.plane;
          b.aidx[u] = i < args.A ? i : -1;
          b.th[u] = it.fixed;
        } else {
          const int k = base + i;
          b.aidx[u] = pstep ? (int)args.p_aidx[k] : args.steps[k].aidx;
          b.plane[u] = pstep ? (int)args.p_plane[k] : args.steps[k].plane;
          b.th[u] = pstep ? args.p_fixed[k] : args.steps[k].fixed;
        }
      }
    }
  };
  // one-chunk circuits with host-mapped inputs read their angles from the
  // warp's staged rows (one round trip over the CPU-GPU link for all of
  // them); from device memory the per-lane loads, four in flight while the
  // previous four are turned into coefficients, are faster
  const bool stage_ang = HOST && host_in && items != nullptr && sv_stage_ang(LL, kc);
  auto load4_angles = [&](Batch &b) {
#pragma unroll
    for (int u = 0; u < 4; ++u)
      if (b.aidx[u] >= 0) b.th[u] = stage_ang ? s_ang[sub * args.A + b.aidx[u]] : angle_at(b.aidx[u]);
  };
  auto load4 = [&](int base, int n, int u0, Batch &b) {
    load4_plan(base, n, u0, b);
    load4_angles(b);
  };
  CT phase = mk<T>(T(1), T(0));  // product of this lane's step phases
  auto comp4 = [&](int base, int n, int u0, const Batch &b) {
#pragma unroll
    for (int u = 0; u < 4; ++u) {
      const int i = li + (u0 + u) * L;
      if (i < n) {
        CT c, ph;
        if constexpr (GEN) {
          T amp;
          sv_coef_gen(b.plane[u], b.th[u], want_phase, c, amp, ph);
          s_amp[(b.step[u] - base) * RPW + sub] = amp;
        } else {
          sv_coef(b.plane[u], b.th[u], want_phase, c, ph);
        }
        s_coef[(b.step[u] - base) * RPW + sub] = c;
        if (want_phase) phase = cmul(phase, ph);
      }
    }
  };
  // Before the wait for the previous kernel on the stream: the plan half of
  // the first batch, this lane's entries of the index map, and L2 prefetches
  // of the warp's angle rows and input rows (device memory only: the L2 is
  // the coherence point, so a prefetched line still sees that kernel's
  // writes).  Then the next kernel may start its own prologue.
  Batch bA, bB;
  const int n0 = items ? M : min(kc, M);
  load4_plan(0, n0, 0, bA);
  int mx[R], my[R];
#pragma unroll
  for (int j = 0; j < R; ++j) {
    int2 m;
    if constexpr (W <= kParamMapLog)
      m = args.p_map[(li << RB) | j];
    else
      m = __ldg(&args.map[(li << RB) | j]);
    mx[j] = m.x;
    my[j] = m.y;
  }
  if (!host_in && !inputs_ready) {
    // one lane per 128-byte line of the angle rows, then of the input rows;
    // every prefetched address lies inside a row of a valid run
    const int alines = (int)((args.A * (int64_t)sizeof(double) + 127) / 128);
    for (int e = lane; e < alines * RPW; e += 32) {
      const int r = e / alines, q = e - r * alines;
      if (wrun0 + r < args.B)
        prefetch_l2(reinterpret_cast<const char *>(args.angles + (wrun0 + r) * args.astride) + 128 * q);
    }
    if (args.istride) {
      const int64_t ibytes = ((int64_t)1 << args.n_in) * (int64_t)sizeof(CT);
      const int ilines = (int)((ibytes + 127) / 128);
      const CT *in0 = reinterpret_cast<const CT *>(args.psi_in);
      for (int e = lane; e < ilines * RPW; e += 32) {
        const int r = e / ilines, q = e - r * ilines;
        if (wrun0 + r < args.B)
          prefetch_l2(reinterpret_cast<const char *>(in0 + (wrun0 + r) * args.istride) + 128 * q);
      }
    }
  }
  // the next launch may start its own prologue now; the caller's memory is
  // read after the previous launch completes, unless the caller declared
  // its inputs ready (then only the writes wait, in the epilogue)
  griddep_launch_dependents();
  if (!inputs_ready) griddep_wait();
  // a full warp with contiguous rows loads 16 bytes a lane (staged angles,
  // input rows), all issued before any is used: one round trip (over the
  // CPU-GPU link for host-mapped buffers)
  const bool full_warp = wrun0 + RPW <= args.B;
  if (stage_ang) {
    const int A = args.A;
    const double *rows = args.angles + wrun0 * args.astride;
    if (full_warp && args.astride == A && ((RPW * A) & 1) == 0 && (reinterpret_cast<uintptr_t>(rows) & 15) == 0) {
      const double2 *r2 = reinterpret_cast<const double2 *>(rows);
      double2 *d2 = reinterpret_cast<double2 *>(s_ang);
      for (int e2 = lane; e2 < RPW * A / 2; e2 += 32) d2[e2] = host_in ? __ldcv(r2 + e2) : r2[e2];
    } else {
      for (int e = lane; e < RPW * A; e += 32) {
        const int r = e / A;
        const int64_t rr = wrun0 + r < args.B ? wrun0 + r : args.B - 1;
        const double *src = args.angles + rr * args.astride + (e - r * A);
        s_ang[e] = host_in ? __ldcv(src) : *src;
      }
    }
  }

  // ---- initial window: input amplitudes, |+> padding, initial CZ signs
  constexpr int NV = (R + 1) / 2;  // 16-byte input loads per lane (the vector path)
  CT v[kIO ? R : 1];
  float4 vv[kIO && sizeof(CT) == 8 ? NV : 1];
  bool vec_in = false;
  if constexpr (kIO) {
    // the warp's input rows (RPW * 2^n_in <= 32 * R amplitudes)
    const int nin = args.n_in, din = 1 << nin;
    const CT *in0 = reinterpret_cast<const CT *>(args.psi_in);
    if constexpr (sizeof(CT) == 8) {
      const CT *base = in0 + (args.istride ? wrun0 * args.istride : 0);
      vec_in = full_warp && nin >= 1 && (args.istride == din || args.istride == 0) &&
               (reinterpret_cast<uintptr_t>(base) & 15) == 0;
      if (vec_in) {
        const float4 *src4 = reinterpret_cast<const float4 *>(base);
#pragma unroll
        for (int t = 0; t < NV; ++t) {
          const int e2 = lane + 32 * t;
          if (e2 < RPW * din / 2) {
            const float4 *src = src4 + (args.istride ? e2 : ((2 * e2) & (din - 1)) >> 1);
            vv[t] = host_in ? __ldcv(src) : *src;
          }
        }
      }
    }
    if (!vec_in) {
#pragma unroll
      for (int t = 0; t < R; ++t) {
        const int e = lane + 32 * t;
        if (e < RPW * din) {
          const int r = e >> nin;
          const int64_t rr = wrun0 + r < args.B ? wrun0 + r : args.B - 1;
          const CT *src = in0 + (args.istride ? rr * args.istride : 0) + (e & (din - 1));
          if (host_in)
            ldcv_cplx(src, v[t]);
          else
            v[t] = *src;
        }
      }
    }
  }
  if (stage_ang) __syncwarp();
  load4_angles(bA);

  CT a[R];
  if constexpr (kIO) {
    const int nin = args.n_in, din = 1 << nin;
    if constexpr (sizeof(CT) == 8) {
      if (vec_in) {
#pragma unroll
        for (int t = 0; t < NV; ++t) {
          const int e2 = lane + 32 * t;
          if (e2 < RPW * din / 2) {
            const int e = 2 * e2;
            *reinterpret_cast<float4 *>(&s_io[(e >> nin) * (1 << W) + (e & (din - 1))]) = vv[t];
          }
        }
      }
    }
    if (!vec_in) {
#pragma unroll
      for (int t = 0; t < R; ++t) {
        const int e = lane + 32 * t;
        if (e < RPW * din) s_io[(e >> nin) * (1 << W) + (e & (din - 1))] = v[t];
      }
    }
    __syncwarp();
#pragma unroll
    for (int j = 0; j < R; ++j)
      a[j] = flip_sign(s_io[sub * (1 << W) + (mx[j] & 0x7fffffff)], (uint32_t)mx[j] & 0x80000000u);
  } else {
    const CT *in = reinterpret_cast<const CT *>(args.psi_in) + (args.istride ? runc * args.istride : 0);
#pragma unroll
    for (int j = 0; j < R; ++j) {
      CT w;
      if (host_in)
        ldcv_cplx(in + (mx[j] & 0x7fffffff), w);
      else
        w = in[mx[j] & 0x7fffffff];
      a[j] = flip_sign(w, (uint32_t)mx[j] & 0x80000000u);
    }
  }

  int e_applied = 0;
  T x = T(0), t = T(0);  // squared norm being all-reduced, partner value in flight
  for (int base = 0; base < M; base += kc) {
    __syncwarp();
    const int n = items ? M : min(kc, M - base);
    const int per_lane = (n + L - 1) / L;
    if (base != 0) load4(base, n, 0, bA);
#pragma unroll 1
    for (int u0 = 0; u0 < per_lane; u0 += 8) {
      const bool second = u0 + 4 < per_lane;
      if (second) load4(base, n, u0 + 4, bB);
      comp4(base, n, u0, bA);
      if (second) {
        if (u0 + 8 < per_lane) load4(base, n, u0 + 8, bA);
        comp4(base, n, u0 + 4, bB);
      }
    }
    for (int kk = lane; kk < kc; kk += 32) {
      const int k = base + kk;
      if (k < M) {
        const uint32_t m = pstep ? args.p_mask[k] : args.steps[k].mask;
        s_mask[kk] = m;
        s_treg[kk] = parity_table(m & ((1u << RB) - 1u), RB);
      }
    }
    __syncwarp();
    const int kend = min(kc, M - base);
    for (int p0 = 0; p0 < kend; p0 += W) {
      run_period<T, W, LL, RPW, GEN>(std::make_integer_sequence<int, W>{}, a, s_coef + sub,
                                     GEN ? s_amp + sub : nullptr, s_mask, s_treg, p0, kend, li,
                                     x, t);
      // period end: the butterfly of the previous period's squared norm is
      // complete; rescale by the exact power of two it gives, then start the
      // next one
      if constexpr (LL > 0) x += t;
      int f = RealBits<T>::finite_pos(x) ? (RealBits<T>::expo(x) >> 1) : 0;
      f = f > 100 ? 100 : (f < -100 ? -100 : f);
      const T g = RealBits<T>::pow2(-f);
#pragma unroll
      for (int j = 0; j < R; ++j) a[j] = mk<T>(a[j].x * g, a[j].y * g);
      e_applied += f;
      x = lane_norm2<T, R>(a);
      t = T(0);
    }
  }

  // ---- epilogue: norm, pairwise within the lane; across lanes an
  // error-free (double-float) sum in the float path -- FP64-level accuracy
  // without the slow FP64 pipe -- and FP64 in the double path.  Both are xor
  // butterflies, so every lane of a run holds the same bits.
  T n2t, n2lo = T(0);
  {
    T hi = lane_norm2<T, R>(a);
    if constexpr (sizeof(T) == 4) {
      T lo = T(0);
#pragma unroll
      for (int o = 1; o < L; o <<= 1) {
        const T oh = __shfl_xor_sync(0xffffffffu, hi, o);
        const T ol = __shfl_xor_sync(0xffffffffu, lo, o);
        const T sum = hi + oh;  // two-sum: sum + err == hi + oh exactly
        const T bb = sum - hi;
        const T err = (hi - (sum - bb)) + (oh - bb);
        hi = sum;
        lo = (lo + ol) + err;
      }
      const T sum = hi + lo;  // renormalise the pair
      n2lo = lo - (sum - hi);
      hi = sum;
    } else {
#pragma unroll
      for (int o = 1; o < L; o <<= 1) hi += __shfl_xor_sync(0xffffffffu, hi, o);
    }
    n2t = hi;
  }
  if (want_phase) {
#pragma unroll
    for (int o = 1; o < L; o <<= 1) {
      CT q;
      q.x = __shfl_xor_sync(0xffffffffu, phase.x, o);
      q.y = __shfl_xor_sync(0xffffffffu, phase.y, o);
      phase = cmul(phase, q);
    }
  }

  T inv;
  bool ok;
  if constexpr (sizeof(T) == 4) {
    ok = (n2t > 0.f) && (n2t < 3.0e38f);
    float y = rsqrtf(n2t);
    y = y * (1.5f - 0.5f * n2t * y * y);  // one Newton step
    inv = ok ? y : T(NAN);
  } else {
    ok = (n2t > 0.0) && (n2t < 1.0e300);
    inv = ok ? 1.0 / sqrt(n2t) : T(NAN);
  }
  const CT sc = mk<T>(phase.x * inv, phase.y * inv);
  if (inputs_ready) griddep_wait();  // before the first write

  if constexpr (kIO) {
    // outputs: scattered into the staging rows, then coalesced row stores
    __syncwarp();
#pragma unroll
    for (int j = 0; j < R; ++j)
      if (my[j] >= 0) s_io[sub * (1 << W) + my[j]] = cmul(a[j], sc);
    __syncwarp();
    const int dout = 1 << n_out;
    CT *out0 = reinterpret_cast<CT *>(args.psi_out);
    for (int e = lane; e < RPW * dout; e += 32) {
      const int64_t rr = wrun0 + (e >> n_out);
      if (rr < args.B) out0[rr * dout + (e & (dout - 1))] = s_io[(e >> n_out) * (1 << W) + (e & (dout - 1))];
    }
  }
  if (valid) {
    if constexpr (!kIO) {
      CT *out = reinterpret_cast<CT *>(args.psi_out) + run * ((int64_t)1 << n_out);
#pragma unroll
      for (int j = 0; j < R; ++j)
        if (my[j] >= 0) out[my[j]] = cmul(a[j], sc);
    }
    if (li == 0) {
      if (args.status)
        args.status[run] = ok ? MBQC_RUN_OK : (isnan(n2t) ? MBQC_RUN_NAN : MBQC_RUN_ZERO_NORM);
      if (args.logprob) {
        // ln(n2 / |in|^2) + ln2 * (2 e_applied + lp_const): exact exponents,
        // float logs of the mantissas
        const CT *in = reinterpret_cast<const CT *>(args.psi_in) + (args.istride ? run * args.istride : 0);
        T nin = T(0);
        for (int x = 0; x < (1 << args.n_in); ++x) nin += in[x].x * in[x].x + in[x].y * in[x].y;
        int e1, e2;
        const float m1 = frexpf((float)n2t, &e1), m2 = frexpf((float)nin, &e2);
        const double ln2 = 0.6931471805599453;
        args.logprob[run] = (double)(logf(m1) - logf(m2)) + (double)n2lo / (double)n2t +
                            ln2 * (double)(e1 - e2 + 2 * e_applied + args.lp_const);
      }
    }
  }
}

}  // namespace mbqc
