// Adjoint (reverse-mode) gradient of the statevector sweep, windows w <= 8.
//
// The forward sweep of one run is a chain of linear maps on the 2^w window,
//   psi_k = E_k C_k(theta_k) psi_{k-1},
//   C_k:  phi[r] = psi[r, 0] + c_k psi[r, 1],   c_k = e^{-i theta_k}
//   E_k:  psi'[r, 0] = phi[r],  psi'[r, 1] = s_k(r) phi[r]   (or 0: no qubit enters)
// followed by the normalisation z = psi_M / |psi_M| and the output gather.
// With lambda_M = dL/dz projected on the tangent of the sphere and divided by
// |psi_M| (PyTorch's convention: dL = Re <g|dz>), the backward sweep is
//   mu[r]              = lambda_k[r, 0] + s_k(r) lambda_k[r, 1]
//   dL/dtheta_k       += Im(c_k * sum_r conj(mu[r]) psi_{k-1}[r, 1])
//   lambda_{k-1}[r, 0] = mu[r],  lambda_{k-1}[r, 1] = conj(c_k) mu[r].
// Positive power-of-two renormalisations between periods are constants of the
// chain (they cancel in z) and are undone on lambda.
//
// Memory stays O(window) per run: the state at the start of every period of w
// steps is checkpointed to a workspace indexed by in-flight slot (a persistent
// grid bounds the workspace to the runs resident on the GPU, which fits L2),
// and during the backward sweep each period is recomputed from its checkpoint
// keeping the pre-step half-states psi_{k-1}[., 1] of that period in
// registers.  Per-lane gradient partials go to shared-memory slots and are
// reduced across lanes in FP64 at the end of the run.
//
// Two seeds:
//  * generic: grad_out[run] = dL/dz (for torch.autograd.Function backward);
//  * fidelity: run = (v, j), loss_v = 1 - (1/J) sum_j |<t_j|z_vj>|^2, with
//    the loss (FP64) and the gradient summed over j in the kernel.
#pragma once

#include <utility>

#include "sv_reg.cuh"

namespace mbqc {

struct SvAdjArgs {
  const DevStep *steps;
  const int2 *map;
  int M, W, n_in, n_out, n_angles;
  int64_t B;             // runs
  int64_t J;             // fidelity mode: inputs per angle vector; 0 = generic mode
  const double *angles;  // generic: row per run; fidelity: row per vector (run / J)
  int64_t astride;
  const void *psi_in;    // generic: row per run (istride 0 = broadcast); fidelity: row j
  int64_t istride;
  const void *grad_out;  // generic: [B, 2^n_out]
  const void *targets;   // fidelity: [J, 2^n_out]
  double *loss;          // fidelity: [B / J]
  double *grad;          // generic: [B, n_angles]; fidelity: [B / J, n_angles] (accumulated)
  int32_t *status;
  void *ckpt;            // workspace
  int64_t n_slots;       // checkpoint slots (= grid warps * runs per warp)
};

// log2(lanes per run) of the adjoint kernel: <= 8 (f32) / 4 (f64) amplitudes
// per lane, so that one period of pre-step half-states stays in registers.
constexpr int adj_ll(int w, bool f64) {
  const int r = f64 ? 2 : 3;
  return w - r > 0 ? w - r : 0;
}
constexpr int kAdjMaxWindow = 8;

template <int W, int RB, int R> struct AdjHist {
  static constexpr int sz(int t) { return t < RB ? R / 2 : R; }
  static constexpr int off(int t) { return t == 0 ? 0 : off(t - 1) + sz(t - 1); }
  static constexpr int total = off(W - 1) + sz(W - 1);
};

// index of j with bit BIT removed
template <int BIT> __host__ __device__ constexpr int squeeze(int j) {
  return (j & ((1 << BIT) - 1)) | ((j >> (BIT + 1)) << BIT);
}

// ------------------------------------------------ forward step with history
template <typename T, int R, int BIT, int HOFF, int HN>
__device__ __forceinline__ void reg_step_h(cplx<T> (&a)[R], cplx<T> (&h)[HN], cplx<T> c,
                                           uint32_t ts, bool dead) {
#pragma unroll
  for (int j = 0; j < R; ++j) {
    if (j & (1 << BIT)) continue;
    const int jh = j | (1 << BIT);
    h[HOFF + squeeze<BIT>(j)] = a[jh];
  }
  reg_step<T, R, BIT>(a, c, ts, dead);
}

template <typename T, int R, int Q, int HOFF, int HN>
__device__ __forceinline__ void lane_step_h(cplx<T> (&a)[R], cplx<T> (&h)[HN], cplx<T> c, uint32_t ts,
                                            bool dead, int li) {
  // the history keeps the hi lane's amplitudes (zero on the lo lane): a
  // multiply by 1 or 0 on the FMA pipe instead of selects on the ALU, which
  // bounds this kernel
  const T hm = ((li >> Q) & 1) ? T(1) : T(0);
#pragma unroll
  for (int j = 0; j < R; ++j) h[HOFF + j] = mk<T>(a[j].x * hm, a[j].y * hm);
  lane_step<T, R, Q>(a, c, ts, dead, li);
}

// ---------------------------------------------------------- backward steps
template <typename T, int R, int BIT, int HOFF, int HN>
__device__ __forceinline__ cplx<T> reg_step_b(cplx<T> (&lam)[R], const cplx<T> (&h)[HN], cplx<T> c,
                                              uint32_t ts, bool dead) {
  cplx<T> t = mk<T>(T(0), T(0));
#pragma unroll
  for (int j = 0; j < R; ++j) {
    if (j & (1 << BIT)) continue;
    const int jh = j | (1 << BIT);
    cplx<T> mu = lam[j];
    if (!dead) {
      cplx<T> l1;
      if constexpr (sizeof(T) == 4)
        l1 = sign_bit_flip(lam[jh], ts * (1u << (31 - jh)));
      else
        l1 = flip_sign(lam[jh], (ts << (31 - jh)) & 0x80000000u);
      mu.x += l1.x;
      mu.y += l1.y;
    }
    const cplx<T> hv = h[HOFF + squeeze<BIT>(j)];
    t.x += mu.x * hv.x + mu.y * hv.y;
    t.y += mu.x * hv.y - mu.y * hv.x;
    lam[j] = mu;
    lam[jh] = mk<T>(c.x * mu.x + c.y * mu.y, c.x * mu.y - c.y * mu.x);  // conj(c) mu
  }
  return t;
}

template <typename T, int R, int Q, int HOFF, int HN>
__device__ __forceinline__ cplx<T> lane_step_b(cplx<T> (&lam)[R], const cplx<T> (&h)[HN], cplx<T> c,
                                               uint32_t ts, bool dead, int li) {
  const bool hi = (li >> Q) & 1;
  const uint32_t tl = hi ? ts : 0u;
  // per-step lane factors, applied by multiplies (FMA pipe) rather than
  // per-amplitude selects (ALU pipe): the hi lane's term vanishes on a
  // shrinking step, and only the hi lane takes conj(c)
  const T keepf = (dead && hi) ? T(0) : T(1);
  const cplx<T> cm = hi ? mk<T>(c.x, -c.y) : mk<T>(T(1), T(0));
  cplx<T> t = mk<T>(T(0), T(0));
#pragma unroll
  for (int j = 0; j < R; ++j) {
    cplx<T> term;
    if constexpr (sizeof(T) == 4)
      term = sign_bit_flip(lam[j], tl * (1u << (31 - j)));
    else
      term = flip_sign(lam[j], (tl << (31 - j)) & 0x80000000u);
    term = mk<T>(term.x * keepf, term.y * keepf);
    cplx<T> mu;
    mu.x = term.x + __shfl_xor_sync(0xffffffffu, term.x, 1 << Q);
    mu.y = term.y + __shfl_xor_sync(0xffffffffu, term.y, 1 << Q);
    const cplx<T> hv = h[HOFF + j];  // zero on the lo lanes
    t.x += mu.x * hv.x + mu.y * hv.y;
    t.y += mu.x * hv.y - mu.y * hv.x;
    lam[j] = mk<T>(cm.x * mu.x - cm.y * mu.y, cm.x * mu.y + cm.y * mu.x);  // conj(c) mu on the hi lane
  }
  return t;
}

template <typename T, int W, int LL> struct AdjCfg {
  static constexpr int L = 1 << LL;
  static constexpr int RB = W - LL;
  static constexpr int R = 1 << RB;
  static constexpr int RPW = 32 / L;
  using H = AdjHist<W, RB, R>;
  static constexpr int HN = H::total;
};

// per-warp carve-up of dynamic shared memory: coefficients [rpw][M],
// step tables [3][M], per-lane gradient slots [32][n_angles]
struct AdjSmem {
  static __host__ __device__ size_t al(size_t b) { return (b + 15) & ~(size_t)15; }
  static __host__ __device__ size_t coef_bytes(int M, int rpw, size_t cb) { return al((size_t)rpw * M * cb); }
  static __host__ __device__ size_t tab_bytes(int M) { return al((size_t)M * 3 * sizeof(uint32_t)); }
  static __host__ __device__ size_t bytes_per_warp(int M, int n_angles, int rpw, size_t cb, size_t gb) {
    return coef_bytes(M, rpw, cb) + tab_bytes(M) + al((size_t)32 * n_angles * gb);
  }
};

template <typename T, int W, int LL, int BIT>
__device__ __forceinline__ void adj_fwd_step(cplx<T> (&a)[AdjCfg<T, W, LL>::R],
                                             cplx<T> (&h)[AdjCfg<T, W, LL>::HN], const cplx<T> *coef,
                                             const uint32_t *smask, const uint32_t *streg, int k,
                                             int li) {
  using Cfg = AdjCfg<T, W, LL>;
  const uint32_t mask = smask[k];
  const uint32_t lp = __popc(((uint32_t)li << Cfg::RB) & mask) & 1u;
  const uint32_t ts = streg[k] ^ (0u - lp);
  const bool dead = (mask & kDead) != 0u;
  constexpr int HOFF = Cfg::H::off(BIT);
  if constexpr (BIT < Cfg::RB)
    reg_step_h<T, Cfg::R, BIT, HOFF, Cfg::HN>(a, h, coef[k], ts, dead);
  else
    lane_step_h<T, Cfg::R, BIT - Cfg::RB, HOFF, Cfg::HN>(a, h, coef[k], ts, dead, li);
}

template <typename T, int W, int LL, int BIT>
__device__ __forceinline__ void adj_bwd_step(cplx<T> (&lam)[AdjCfg<T, W, LL>::R],
                                             const cplx<T> (&h)[AdjCfg<T, W, LL>::HN],
                                             const cplx<T> *coef, const uint32_t *smask,
                                             const uint32_t *streg, const int32_t *saidx, T *sgrad,
                                             int k, int li) {
  using Cfg = AdjCfg<T, W, LL>;
  const uint32_t mask = smask[k];
  const uint32_t lp = __popc(((uint32_t)li << Cfg::RB) & mask) & 1u;
  const uint32_t ts = streg[k] ^ (0u - lp);
  const bool dead = (mask & kDead) != 0u;
  const cplx<T> c = coef[k];
  constexpr int HOFF = Cfg::H::off(BIT);
  cplx<T> t;
  if constexpr (BIT < Cfg::RB)
    t = reg_step_b<T, Cfg::R, BIT, HOFF, Cfg::HN>(lam, h, c, ts, dead);
  else
    t = lane_step_b<T, Cfg::R, BIT - Cfg::RB, HOFF, Cfg::HN>(lam, h, c, ts, dead, li);
  const int ai = saidx[k];
  if (ai >= 0) sgrad[ai] = c.x * t.y + c.y * t.x;  // Im(c t), this lane's share
}

template <typename T, int W, int LL, int... I>
__device__ __forceinline__ void adj_fwd_period(std::integer_sequence<int, I...>,
                                               cplx<T> (&a)[AdjCfg<T, W, LL>::R],
                                               cplx<T> (&h)[AdjCfg<T, W, LL>::HN], const cplx<T> *coef,
                                               const uint32_t *smask, const uint32_t *streg, int k0,
                                               int k1, int li) {
  ((k0 + I < k1 ? adj_fwd_step<T, W, LL, I>(a, h, coef, smask, streg, k0 + I, li) : void()), ...);
}

template <typename T, int W, int LL, int... I>
__device__ __forceinline__ void adj_bwd_period(std::integer_sequence<int, I...>,
                                               cplx<T> (&lam)[AdjCfg<T, W, LL>::R],
                                               const cplx<T> (&h)[AdjCfg<T, W, LL>::HN],
                                               const cplx<T> *coef, const uint32_t *smask,
                                               const uint32_t *streg, const int32_t *saidx, T *sgrad,
                                               int k0, int k1, int li) {
  ((k0 + (W - 1 - I) < k1
        ? adj_bwd_step<T, W, LL, W - 1 - I>(lam, h, coef, smask, streg, saidx, sgrad,
                                            k0 + (W - 1 - I), li)
        : void()),
   ...);
}

// squared norm of the run's window, all-reduced over its lanes (FP32/FP64 per T)
template <typename T, int R, int L>
__device__ __forceinline__ T run_norm2(const cplx<T> (&a)[R]) {
  T s = T(0);
#pragma unroll
  for (int j = 0; j < R; ++j) s += a[j].x * a[j].x + a[j].y * a[j].y;
#pragma unroll
  for (int o = 1; o < L; o <<= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  return s;
}

template <typename T>
__device__ __forceinline__ int renorm_exponent(T s) {
  if (!RealBits<T>::finite_pos(s)) return 0;
  const int f = RealBits<T>::expo(s) >> 1;
  return f > 100 ? 100 : (f < -100 ? -100 : f);
}

template <typename T, int W, int LL>
__global__ void __launch_bounds__(128) sv_adj_reg(SvAdjArgs A) {
  using Cfg = AdjCfg<T, W, LL>;
  constexpr int L = Cfg::L, RB = Cfg::RB, R = Cfg::R, RPW = Cfg::RPW, HN = Cfg::HN;
  using CT = cplx<T>;

  extern __shared__ __align__(16) unsigned char smem[];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const int sub = lane >> LL, li = lane & (L - 1);
  const int M = A.M, NA = A.n_angles;
  const size_t per_warp = AdjSmem::bytes_per_warp(M, NA, RPW, sizeof(CT), sizeof(T));
  unsigned char *wbase = smem + per_warp * wid;
  CT *s_coef = reinterpret_cast<CT *>(wbase);
  uint32_t *s_mask = reinterpret_cast<uint32_t *>(wbase + AdjSmem::coef_bytes(M, RPW, sizeof(CT)));
  uint32_t *s_treg = s_mask + M;
  int32_t *s_aidx = reinterpret_cast<int32_t *>(s_treg + M);
  T *s_grad = reinterpret_cast<T *>(wbase + AdjSmem::coef_bytes(M, RPW, sizeof(CT)) +
                                    AdjSmem::tab_bytes(M));  // [32 lanes][NA]

  for (int k = lane; k < M; k += 32) {
    const DevStep st = A.steps[k];
    s_mask[k] = st.mask;
    s_treg[k] = parity_table(st.mask & ((1u << RB) - 1u), RB);
    s_aidx[k] = st.aidx;
  }

  const int P = (M + W - 1) / W;
  const int64_t gwarp = (int64_t)blockIdx.x * (blockDim.x >> 5) + wid;
  const int64_t nwarps = (int64_t)gridDim.x * (blockDim.x >> 5);
  const int64_t slot = gwarp * RPW + sub;
  CT *ck = reinterpret_cast<CT *>(A.ckpt) + slot * (int64_t)P * (R * L);
  const int n_out = A.n_out;
  const int64_t dout = (int64_t)1 << n_out;
  const bool fid = A.J > 0;
  T *mygrad = s_grad + (size_t)lane * NA;

  for (int64_t base = gwarp * RPW; base < A.B; base += nwarps * RPW) {
    const int64_t run = base + sub;
    const bool valid = run < A.B;
    const int64_t runc = valid ? run : A.B - 1;
    const int64_t vrow = fid ? runc / A.J : runc;
    const int64_t irow = fid ? runc % A.J : (A.istride ? runc : 0);
    __syncwarp();
    for (int k = li; k < M; k += L) {
      const DevStep st = A.steps[k];
      const double th = st.aidx >= 0 ? A.angles[vrow * A.astride + st.aidx] : st.fixed;
      CT c, ph;
      sv_coef(st.plane, th, false, c, ph);
      s_coef[sub * M + k] = c;
    }
    for (int ai = 0; ai < NA; ++ai) mygrad[ai] = T(0);
    __syncwarp();
    const CT *coef = s_coef + sub * M;

    // ---- forward with period checkpoints
    CT a[R];
    {
      const CT *in = reinterpret_cast<const CT *>(A.psi_in) + irow * (fid ? ((int64_t)1 << A.n_in) : A.istride);
#pragma unroll
      for (int j = 0; j < R; ++j) {
        const int2 mp = __ldg(&A.map[(li << RB) | j]);
        a[j] = flip_sign(in[mp.x & 0x7fffffff], (uint32_t)mp.x & 0x80000000u);
      }
    }
    CT h[HN];
    for (int p = 0; p < P; ++p) {
#pragma unroll
      for (int j = 0; j < R; ++j) ck[((int64_t)p * R + j) * L + li] = a[j];
      run_period<T, W, LL, 1>(std::make_integer_sequence<int, W>{}, a, coef, s_mask, s_treg, p * W,
                           min(M, p * W + W), li);
      const int f = renorm_exponent(run_norm2<T, R, L>(a));
      if (f) {
        const T g = RealBits<T>::pow2(-f);
#pragma unroll
        for (int j = 0; j < R; ++j) a[j] = mk<T>(a[j].x * g, a[j].y * g);
      }
    }

    // ---- output, seed lambda_M
    T part = T(0);
#pragma unroll
    for (int j = 0; j < R; ++j) part += a[j].x * a[j].x + a[j].y * a[j].y;
    const T n2 = lane_group_sum<T, L>(part);  // float pairs / FP64: no FP64 pipe in the float path
    const bool ok = (n2 > T(0)) && (n2 < (sizeof(T) == 4 ? T(3.0e38f) : T(1.0e300)));
    T inv;
    if constexpr (sizeof(T) == 4) {
      float y = rsqrtf(n2);
      inv = ok ? y * (1.5f - 0.5f * n2 * y * y) : 0.f;  // one Newton step
    } else {
      inv = ok ? 1.0 / sqrt(n2) : 0.0;
    }
    CT lam[R];
    T loss_term = T(0);  // this run's share of the fidelity loss (lane li == 0)
    if (fid) {
      const CT *tg = reinterpret_cast<const CT *>(A.targets) + irow * dout;
      T pr = T(0), pi = T(0);  // a = <t|z>
#pragma unroll
      for (int j = 0; j < R; ++j) {
        const int y = __ldg(&A.map[(li << RB) | j]).y;
        if (y >= 0) {
          const CT t = tg[y];
          pr += t.x * a[j].x + t.y * a[j].y;
          pi += t.x * a[j].y - t.y * a[j].x;
        }
      }
      const T ar = lane_group_sum<T, L>(pr * inv);
      const T ai_ = lane_group_sum<T, L>(pi * inv);
      const T F = ar * ar + ai_ * ai_;
      const T wJ = T(1) / (T)A.J;
      loss_term = (valid && li == 0 && ok) ? (T(1) - F) * wJ : T(0);
      // lambda = (2/J)(F z - a t) / |psi|
      const T k2 = T(2) * wJ * inv;
      const T fz = F * inv;
#pragma unroll
      for (int j = 0; j < R; ++j) {
        const int y = __ldg(&A.map[(li << RB) | j]).y;
        if (y >= 0 && ok) {
          const CT t = tg[y];
          const T atr = (T)ar * t.x - (T)ai_ * t.y, ati = (T)ar * t.y + (T)ai_ * t.x;
          lam[j] = mk<T>(k2 * (fz * a[j].x - atr), k2 * (fz * a[j].y - ati));
        } else {
          lam[j] = mk<T>(T(0), T(0));
        }
      }
    } else {
      const CT *go = reinterpret_cast<const CT *>(A.grad_out) + runc * dout;
      T zr = T(0);
#pragma unroll
      for (int j = 0; j < R; ++j) {
        const int y = __ldg(&A.map[(li << RB) | j]).y;
        if (y >= 0) zr += a[j].x * go[y].x + a[j].y * go[y].y;
      }
      const T zg = lane_group_sum<T, L>(zr * inv);  // Re <z|g>
      const T zgi = zg * inv;
#pragma unroll
      for (int j = 0; j < R; ++j) {
        const int y = __ldg(&A.map[(li << RB) | j]).y;
        if (y >= 0 && ok) {
          const CT g = go[y];
          lam[j] = mk<T>(inv * (g.x - zgi * a[j].x), inv * (g.y - zgi * a[j].y));
        } else {
          lam[j] = mk<T>(T(0), T(0));
        }
      }
    }

    // ---- backward: recompute each period from its checkpoint, then reverse it
    for (int p = P - 1; p >= 0; --p) {
#pragma unroll
      for (int j = 0; j < R; ++j) a[j] = ck[((int64_t)p * R + j) * L + li];
      const int k0 = p * W, k1 = min(M, p * W + W);
      adj_fwd_period<T, W, LL>(std::make_integer_sequence<int, W>{}, a, h, coef, s_mask, s_treg, k0,
                               k1, li);
      const int f = renorm_exponent(run_norm2<T, R, L>(a));
      if (f) {
        const T g = RealBits<T>::pow2(-f);
#pragma unroll
        for (int j = 0; j < R; ++j) lam[j] = mk<T>(lam[j].x * g, lam[j].y * g);
      }
      adj_bwd_period<T, W, LL>(std::make_integer_sequence<int, W>{}, lam, h, coef, s_mask, s_treg,
                               s_aidx, mygrad, k0, k1, li);
    }

    // ---- gradient: sum the lane slots (float pairs in the float path)
    if (fid && !(valid && ok)) {  // a failed run adds nothing
      for (int ai = 0; ai < NA; ++ai) mygrad[ai] = T(0);
    }
    __syncwarp();
    const int64_t last = (base + RPW <= A.B ? base + RPW : A.B) - 1;
    if (fid && (last / A.J) == (base / A.J)) {
      // every run of this iteration uses one angle vector: sum all 32 slots,
      // one FP64 atomic per angle and warp instead of one per run
      const int64_t v0 = base / A.J;
      for (int ai = lane; ai < NA; ai += 32) {
        if constexpr (sizeof(T) == 4) {
          float hi = 0.f, lo = 0.f;
          for (int l = 0; l < 32; ++l) two_sum_acc(hi, lo, s_grad[(size_t)l * NA + ai], 0.f);
          atomicAdd(&A.grad[v0 * NA + ai], (double)hi + (double)lo);
        } else {
          double g = 0.0;
          for (int l = 0; l < 32; ++l) g += s_grad[(size_t)l * NA + ai];
          atomicAdd(&A.grad[v0 * NA + ai], g);
        }
      }
      if constexpr (sizeof(T) == 4) {
        float hi = loss_term, lo = 0.f;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
          const float oh = __shfl_xor_sync(0xffffffffu, hi, o);
          const float ol = __shfl_xor_sync(0xffffffffu, lo, o);
          two_sum_acc(hi, lo, oh, ol);
        }
        if (lane == 0) atomicAdd(&A.loss[v0], (double)hi + (double)lo);
      } else {
        T l2 = loss_term;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) l2 += __shfl_xor_sync(0xffffffffu, l2, o);
        if (lane == 0) atomicAdd(&A.loss[v0], (double)l2);
      }
    } else if (valid && ok) {
      const T *rs = s_grad + (size_t)(sub * L) * NA;
      for (int ai = li; ai < NA; ai += L) {
        double g;
        if constexpr (sizeof(T) == 4) {
          float hi = 0.f, lo = 0.f;
          for (int l = 0; l < L; ++l) two_sum_acc(hi, lo, rs[(size_t)l * NA + ai], 0.f);
          g = (double)hi + (double)lo;
        } else {
          g = 0.0;
          for (int l = 0; l < L; ++l) g += rs[(size_t)l * NA + ai];
        }
        if (fid)
          atomicAdd(&A.grad[vrow * NA + ai], g);
        else
          A.grad[run * NA + ai] = g;
      }
      if (fid && li == 0) atomicAdd(&A.loss[vrow], (double)loss_term);
    } else if (valid && !fid) {
      for (int ai = li; ai < NA; ai += L) A.grad[run * NA + ai] = NAN;
    }
    if (valid && li == 0 && A.status)
      A.status[run] = ok ? MBQC_RUN_OK : (isnan(n2) ? MBQC_RUN_NAN : MBQC_RUN_ZERO_NORM);
  }
}

}  // namespace mbqc
