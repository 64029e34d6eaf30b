// Wide-window statevector sweep (windows 8..30): the state streams through a
// device workspace in passes of several fused steps.
//
// The window of every run is a 2^w complex64 vector in the workspace.  A pass
// applies consecutive steps to tiles whose lanes are index bits 0..4 (32
// consecutive complex64: one fully coalesced 256-byte access per register):
//   * windows >= 10, mixed pass: up to ten steps of the form high* low* high*
//     (at most five high bits, >= 5, and five low bits).  A warp's tile is
//     32 x 32: registers = the five high bits, so high steps are in-register
//     pair updates; for the low steps the tile is transposed through shared
//     memory (registers = bits 0..4) and back.  Warps are persistent over a
//     contiguous range of tiles and the next tile's loads are asynchronous
//     copies into shared memory issued before the current tile is computed;
//   * windows 8..9: high passes (up to five high bits in registers) and low
//     passes (butterflies over the lane bits, one xor-shuffle per step).
// Per pass and run, the squared norm is accumulated (FP32 per warp, FP64
// atomics per run) and the next pass rescales by an exact power of two, so
// amplitudes never under- or overflow and the log-probability bookkeeping is
// exact.  One init kernel builds the first window, the passes follow, one
// epilogue kernel normalises (float-pair sum: FP64-level accuracy), applies
// the reference global phase and gathers the outputs.
#include <cuda_runtime.h>

#include <algorithm>
#include <type_traits>
#include <vector>

#include "dispatch.h"
#include "sv_reg.cuh"

namespace mbqc {

constexpr int kStreamMinWindow = 8;
constexpr int kLowLanes = 5;    // index bits 0..4 are lane bits
constexpr int kLowRegs = 3;     // extra register bits of a low pass

struct StreamArgs {
  const DevStep *steps;  // this circuit's steps
  int W, M, n_in, n_out;
  int64_t B;
  const double *angles;
  int64_t astride;
  const float2 *psi_in;
  int64_t istride;
  float2 *state;   // [B][2^W]
  double *norms;   // [3][B]
  int32_t *expo;   // [B] total applied exponent
  int8_t in_bits[32];
  int8_t out_bits[32];
  uint32_t init_cz[32];
};

struct PassDesc {
  int k0, nsteps, index;  // first step, steps in the pass, pass number
  int bits[5];            // active physical bits in step order
  int npas;               // passive register bits (memory-level parallelism only)
  int pbits[4];
};

// Mixed pass (windows >= 10): up to ten consecutive steps, n1 on high bits,
// then nl on low bits (0..4), then n2 on high bits.  The tile is 32 x 32:
// lanes = index bits 0..4, registers = the five register bits rbits (the
// pass's high bits in step order, padded with passive bits).  High steps are
// register pair updates; for the low steps the tile is transposed through
// shared memory (registers = bits 0..4) and back.  Everything that depends
// only on the pass is computed on the host.
struct MixDesc {
  int k0, nsteps, index;  // nsteps = n1 + nl + n2
  int n1, nl, n2;
  uint32_t bv[5];     // 1 << rbits[i]
  int lbits[5];       // low bits of the nl low steps, in step order
  uint32_t mask[10];  // step masks (dead flag in bit 31)
  uint32_t ptab[10];  // sign pattern over the five register-side bits of each step
  int nrng;           // tile bits: ranges of free index bits (>= 5, not registers)
  int rpos[6], rlen[6];
};

__device__ __forceinline__ uint32_t scatter_bits(uint32_t v, const int *bits, int n) {
  uint32_t r = 0;
  for (int i = 0; i < n; ++i) r |= ((v >> i) & 1u) << bits[i];
  return r;
}

__global__ void stream_init(StreamArgs a) {
  const int64_t total = a.B << a.W;
  const uint32_t wmask = (a.W >= 32) ? 0xffffffffu : ((1u << a.W) - 1u);
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < total;
       e += (int64_t)gridDim.x * blockDim.x) {
    const int64_t run = e >> a.W;
    const uint32_t idx = (uint32_t)e & wmask;
    const int x = gather_bits(idx, a.in_bits, a.n_in);
    const uint32_t par = init_parity(idx, a.init_cz, a.W);
    const float2 v = a.psi_in[(a.istride ? run * a.istride : 0) + x];
    a.state[e] = flip_sign(v, par << 31);
  }
  for (int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; r < a.B;
       r += (int64_t)gridDim.x * blockDim.x) {
    a.norms[r] = 0.0;              // accumulated by pass 0
    a.norms[2 * a.B + r] = 1.0;    // "previous pass" of pass 0: no rescale
    a.expo[r] = 0;
  }
}

// per-run scale for the pass from the norm the previous pass accumulated:
// half its binary exponent, read from the double's bits on the integer ALU
// (every thread computes it; FP64 instructions here kept GB300's narrow FP64
// pipe a fifth busy)
__device__ __forceinline__ int pass_exponent(const StreamArgs &a, int index, int64_t run) {
  const long long b = __double_as_longlong(a.norms[(int64_t)((index + 2) % 3) * a.B + run]);
  const int ef = (int)((b >> 52) & 0x7ff);
  if (b <= 0 || ef == 0 || ef == 0x7ff) return 0;  // negative, zero, subnormal, inf or NaN
  const int e = ((ef - 1022) - 1) >> 1;            // frexp exponent is ef - 1022
  return e > 100 ? 100 : (e < -100 ? -100 : e);
}

template <typename D>
__device__ __forceinline__ void pass_bookkeeping(const StreamArgs &a, const D &d, int64_t run,
                                                 bool tile0, int lane, int f, float part) {
#pragma unroll
  for (int o = 16; o >= 1; o >>= 1) part += __shfl_xor_sync(0xffffffffu, part, o);
  if (lane == 0) {
    atomicAdd(&a.norms[(int64_t)(d.index % 3) * a.B + run], (double)part);
    if (tile0) {
      a.norms[(int64_t)((d.index + 1) % 3) * a.B + run] = 0.0;
      a.expo[run] += f;
    }
  }
}

// lane j (< nsteps) holds the coefficient of the pass's step j for this warp's run
template <typename D>
__device__ __forceinline__ float2 lane_coef(const StreamArgs &a, const D &d, int64_t run, int lane) {
  float2 c = make_float2(1.f, 0.f), ph;
  if (lane < d.nsteps) {
    const DevStep st = a.steps[d.k0 + lane];
    const double th = st.aidx >= 0 ? a.angles[run * a.astride + st.aidx] : st.fixed;
    sv_coef(st.plane, th, false, c, ph);
  }
  return c;
}

__device__ __forceinline__ float2 bcast(float2 c, int j) {
  return make_float2(__shfl_sync(0xffffffffu, c.x, j), __shfl_sync(0xffffffffu, c.y, j));
}

template <int T, int P>
__global__ void __launch_bounds__(128) stream_pass_high(StreamArgs a, PassDesc d) {
  constexpr int NR = T + P;  // register bits: T active (stepped), P passive
  constexpr int R = 1 << NR;
  const int lane = threadIdx.x & 31;
  const int64_t gw = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int tlog = a.W - kLowLanes - NR;
  const int64_t run = gw >> tlog;
  if (run >= a.B) return;
  const uint32_t tile = (uint32_t)(gw & ((1ll << tlog) - 1));
  int rbits[NR];
#pragma unroll
  for (int i = 0; i < NR; ++i) rbits[i] = i < T ? d.bits[i] : d.pbits[i - T];
  uint32_t excl = 0;
#pragma unroll
  for (int i = 0; i < NR; ++i) excl |= 1u << rbits[i];
  uint32_t base = 0;
  for (int b = kLowLanes, t = 0; b < a.W; ++b)
    if (!((excl >> b) & 1u)) base |= ((tile >> t++) & 1u) << b;
  base |= (uint32_t)lane;
  float2 *st = a.state + (run << a.W);
  const int f = pass_exponent(a, d.index, run);
  const float g = RealBits<float>::pow2(-f);
  // a pass's active bits are consecutive (passes split at the lane bits), so
  // without passive bits register r sits at base + r << bits[0]: one
  // multiply-add per address instead of a runtime bit scatter
  const uint32_t stride = 1u << rbits[0];
  auto addr = [&](int r) -> uint32_t {
    if constexpr (P == 0)
      return base + (uint32_t)r * stride;
    else
      return base | scatter_bits(r, rbits, NR);
  };
  float2 v[R];
#pragma unroll
  for (int r = 0; r < R; ++r) {
    const float2 x = st[addr(r)];
    v[r] = make_float2(x.x * g, x.y * g);
  }
  const float2 cl = lane_coef(a, d, run, lane);
#define MBQC_HSTEP(J)                                                                           \
  if (J < d.nsteps) {                                                                           \
    const float2 c = bcast(cl, J);                                                              \
    const uint32_t m = a.steps[d.k0 + J].mask;                                                  \
    uint32_t cm = 0;                                                                            \
    for (int i = 0; i < NR; ++i) cm |= ((m >> rbits[i]) & 1u) << i;                             \
    const uint32_t ts = parity_table(cm, NR) ^ (0u - (__popc(base & m & ~kDead) & 1u));         \
    reg_step<float, R, J < T ? J : 0>(v, c, ts, (m & kDead) != 0u);                             \
  }
  MBQC_HSTEP(0)
  if constexpr (T > 1) { MBQC_HSTEP(1) }
  if constexpr (T > 2) { MBQC_HSTEP(2) }
  if constexpr (T > 3) { MBQC_HSTEP(3) }
  if constexpr (T > 4) { MBQC_HSTEP(4) }
#undef MBQC_HSTEP
  float part[R];
#pragma unroll
  for (int r = 0; r < R; ++r) part[r] = v[r].x * v[r].x + v[r].y * v[r].y;
#pragma unroll
  for (int h = R / 2; h >= 1; h >>= 1)
#pragma unroll
    for (int r = 0; r < h; ++r) part[r] += part[r + h];
#pragma unroll
  for (int r = 0; r < R; ++r) st[addr(r)] = v[r];
  pass_bookkeeping(a, d, run, tile == 0, lane, f, part[0]);
}

// passive register bits for a high pass of T steps: the lowest free bits >= 5,
// up to 4 register bits in total
static void add_passive(PassDesc &d, int W) {
  const int T = d.nsteps;
  int want = 4 - T;
  d.npas = 0;
  if (want <= 0) return;
  uint32_t act = 0;
  for (int i = 0; i < T; ++i) act |= 1u << d.bits[i];
  for (int b = kLowLanes; b < W && d.npas < want; ++b)
    if (!((act >> b) & 1u)) d.pbits[d.npas++] = b;
}

typedef void (*high_pass_fn)(StreamArgs, PassDesc);

static high_pass_fn high_pass(int T, int P) {
  switch (T * 8 + P) {
    case 8: return stream_pass_high<1, 0>;
    case 9: return stream_pass_high<1, 1>;
    case 10: return stream_pass_high<1, 2>;
    case 11: return stream_pass_high<1, 3>;
    case 16: return stream_pass_high<2, 0>;
    case 17: return stream_pass_high<2, 1>;
    case 18: return stream_pass_high<2, 2>;
    case 24: return stream_pass_high<3, 0>;
    case 25: return stream_pass_high<3, 1>;
    case 32: return stream_pass_high<4, 0>;
    case 40: return stream_pass_high<5, 0>;
    default: return nullptr;
  }
}

__global__ void __launch_bounds__(128) stream_pass_low(StreamArgs a, PassDesc d) {
  constexpr int R = 1 << kLowRegs;
  const int lane = threadIdx.x & 31;
  const int64_t gw = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int tlog = a.W - kLowLanes - kLowRegs;
  const int64_t run = gw >> tlog;
  if (run >= a.B) return;
  const uint32_t tile = (uint32_t)(gw & ((1ll << tlog) - 1));
  // registers: bits 5..7; tile: bits 8..W-1
  const uint32_t base = (tile << (kLowLanes + kLowRegs)) | (uint32_t)lane;
  float2 *st = a.state + (run << a.W);
  const int f = pass_exponent(a, d.index, run);
  const float g = RealBits<float>::pow2(-f);
  float2 v[R];
#pragma unroll
  for (int r = 0; r < R; ++r) {
    const float2 x = st[base | ((uint32_t)r << kLowLanes)];
    v[r] = make_float2(x.x * g, x.y * g);
  }
  const float2 cl = lane_coef(a, d, run, lane);
  for (int j = 0; j < d.nsteps; ++j) {
    const float2 c = bcast(cl, j);
    const uint32_t m = a.steps[d.k0 + j].mask;
    const uint32_t cm = (m >> kLowLanes) & (R - 1u);
    const uint32_t ts = parity_table(cm, kLowRegs) ^ (0u - (__popc(base & m & ~kDead) & 1u));
    const bool dead = (m & kDead) != 0u;
    switch (d.bits[j]) {
      case 0: lane_step<float, R, 0>(v, c, ts, dead, lane); break;
      case 1: lane_step<float, R, 1>(v, c, ts, dead, lane); break;
      case 2: lane_step<float, R, 2>(v, c, ts, dead, lane); break;
      case 3: lane_step<float, R, 3>(v, c, ts, dead, lane); break;
      default: lane_step<float, R, 4>(v, c, ts, dead, lane); break;
    }
  }
  float part = 0.f;
#pragma unroll
  for (int r = 0; r < R; ++r) {
    part += v[r].x * v[r].x + v[r].y * v[r].y;
    st[base | ((uint32_t)r << kLowLanes)] = v[r];
  }
  pass_bookkeeping(a, d, run, tile == 0, lane, f, part);
}

// Asynchronous 16-byte global -> shared copies (cached in L2 only).  Each
// thread waits for its own copies; a __syncwarp then makes the whole warp's
// copies visible to every lane.
__device__ __forceinline__ void cp_async16(void *smem, const void *gmem) {
  const unsigned s = (unsigned)__cvta_generic_to_shared(smem);
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(s), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait_prev() { asm volatile("cp.async.wait_group 1;" ::: "memory"); }

constexpr int kMixWarps = 4;
// shared-memory slot of tile element (row r = register pattern, column c =
// index bits 0..4): 16-byte pairs of a row XOR-swizzled by the row, so row
// accesses and the 16-byte copies are conflict free and column accesses take
// two wavefronts per 128 bytes
__device__ __forceinline__ int tslot(int r, int c) { return r * 32 + ((((c >> 1) ^ (r & 15)) << 1) | (c & 1)); }

// Persistent warps, each owning a contiguous range of tiles (consecutive
// tiles mostly share a run, whose scale and step coefficients are reused);
// while a warp computes tile i, tile i + 1 is already on its way into the
// warp's other shared-memory buffer.
__global__ void __launch_bounds__(32 * kMixWarps) stream_pass_mixed(StreamArgs a, MixDesc d) {
  extern __shared__ __align__(16) float2 s_mix[];  // [warp][2][32 x 32]
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  float2 *buf = s_mix + (size_t)wid * 2 * 1024;
  const int tlog = a.W - 10;
  const int64_t n_tiles = a.B << tlog;
  const int64_t n_warps = (int64_t)gridDim.x * kMixWarps;
  const int64_t w = (int64_t)blockIdx.x * kMixWarps + wid;
  const int64_t g0 = w * n_tiles / n_warps, g1 = (w + 1) * n_tiles / n_warps;
  auto roff = [&](int r) -> uint32_t {  // index bits of register pattern r
    uint32_t o = 0;
#pragma unroll
    for (int i = 0; i < 5; ++i)
      if ((r >> i) & 1) o |= d.bv[i];
    return o;
  };
  auto tile_bits = [&](int64_t g) -> uint32_t {
    uint32_t t = (uint32_t)(g & ((1ll << tlog) - 1)), tb = 0;
    for (int i = 0; i < d.nrng; ++i) {
      tb |= (t & ((1u << d.rlen[i]) - 1u)) << d.rpos[i];
      t >>= d.rlen[i];
    }
    return tb;
  };
  const uint32_t lane_roff = roff(lane);
  auto issue = [&](int64_t g, float2 *dst) {  // lane: pair lane & 15 of rows 2i + (lane >> 4)
    const float2 *st = a.state + ((g >> tlog) << a.W) + tile_bits(g);
    const int pr = lane & 15;
#pragma unroll
    for (int i = 0; i < 16; ++i) {
      const int r = 2 * i + (lane >> 4);
      cp_async16(dst + r * 32 + ((pr ^ (r & 15)) << 1), st + (roff(r) | (uint32_t)(2 * pr)));
    }
  };

  if (g0 < g1) issue(g0, buf);
  cp_async_commit();
  int64_t cur_run = -1;
  int f = 0;
  float gsc = 1.f;
  float2 cl = make_float2(1.f, 0.f);
  float part = 0.f;
  bool tile0 = false;
  for (int64_t g = g0; g < g1; ++g) {
    float2 *cur = buf + ((g - g0) & 1) * 1024;
    if (g + 1 < g1) issue(g + 1, buf + ((g + 1 - g0) & 1) * 1024);
    cp_async_commit();
    const int64_t run = g >> tlog;
    if (run != cur_run) {
      if (cur_run >= 0) pass_bookkeeping(a, d, cur_run, tile0, lane, f, part);
      cur_run = run;
      part = 0.f;
      tile0 = false;
      f = pass_exponent(a, d.index, run);
      gsc = RealBits<float>::pow2(-f);
      cl = lane_coef(a, d, run, lane);
    }
    tile0 = tile0 || (g & ((1ll << tlog) - 1)) == 0;
    const uint32_t tb = tile_bits(g);
    const uint32_t nbase = tb | (uint32_t)lane;   // normal layout: lane = bits 0..4
    const uint32_t tbase = tb | lane_roff;        // transposed: lane = register pattern
    cp_async_wait_prev();
    __syncwarp();
    float2 v[32];
    const bool start_low = d.n1 == 0 && d.nl > 0;
    if (start_low) {
#pragma unroll
      for (int c = 0; c < 32; ++c) {
        const float2 x = cur[tslot(lane, c)];
        v[c] = make_float2(x.x * gsc, x.y * gsc);
      }
    } else {
#pragma unroll
      for (int r = 0; r < 32; ++r) {
        const float2 x = cur[tslot(r, lane)];
        v[r] = make_float2(x.x * gsc, x.y * gsc);
      }
    }
    auto hstep = [&](auto jc, int j) {  // high step j of the pass on register bit J
      constexpr int J = decltype(jc)::value;
      const uint32_t m = d.mask[j];
      const uint32_t ts = d.ptab[j] ^ (0u - (__popc(nbase & m & ~kDead) & 1u));
      reg_step<float, 32, J>(v, bcast(cl, j), ts, (m & kDead) != 0u);
    };
#define MBQC_MSTEP(J) \
  if (J < d.n1) hstep(std::integral_constant<int, J>{}, J);
    MBQC_MSTEP(0)
    MBQC_MSTEP(1)
    MBQC_MSTEP(2)
    MBQC_MSTEP(3)
    MBQC_MSTEP(4)
#undef MBQC_MSTEP
    if (d.nl > 0) {
      if (!start_low) {  // to the transposed layout
        __syncwarp();
#pragma unroll
        for (int r = 0; r < 32; ++r) cur[tslot(r, lane)] = v[r];
        __syncwarp();
#pragma unroll
        for (int c = 0; c < 32; ++c) v[c] = cur[tslot(lane, c)];
      }
      for (int j = 0; j < d.nl; ++j) {
        const int js = d.n1 + j;
        const uint32_t m = d.mask[js];
        const uint32_t ts = d.ptab[js] ^ (0u - (__popc(tbase & m & ~kDead) & 1u));
        const float2 c = bcast(cl, js);
        const bool dead = (m & kDead) != 0u;
        switch (d.lbits[j]) {
          case 0: reg_step<float, 32, 0>(v, c, ts, dead); break;
          case 1: reg_step<float, 32, 1>(v, c, ts, dead); break;
          case 2: reg_step<float, 32, 2>(v, c, ts, dead); break;
          case 3: reg_step<float, 32, 3>(v, c, ts, dead); break;
          default: reg_step<float, 32, 4>(v, c, ts, dead); break;
        }
      }
      __syncwarp();  // back to the normal layout
#pragma unroll
      for (int c = 0; c < 32; ++c) cur[tslot(lane, c)] = v[c];
      __syncwarp();
#pragma unroll
      for (int r = 0; r < 32; ++r) v[r] = cur[tslot(r, lane)];
    }
    // the second high run: register bit J is pass step nl + J
#define MBQC_MSTEP(J) \
  if (J >= d.n1 && J < d.n1 + d.n2) hstep(std::integral_constant<int, J>{}, d.nl + J);
    MBQC_MSTEP(0)
    MBQC_MSTEP(1)
    MBQC_MSTEP(2)
    MBQC_MSTEP(3)
    MBQC_MSTEP(4)
#undef MBQC_MSTEP
    float2 *st = a.state + (run << a.W);
#pragma unroll
    for (int r = 0; r < 32; ++r) {
      part += v[r].x * v[r].x + v[r].y * v[r].y;
      st[nbase | roff(r)] = v[r];
    }
    __syncwarp();  // every lane is done with `cur` before the copy two tiles on refills it
  }
  if (cur_run >= 0) pass_bookkeeping(a, d, cur_run, tile0, lane, f, part);
}

// Output index y -> window index through four byte-wide lookup tables
// (byte t of y selects s_tab[t][...]), built per block in shared memory.
__device__ __forceinline__ uint32_t out_to_window(const uint32_t (*tab)[256], uint32_t y) {
  return tab[0][y & 255u] | tab[1][(y >> 8) & 255u] | tab[2][(y >> 16) & 255u] | tab[3][y >> 24];
}

__global__ void __launch_bounds__(1024) stream_epilogue(StreamArgs a, float2 *out, uint32_t flags,
                                                        int32_t lp_const, double *logprob,
                                                        int32_t *status) {
  __shared__ uint32_t s_tab[4][256];
  __shared__ float2 s_red[32];
  __shared__ float2 s_ph[32];
  const int64_t run = blockIdx.x;
  if (run >= a.B) return;
  const float2 *st = a.state + (run << a.W);
  const int n_out = a.n_out, dout = 1 << n_out;
  const int tid = threadIdx.x, nthr = blockDim.x;
  for (int v = tid; v < 4 * 256; v += nthr) {
    const int t = v >> 8, byte = v & 255;
    uint32_t w = 0;
    for (int j = 0; j < n_out; ++j) {
      const int ybit = n_out - 1 - j;  // output j is bit n_out-1-j of y
      if ((ybit >> 3) == t && ((byte >> (ybit & 7)) & 1)) w |= 1u << a.out_bits[j];
    }
    s_tab[t][byte] = w;
  }
  // phase product over this thread's steps
  float2 ph = make_float2(1.f, 0.f);
  if (flags & MBQC_F_REF_PHASE) {
    for (int k = tid; k < a.M; k += nthr) {
      const DevStep s = a.steps[k];
      const double th = s.aidx >= 0 ? a.angles[run * a.astride + s.aidx] : s.fixed;
      float2 c, p;
      sv_coef(s.plane, th, true, c, p);
      ph = cmul(ph, p);
    }
  }
  __syncthreads();
  // squared norm as an error-free float pair (FP64-level accuracy without
  // the FP64 pipe)
  float nh = 0.f, nl = 0.f;
  for (int y = tid; y < dout; y += nthr) {
    const float2 x = st[out_to_window(s_tab, (uint32_t)y)];
    two_sum_acc(nh, nl, x.x * x.x + x.y * x.y, 0.f);
  }
#pragma unroll
  for (int o = 16; o >= 1; o >>= 1) {
    two_sum_acc(nh, nl, __shfl_xor_sync(0xffffffffu, nh, o), __shfl_xor_sync(0xffffffffu, nl, o));
    float2 q;
    q.x = __shfl_xor_sync(0xffffffffu, ph.x, o);
    q.y = __shfl_xor_sync(0xffffffffu, ph.y, o);
    ph = cmul(ph, q);
  }
  if ((tid & 31) == 0) {
    s_red[tid >> 5] = make_float2(nh, nl);
    s_ph[tid >> 5] = ph;
  }
  __syncthreads();
  float2 n2p = s_red[0];
  float2 phase = s_ph[0];
  for (int i = 1; i < (nthr >> 5); ++i) {
    two_sum_acc(n2p.x, n2p.y, s_red[i].x, s_red[i].y);
    phase = cmul(phase, s_ph[i]);
  }
  const float n2 = n2p.x + n2p.y;
  const bool ok = (n2 > 0.f) && (n2 < 3.0e38f);
  float inv = rsqrtf(n2);
  inv = ok ? inv * (1.5f - 0.5f * n2 * inv * inv) : NAN;  // one Newton step
  const float2 sc = make_float2(phase.x * inv, phase.y * inv);
  for (int y = tid; y < dout; y += nthr)
    out[run * dout + y] = cmul(st[out_to_window(s_tab, (uint32_t)y)], sc);
  if (tid == 0) {
    if (status) status[run] = ok ? MBQC_RUN_OK : (isnan(n2) ? MBQC_RUN_NAN : MBQC_RUN_ZERO_NORM);
    if (logprob) {
      double nin = 0.0;
      for (int x = 0; x < (1 << a.n_in); ++x) {
        const float2 v = a.psi_in[(a.istride ? run * a.istride : 0) + x];
        nin += (double)v.x * v.x + (double)v.y * v.y;
      }
      const double n2d = (double)n2p.x + (double)n2p.y;
      logprob[run] = log(n2d) - log(nin) + 0.6931471805599453 * (2.0 * a.expo[run] + lp_const);
    }
  }
}

// bit r of the result: parity of popcount(r & side), r over 5-bit patterns
static uint32_t host_parity_table(uint32_t side) {
  uint32_t t = 0;
  for (int r = 0; r < 32; ++r)
    if (__builtin_popcount((unsigned)r & side) & 1) t |= 1u << r;
  return t;
}

// mixed pass schedule (windows >= 10): greedy runs of consecutive steps of
// the form high* low* high* with at most five high and five low bits; the
// register bits are the high bits in step order, padded with the lowest free
// high bits
static std::vector<MixDesc> make_mixed_passes(int W, int M, const DevStep *steps) {
  std::vector<MixDesc> out;
  int k = 0;
  while (k < M) {
    MixDesc d{};
    int rbits[5] = {0, 0, 0, 0, 0};
    d.k0 = k;
    d.index = (int)out.size();
    int phase = 0, nh = 0;  // phase 0: first high run, 1: low run, 2: second high run
    while (k < M) {
      const int b = k % W;
      if (b < kLowLanes) {
        if (phase == 2 || d.nl == 5) break;
        phase = 1;
        d.lbits[d.nl++] = b;
      } else {
        if (nh == 5) break;
        if (phase == 1) phase = 2;
        rbits[nh++] = b;
        if (phase == 0)
          ++d.n1;
        else
          ++d.n2;
      }
      ++k;
    }
    d.nsteps = k - d.k0;
    uint32_t used = 0;
    for (int i = 0; i < nh; ++i) used |= 1u << rbits[i];
    for (int b = kLowLanes; b < W && nh < 5; ++b)
      if (!((used >> b) & 1u)) rbits[nh++] = b;
    used = 31u;
    for (int i = 0; i < 5; ++i) {
      d.bv[i] = 1u << rbits[i];
      used |= d.bv[i];
    }
    for (int j = 0; j < d.nsteps; ++j) {
      const uint32_t m = steps[d.k0 + j].mask;
      d.mask[j] = m;
      uint32_t side = 0;  // the step's mask bits on the register side of its layout
      if (j >= d.n1 && j < d.n1 + d.nl) {
        side = m & 31u;
      } else {
        for (int i = 0; i < 5; ++i)
          if (m & d.bv[i]) side |= 1u << i;
      }
      d.ptab[j] = host_parity_table(side);
    }
    for (int b = kLowLanes; b < W;) {  // free bits as ranges
      if ((used >> b) & 1u) {
        ++b;
        continue;
      }
      int e = b;
      while (e < W && !((used >> e) & 1u)) ++e;
      d.rpos[d.nrng] = b;
      d.rlen[d.nrng] = e - b;
      ++d.nrng;
      b = e;
    }
    out.push_back(d);
  }
  return out;
}

// pass schedule: consecutive steps grouped by low (< 5) / high bits, <= 5 each
static std::vector<PassDesc> make_passes(int W, int M) {
  std::vector<PassDesc> out;
  int k = 0;
  while (k < M) {
    PassDesc d{};
    d.k0 = k;
    const bool low = (k % W) < kLowLanes;
    int n = 0;
    while (k < M && n < 5 && (((k % W) < kLowLanes) == low)) {
      d.bits[n++] = k % W;
      ++k;
    }
    d.nsteps = n;
    d.index = (int)out.size();
    out.push_back(d);
  }
  return out;
}

static size_t stream_ws_bytes(int W, int64_t B) {
  return (size_t)B * ((size_t)1 << W) * sizeof(float2) + (size_t)3 * B * sizeof(double) +
         (size_t)B * sizeof(int32_t) + 256;
}

}  // namespace mbqc

using namespace mbqc;

extern "C" {

int mbqc_sv_stream_workspace(const mbqc_plan *plan, int64_t batch, size_t *bytes) {
  if (!plan || !bytes || batch < 0) return fail(MBQC_E_INVALID, "stream_workspace: bad arguments");
  const DevCircuit &hc = host_circuit(plan, 0);
  if (hc.w < kStreamMinWindow)
    return fail(MBQC_E_UNSUPPORTED, "stream_workspace: window %d < %d", hc.w, kStreamMinWindow);
  *bytes = stream_ws_bytes(hc.w, batch);
  return MBQC_OK;
}

int mbqc_sv_forward_stream(const mbqc_plan *plan, int64_t batch, const double *angles,
                           int64_t angle_stride, const float *psi_in, int64_t in_stride,
                           float *psi_out, uint32_t flags, double *logprob, int32_t *status,
                           void *workspace, size_t workspace_bytes, mbqc_stream_t stream) {
  if (!plan) return fail(MBQC_E_INVALID, "sv_forward_stream: null plan");
  if (batch < 0) return fail(MBQC_E_INVALID, "sv_forward_stream: negative batch");
  if (batch == 0) return MBQC_OK;
  const DevCircuit &hc = host_circuit(plan, 0);
  if (hc.w < kStreamMinWindow)
    return fail(MBQC_E_UNSUPPORTED, "sv_forward_stream: window %d < %d", hc.w, kStreamMinWindow);
  if (!psi_in || !psi_out) return fail(MBQC_E_INVALID, "sv_forward_stream: null state buffer");
  if (!hc.sv_planes_ok)
    return fail(MBQC_E_UNSUPPORTED, "sv_forward_stream: statevector steps in XY, X or Y only");
  if (hc.n_angles > 0 && (!angles || angle_stride < hc.n_angles))
    return fail(MBQC_E_INVALID, "sv_forward_stream: bad angle array");
  if (in_stride != 0 && in_stride < ((int64_t)1 << hc.n_in))
    return fail(MBQC_E_INVALID, "sv_forward_stream: input stride too small");
  const size_t need = stream_ws_bytes(hc.w, batch);
  if (!workspace || workspace_bytes < need)
    return fail(MBQC_E_INVALID, "sv_forward_stream: workspace of %zu bytes, %zu needed", workspace_bytes,
                need);
  const PlanView v = view_of(plan);
  StreamArgs a{};
  a.steps = v.d_steps + hc.step_off;
  a.W = hc.w;
  a.M = hc.n_steps;
  a.n_in = hc.n_in;
  a.n_out = hc.n_out;
  a.B = batch;
  a.angles = angles;
  a.astride = angle_stride;
  a.psi_in = reinterpret_cast<const float2 *>(psi_in);
  a.istride = in_stride;
  char *ws = static_cast<char *>(workspace);
  a.state = reinterpret_cast<float2 *>(ws);
  size_t off = (size_t)batch * ((size_t)1 << hc.w) * sizeof(float2);
  a.norms = reinterpret_cast<double *>(ws + off);
  off += (size_t)3 * batch * sizeof(double);
  a.expo = reinterpret_cast<int32_t *>(ws + off);
  for (int i = 0; i < 32; ++i) {
    a.in_bits[i] = hc.in_bits[i];
    a.out_bits[i] = hc.out_bits[i];
    a.init_cz[i] = hc.init_cz[i];
  }
  cudaStream_t s = (cudaStream_t)stream;
  const int64_t total = batch << hc.w;
  int64_t blocks = (total + 255) / 256;
  const int64_t cap = (int64_t)sm_count() * 32;
  if (blocks > cap) blocks = cap;
  stream_init<<<(int)blocks, 256, 0, s>>>(a);
  int rc = check_launch("stream_init");
  if (rc) return rc;
  // plain launches: as programmatic dependents these multi-wave passes ran
  // slower (the next pass's resident blocks idle through the last wave)
  if (hc.w >= 10) {
    // persistent grid: as many blocks as are resident at once
    const size_t smem = (size_t)kMixWarps * 2 * 1024 * sizeof(float2);
    int occ = 0;
    rc = cuda_check(cudaFuncSetAttribute(stream_pass_mixed, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem),
                    "stream_pass_mixed smem");
    if (rc) return rc;
    rc = cuda_check(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, stream_pass_mixed, 32 * kMixWarps, smem),
                    "stream_pass_mixed occupancy");
    if (rc) return rc;
    const int64_t need = ((batch << (hc.w - 10)) + kMixWarps - 1) / kMixWarps;
    const int64_t nb = std::min<int64_t>(need, (int64_t)sm_count() * std::max(occ, 1));
    for (const MixDesc &d : make_mixed_passes(hc.w, hc.n_steps, host_steps(plan, 0))) {
      stream_pass_mixed<<<(int)nb, 32 * kMixWarps, smem, s>>>(a, d);
      rc = check_launch("stream_pass_mixed");
      if (rc) return rc;
    }
  } else {
    for (PassDesc d : make_passes(hc.w, hc.n_steps)) {
      const bool low = d.bits[0] < kLowLanes;
      if (!low) add_passive(d, hc.w);
      const int NR = low ? kLowRegs : d.nsteps + d.npas;
      const int64_t warps = batch << (hc.w - kLowLanes - NR);
      const int64_t nb = (warps + 3) / 4;
      if (nb > 0x7fffffff) return fail(MBQC_E_INVALID, "sv_forward_stream: batch too large");
      high_pass_fn fn = low ? stream_pass_low : high_pass(d.nsteps, d.npas);
      if (!fn) return fail(MBQC_E_INVALID, "sv_forward_stream: pass shape %d+%d", d.nsteps, d.npas);
      fn<<<(int)nb, 128, 0, s>>>(a, d);
      rc = check_launch("stream_pass");
      if (rc) return rc;
    }
  }
  stream_epilogue<<<(int)batch, 1024, 0, s>>>(a, reinterpret_cast<float2 *>(psi_out), flags, hc.lp_const,
                                              logprob, status);
  return check_launch("stream_epilogue");
}

}  // extern "C"
