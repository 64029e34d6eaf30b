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
// exact.  One init kernel builds the first window (table-driven input
// gather and CZ signs), the passes follow, and two grid-wide epilogue
// kernels normalise (float-pair sums: FP64-level accuracy), apply the
// reference global phase and write the outputs in the reference's order.
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

// First window: amplitude idx = psi_in[x(idx)] * (-1)^Q(idx), x gathering
// the input bits and Q the quadratic form of the initial CZ layer.  A block
// handles chunks of 2^K amplitudes that differ in a bit set S (window bits
// 0..4, so writes are coalesced, and the window bits holding the lowest
// input bits, so the chunk's input reads share sectors and hit L1).  With
// idx = hi | lo (lo in S): x(idx) = x(hi) | x(lo) and Q(idx) = Q(hi) ^ Q(lo)
// ^ parity(lo & M(hi)), M(hi) bit p = bit p of XOR_{q in hi} cz[q] ^
// parity(hi & cz[p]).  x(lo) | Q(lo) << 31 is tabulated per block by
// doubling over the bits of S (entry 2^b + l from entry l; the couplings and
// the single-bit terms come from the host).
constexpr int kInitLo = 11;
constexpr int kInitThreads = 256;
struct InitDesc {
  int K;
  int pos[kInitLo];        // S in increasing order (pos[i] = i for i < 5)
  uint32_t nb[kInitLo];    // bit i (< b): coupling of pos[b] and pos[i]
  uint32_t head[kInitLo];  // x(1 << pos[b]) | Q(1 << pos[b]) << 31
  uint32_t smask;
};

__global__ void __launch_bounds__(kInitThreads) stream_init(StreamArgs a, InitDesc id) {
  __shared__ uint32_t s_t[1 << kInitLo];
  __shared__ uint32_t s_dep[1 << (kInitLo - 5)];  // window bits of l >> 5
  const int K = id.K, tid = threadIdx.x;
  if (tid == 0) s_t[0] = 0u;
  for (int j = tid; j < (1 << (K - 5)); j += blockDim.x) {
    uint32_t d = 0;
    for (int i = 5; i < K; ++i)
      if ((j >> (i - 5)) & 1) d |= 1u << id.pos[i];
    s_dep[j] = d;
  }
  __syncthreads();
  for (int b = 0; b < K; ++b) {
    const uint32_t one = 1u << b, head = id.head[b], nb = id.nb[b];
    for (int l = tid; l < (int)one; l += blockDim.x) {
      const uint32_t t = s_t[l];
      const uint32_t q = ((t ^ head) >> 31) ^ (__popc((uint32_t)l & nb) & 1u);
      s_t[one | (uint32_t)l] = ((t | head) & 0x7fffffffu) | (q << 31);
    }
    __syncthreads();
  }
  const int hlog = a.W - K;
  const int64_t n_chunks = a.B << hlog;
  for (int64_t c = blockIdx.x; c < n_chunks; c += gridDim.x) {
    const int64_t run = c >> hlog;
    uint32_t hi = 0;  // chunk bits deposited on the window bits outside S
    for (int q = 0, t = 0; q < a.W; ++q)
      if (!((id.smask >> q) & 1u)) hi |= (uint32_t)((c >> t++) & 1) << q;
    uint32_t acc = 0;
    for (int q = 0; q < a.W; ++q)
      if ((hi >> q) & 1u) acc ^= a.init_cz[q];
    uint32_t m = 0;
    for (int i = 0; i < K; ++i) m |= (((acc >> id.pos[i]) ^ (uint32_t)__popc(hi & a.init_cz[id.pos[i]])) & 1u) << i;
    const uint32_t qhi = init_parity(hi, a.init_cz, a.W);
    const uint32_t xhi = (uint32_t)gather_bits(hi, a.in_bits, a.n_in);
    const float2 *in = a.psi_in + (a.istride ? run * a.istride : 0);
    float2 *out = a.state + (run << a.W) + hi;
    for (int l = tid; l < (1 << K); l += kInitThreads) {
      const uint32_t t = s_t[l];
      const uint32_t par = qhi ^ (t >> 31) ^ (__popc((uint32_t)l & m) & 1u);
      out[(uint32_t)(l & 31) | s_dep[l >> 5]] = flip_sign(__ldg(in + (xhi | (t & 0x7fffffffu))), par << 31);
    }
  }
  for (int64_t r = (int64_t)blockIdx.x * blockDim.x + tid; r < a.B; r += (int64_t)gridDim.x * blockDim.x) {
    a.norms[r] = 0.0;            // accumulated by pass 0
    a.norms[2 * a.B + r] = 1.0;  // "previous pass" of pass 0: no rescale
    a.expo[r] = 0;
  }
}

// host copies of the index helpers, for the init descriptor
static uint32_t host_gather(uint32_t idx, const int8_t *bits, int n) {
  uint32_t x = 0;
  for (int i = 0; i < n; ++i) x = (x << 1) | ((idx >> bits[i]) & 1u);
  return x;
}
static uint32_t host_init_parity(uint32_t idx, const uint32_t *cz, int w) {
  uint32_t p = 0;
  for (int q = 0; q < w; ++q) p ^= ((idx >> q) & 1u) & ((uint32_t)__builtin_popcount(idx & cz[q]) & 1u);
  return p;
}

static InitDesc make_init_desc(const DevCircuit &hc) {
  InitDesc id{};
  const int W = hc.w, K = W < kInitLo ? W : kInitLo;
  uint32_t S = 31u;
  for (int j = 0; j < 6 && j < hc.n_in; ++j) {  // input bit j sits at window bit in_bits[n_in - 1 - j]
    if (__builtin_popcount(S) >= K) break;
    S |= 1u << hc.in_bits[hc.n_in - 1 - j];
  }
  for (int b = 0; b < W && __builtin_popcount(S) < K; ++b) S |= 1u << b;
  id.K = K;
  id.smask = S;
  for (int b = 0, i = 0; b < W; ++b)
    if ((S >> b) & 1u) id.pos[i++] = b;
  for (int b = 0; b < K; ++b) {
    const int pb = id.pos[b];
    uint32_t nb = 0;
    for (int i = 0; i < b; ++i) {
      const int pi = id.pos[i];
      nb |= (((hc.init_cz[pb] >> pi) ^ (hc.init_cz[pi] >> pb)) & 1u) << i;
    }
    id.nb[b] = nb;
    id.head[b] = host_gather(1u << pb, hc.in_bits, hc.n_in) | (host_init_parity(1u << pb, hc.init_cz, W) << 31);
  }
  return id;
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

// lane j (< nsteps) holds the coefficient of the pass's step j for this
// warp's run (and, for plans with XZ / YZ steps, the real coefficient amp of
// the step's lower half)
template <bool GEN, typename D>
__device__ __forceinline__ float2 lane_coef(const StreamArgs &a, const D &d, int64_t run, int lane, float &amp) {
  float2 c = make_float2(1.f, 0.f), ph;
  amp = 1.f;
  if (lane < d.nsteps) {
    const DevStep st = a.steps[d.k0 + lane];
    const double th = st.aidx >= 0 ? a.angles[run * a.astride + st.aidx] : st.fixed;
    if constexpr (GEN)
      sv_coef_gen(st.plane, th, false, c, amp, ph);
    else
      sv_coef(st.plane, th, false, c, ph);
  }
  return c;
}

__device__ __forceinline__ float2 bcast(float2 c, int j) {
  return make_float2(__shfl_sync(0xffffffffu, c.x, j), __shfl_sync(0xffffffffu, c.y, j));
}

// a pass step on register bit J (lower half amp = 1 unless GEN)
template <bool GEN, int R, int J>
__device__ __forceinline__ void pass_reg_step(float2 (&v)[R], float2 c, float amp, uint32_t ts, bool dead) {
  if constexpr (GEN)
    reg_step_g<float, R, J>(v, c, amp, ts, dead);
  else
    reg_step<float, R, J>(v, c, ts, dead);
}
template <bool GEN, int R, int Q>
__device__ __forceinline__ void pass_lane_step(float2 (&v)[R], float2 c, float amp, uint32_t ts, bool dead,
                                               int lane) {
  if constexpr (GEN)
    lane_step_g<float, R, Q>(v, c, amp, ts, dead, lane);
  else
    lane_step<float, R, Q>(v, c, ts, dead, lane);
}

template <int T, int P, bool GEN>
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
  float al;
  const float2 cl = lane_coef<GEN>(a, d, run, lane, al);
#define MBQC_HSTEP(J)                                                                           \
  if (J < d.nsteps) {                                                                           \
    const float2 c = bcast(cl, J);                                                              \
    const float am = GEN ? __shfl_sync(0xffffffffu, al, J) : 1.f;                               \
    const uint32_t m = a.steps[d.k0 + J].mask;                                                  \
    uint32_t cm = 0;                                                                            \
    for (int i = 0; i < NR; ++i) cm |= ((m >> rbits[i]) & 1u) << i;                             \
    const uint32_t ts = parity_table(cm, NR) ^ (0u - (__popc(base & m & ~kDead) & 1u));         \
    pass_reg_step<GEN, R, J < T ? J : 0>(v, c, am, ts, (m & kDead) != 0u);                      \
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

template <bool GEN>
static high_pass_fn high_pass(int T, int P) {
  switch (T * 8 + P) {
    case 8: return stream_pass_high<1, 0, GEN>;
    case 9: return stream_pass_high<1, 1, GEN>;
    case 10: return stream_pass_high<1, 2, GEN>;
    case 11: return stream_pass_high<1, 3, GEN>;
    case 16: return stream_pass_high<2, 0, GEN>;
    case 17: return stream_pass_high<2, 1, GEN>;
    case 18: return stream_pass_high<2, 2, GEN>;
    case 24: return stream_pass_high<3, 0, GEN>;
    case 25: return stream_pass_high<3, 1, GEN>;
    case 32: return stream_pass_high<4, 0, GEN>;
    case 40: return stream_pass_high<5, 0, GEN>;
    default: return nullptr;
  }
}

template <bool GEN>
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
  float al;
  const float2 cl = lane_coef<GEN>(a, d, run, lane, al);
  for (int j = 0; j < d.nsteps; ++j) {
    const float2 c = bcast(cl, j);
    const float am = GEN ? __shfl_sync(0xffffffffu, al, j) : 1.f;
    const uint32_t m = a.steps[d.k0 + j].mask;
    const uint32_t cm = (m >> kLowLanes) & (R - 1u);
    const uint32_t ts = parity_table(cm, kLowRegs) ^ (0u - (__popc(base & m & ~kDead) & 1u));
    const bool dead = (m & kDead) != 0u;
    switch (d.bits[j]) {
      case 0: pass_lane_step<GEN, R, 0>(v, c, am, ts, dead, lane); break;
      case 1: pass_lane_step<GEN, R, 1>(v, c, am, ts, dead, lane); break;
      case 2: pass_lane_step<GEN, R, 2>(v, c, am, ts, dead, lane); break;
      case 3: pass_lane_step<GEN, R, 3>(v, c, am, ts, dead, lane); break;
      default: pass_lane_step<GEN, R, 4>(v, c, am, ts, dead, lane); break;
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

// Tile staging by the TMA engine: each 256-byte row of a 32 x 32 tile (index
// bits 0..4 of one register pattern) is one bulk asynchronous copy
// (cp.async.bulk, the TMA unit's non-tensor mode) into the warp's shared
// buffer, all 32 completing on the buffer's mbarrier (8 KB of transaction
// bytes).  The rows of a tile sit at five arbitrary index bits above bit 4,
// which a tensor map of at most five dimensions cannot describe together with
// the free tile bits, so the copies are per row (one instruction per lane).
// Rows are padded to 272 bytes: row accesses are conflict free, column
// accesses (the transposed layout) take two wavefronts per 16 lanes.
constexpr int kMixRow = 34;            // float2 per padded row (272 bytes)
constexpr int kMixBuf = 32 * kMixRow;  // float2 per tile buffer (both layouts fit)
// Warps per block of the mixed pass.  Shared memory (two 8 KB tiles a warp)
// and registers allow 12-14 warps per SM; small blocks fill an SM closest to
// that (grid 16 x 10 batch: 4 warps 0.649 ms, 2 warps 0.631 ms, 7 warps
// 0.643 ms, 1 warp 0.690 ms; 1 / 2 / 3 blocks of 4 warps per SM: 1.18 / 0.74
// / 0.65 ms -- the pass is near its issue limit at this occupancy).
constexpr int kMixWarps = 2;

// The default staging: asynchronous 16-byte global -> shared copies (cached
// in L2 only), each lane copying 16 of the tile's 256 pairs; each thread
// waits for its own copies and a __syncwarp makes the warp's copies visible.
// It measured 10 % faster per batch than the bulk-copy path above on the
// grid 16 x 10 workload (0.649 vs 0.720 ms): 32 bulk copies of 256 bytes per
// tile keep the TMA unit busier than the 512 small copies keep the load unit.
__device__ __forceinline__ void cp_async16(void *smem, const void *gmem) {
  const unsigned s = (unsigned)__cvta_generic_to_shared(smem);
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(s), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait_prev() { asm volatile("cp.async.wait_group 1;" ::: "memory"); }
// Bound of every mbarrier wait: tries of at most kMbarSuspendNs each (the
// waiting thread is suspended until the phase completes or the hint
// elapses), about a second in all.
constexpr uint32_t kMbarTries = 100000u;
constexpr uint32_t kMbarSuspendNs = 10000u;

// shared-memory slot of tile element (row r = register pattern, column c =
// index bits 0..4).  Bulk copies: rows padded to 272 bytes.  16-byte copies:
// 16-byte pairs of a row XOR-swizzled by the row.  Either way row accesses
// are conflict free and column accesses take two wavefronts per 128 bytes.
template <bool TMA>
__device__ __forceinline__ int tslot(int r, int c) {
  if constexpr (TMA)
    return r * kMixRow + c;
  else
    return r * 32 + ((((c >> 1) ^ (r & 15)) << 1) | (c & 1));
}

__device__ __forceinline__ uint32_t smem_u32(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }
__device__ __forceinline__ void mbar_init(uint64_t *m, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(m)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t *m, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(m)), "r"(bytes) : "memory");
}
// true when the phase of the given parity completed within the bound
__device__ __forceinline__ bool mbar_wait(uint64_t *m, uint32_t parity) {
  const uint32_t a = smem_u32(m);
  for (uint32_t i = 0; i < kMbarTries; ++i) {
    uint32_t done;
    asm volatile(
        "{ .reg .pred p; mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2, %3; selp.u32 %0, 1, 0, p; }"
        : "=r"(done)
        : "r"(a), "r"(parity), "r"(kMbarSuspendNs)
        : "memory");
    if (done) return true;
  }
  return false;
}
__device__ __forceinline__ void bulk_row_copy(void *dst, const void *src, uint32_t bytes, uint64_t *m) {
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                   smem_u32(dst)),
               "l"(src), "r"(bytes), "r"(smem_u32(m))
               : "memory");
}
// generic-proxy accesses of this thread to shared memory are ordered before
// its later asynchronous-proxy (bulk copy) accesses
__device__ __forceinline__ void fence_proxy_async() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

// Persistent warps, each owning a contiguous range of tiles (consecutive
// tiles mostly share a run, whose scale and step coefficients are reused);
// while a warp computes tile i, tile i + 1 is already on its way into the
// warp's other shared-memory buffer (TMA: bulk copies on an mbarrier; else
// 16-byte asynchronous copies).  A bulk-copy wait that exceeds its bound
// poisons the warp's tiles with NaN (the runs end with status MBQC_RUN_NAN)
// after a bounded wait for the copies still in flight.
template <bool TMA, bool GEN>
__global__ void __launch_bounds__(32 * kMixWarps) stream_pass_mixed(StreamArgs a, MixDesc d) {
  extern __shared__ __align__(16) float2 s_mix[];  // [warp][2][32 rows x 34]
  __shared__ __align__(8) uint64_t s_mbar[kMixWarps][2];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  constexpr int BUF = TMA ? kMixBuf : 1024;  // float2 per tile buffer
  float2 *buf = s_mix + (size_t)wid * 2 * BUF;
  uint64_t *mbar = s_mbar[wid];
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
  if constexpr (TMA) {
    if (lane == 0) {
      mbar_init(&mbar[0], 1);
      mbar_init(&mbar[1], 1);
      asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncwarp();
  }
  auto issue = [&](int64_t g, int b) {
    float2 *dst = buf + b * BUF;
    if constexpr (TMA) {  // lane r copies row r of tile g
      if (lane == 0) mbar_expect_tx(&mbar[b], 32 * 256);
      __syncwarp();
      const float2 *src = a.state + ((g >> tlog) << a.W) + (tile_bits(g) | lane_roff);
      bulk_row_copy(dst + lane * kMixRow, src, 256, &mbar[b]);
    } else {  // lane: pair lane & 15 of rows 2i + (lane >> 4)
      const float2 *st = a.state + ((g >> tlog) << a.W) + tile_bits(g);
      const int pr = lane & 15;
#pragma unroll
      for (int i = 0; i < 16; ++i) {
        const int r = 2 * i + (lane >> 4);
        cp_async16(dst + r * 32 + ((pr ^ (r & 15)) << 1), st + (roff(r) | (uint32_t)(2 * pr)));
      }
      cp_async_commit();
    }
  };
  uint32_t parity[2] = {0u, 0u};
  bool failed = false;

  if (g0 < g1) issue(g0, 0);
  else if constexpr (!TMA) cp_async_commit();
  int64_t cur_run = -1;
  int f = 0;
  float gsc = 1.f;
  float2 cl = make_float2(1.f, 0.f);
  float al = 1.f;
  float part = 0.f;
  bool tile0 = false;
  for (int64_t g = g0; g < g1; ++g) {
    const int b = (int)((g - g0) & 1);
    float2 *cur = buf + b * BUF;
    if (g + 1 < g1) issue(g + 1, b ^ 1);
    if constexpr (TMA) {
      if (!mbar_wait(&mbar[b], parity[b])) {
        failed = true;
        break;
      }
      parity[b] ^= 1u;
    } else {
      if (!(g + 1 < g1)) cp_async_commit();  // an empty group keeps the wait depth at one
      cp_async_wait_prev();
      __syncwarp();
    }
    const int64_t run = g >> tlog;
    if (run != cur_run) {
      if (cur_run >= 0) pass_bookkeeping(a, d, cur_run, tile0, lane, f, part);
      cur_run = run;
      part = 0.f;
      tile0 = false;
      f = pass_exponent(a, d.index, run);
      gsc = RealBits<float>::pow2(-f);
      cl = lane_coef<GEN>(a, d, run, lane, al);
    }
    tile0 = tile0 || (g & ((1ll << tlog) - 1)) == 0;
    const uint32_t tb = tile_bits(g);
    const uint32_t nbase = tb | (uint32_t)lane;   // normal layout: lane = bits 0..4
    const uint32_t tbase = tb | lane_roff;        // transposed: lane = register pattern
    float2 v[32];
    const bool start_low = d.n1 == 0 && d.nl > 0;
    if (start_low) {
#pragma unroll
      for (int c = 0; c < 32; ++c) {
        const float2 x = cur[tslot<TMA>(lane, c)];
        v[c] = make_float2(x.x * gsc, x.y * gsc);
      }
    } else {
#pragma unroll
      for (int r = 0; r < 32; ++r) {
        const float2 x = cur[tslot<TMA>(r, lane)];
        v[r] = make_float2(x.x * gsc, x.y * gsc);
      }
    }
    auto hstep = [&](auto jc, int j) {  // high step j of the pass on register bit J
      constexpr int J = decltype(jc)::value;
      const uint32_t m = d.mask[j];
      const uint32_t ts = d.ptab[j] ^ (0u - (__popc(nbase & m & ~kDead) & 1u));
      pass_reg_step<GEN, 32, J>(v, bcast(cl, j), GEN ? __shfl_sync(0xffffffffu, al, j) : 1.f, ts,
                                (m & kDead) != 0u);
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
        for (int r = 0; r < 32; ++r) cur[tslot<TMA>(r, lane)] = v[r];
        __syncwarp();
#pragma unroll
        for (int c = 0; c < 32; ++c) v[c] = cur[tslot<TMA>(lane, c)];
      }
      for (int j = 0; j < d.nl; ++j) {
        const int js = d.n1 + j;
        const uint32_t m = d.mask[js];
        const uint32_t ts = d.ptab[js] ^ (0u - (__popc(tbase & m & ~kDead) & 1u));
        const float2 c = bcast(cl, js);
        const float am = GEN ? __shfl_sync(0xffffffffu, al, js) : 1.f;
        const bool dead = (m & kDead) != 0u;
        switch (d.lbits[j]) {
          case 0: pass_reg_step<GEN, 32, 0>(v, c, am, ts, dead); break;
          case 1: pass_reg_step<GEN, 32, 1>(v, c, am, ts, dead); break;
          case 2: pass_reg_step<GEN, 32, 2>(v, c, am, ts, dead); break;
          case 3: pass_reg_step<GEN, 32, 3>(v, c, am, ts, dead); break;
          default: pass_reg_step<GEN, 32, 4>(v, c, am, ts, dead); break;
        }
      }
      __syncwarp();  // back to the normal layout
#pragma unroll
      for (int c = 0; c < 32; ++c) cur[tslot<TMA>(lane, c)] = v[c];
      __syncwarp();
#pragma unroll
      for (int r = 0; r < 32; ++r) v[r] = cur[tslot<TMA>(r, lane)];
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
    // every lane is done with `cur` (and, for bulk copies, its generic
    // writes are ordered before them) before the copy two tiles on refills it
    if constexpr (TMA) fence_proxy_async();
    __syncwarp();
  }
  if (TMA && failed) {
    // a copy did not arrive within the bound: wait (bounded) for the
    // copies still in flight, then poison this warp's tiles
    mbar_wait(&mbar[0], parity[0]);
    mbar_wait(&mbar[1], parity[1]);
    const float2 bad = make_float2(NAN, NAN);
    for (int64_t g = g0; g < g1; ++g) {
      float2 *st = a.state + ((g >> tlog) << a.W);
      const uint32_t nbase = tile_bits(g) | (uint32_t)lane;
      for (int r = 0; r < 32; ++r) st[nbase | roff(r)] = bad;
    }
    return;
  }
  if (cur_run >= 0) pass_bookkeeping(a, d, cur_run, tile0, lane, f, part);
}

// Epilogue: normalise (float-pair sums: FP64-level accuracy), apply the
// reference global phase and write the outputs in the reference's order.
// The outputs of a run are split into chunks of 2^K consecutive output
// indices y (y bits 0..K-1 vary; their window bits, sorted, enumerate the
// chunk so that reads follow the window order).  Two grid-wide kernels:
// stream_out_norm writes each chunk's partial squared norm (and, per run,
// the phase product and the input norm); stream_out_write sums a run's
// partials in a fixed order (deterministic), scales, and writes its chunk
// through shared memory in output order (coalesced).
constexpr int kOutLo = 10;
constexpr int kOutThreads = 256;
struct OutDesc {
  int K, nch_log;        // chunk bits; log2 of the chunks per run
  uint32_t wlo[32], whi[32];  // window offset of chunk-local index bits 0..4 / 5..9 (window order)
  uint16_t ylo[32], yhi[32];  // output offset of the same
  int ywin[32];               // window bit of output bit j (j < n_out)
};

__device__ __forceinline__ uint32_t chunk_window_base(const OutDesc &od, int n_out, uint32_t y) {
  uint32_t w = 0;
  for (int j = od.K; j < n_out; ++j)
    if ((y >> j) & 1u) w |= 1u << od.ywin[j];
  return w;
}

__device__ __forceinline__ float2 block_pair_sum(float2 v, float2 *s_red) {
#pragma unroll
  for (int o = 16; o >= 1; o >>= 1)
    two_sum_acc(v.x, v.y, __shfl_xor_sync(0xffffffffu, v.x, o), __shfl_xor_sync(0xffffffffu, v.y, o));
  const int tid = threadIdx.x;
  if ((tid & 31) == 0) s_red[tid >> 5] = v;
  __syncthreads();
  float2 t = s_red[0];
  for (int i = 1; i < (int)(blockDim.x >> 5); ++i) two_sum_acc(t.x, t.y, s_red[i].x, s_red[i].y);
  __syncthreads();
  return t;
}

__global__ void __launch_bounds__(kOutThreads) stream_out_norm(StreamArgs a, OutDesc od, uint32_t flags, float2 *part,
                                                      float2 *phase, double *nin, bool want_nin) {
  __shared__ float2 s_red[8];
  __shared__ float2 s_ph[8];
  __shared__ uint32_t s_w[64];  // per-lane table reads from shared memory, not the constant bank
  const int64_t run = blockIdx.x >> od.nch_log;
  const uint32_t ch = blockIdx.x & ((1u << od.nch_log) - 1u);
  const int tid = threadIdx.x;
  if (tid < 64) s_w[tid] = tid < 32 ? od.wlo[tid] : od.whi[tid - 32];
  __syncthreads();
  const uint32_t wbase = chunk_window_base(od, a.n_out, ch << od.K);
  const float2 *st = a.state + (run << a.W) + wbase;
  float2 acc = make_float2(0.f, 0.f);
  for (int l = tid; l < (1 << od.K); l += kOutThreads) {
    const float2 x = st[s_w[l & 31] | s_w[32 + (l >> 5)]];
    two_sum_acc(acc.x, acc.y, x.x * x.x + x.y * x.y, 0.f);
  }
  const float2 t = block_pair_sum(acc, s_red);
  if (tid == 0) part[blockIdx.x] = t;
  if (ch != 0) return;
  // per run: phase product over the steps, and the input's squared norm
  float2 ph = make_float2(1.f, 0.f);
  if (flags & MBQC_F_REF_PHASE) {
    for (int k = tid; k < a.M; k += blockDim.x) {
      const DevStep s = a.steps[k];
      const double th = s.aidx >= 0 ? a.angles[run * a.astride + s.aidx] : s.fixed;
      float2 c, p;
      float amp;
      sv_coef_gen(s.plane, th, true, c, amp, p);
      ph = cmul(ph, p);
    }
  }
#pragma unroll
  for (int o = 16; o >= 1; o >>= 1)
    ph = cmul(ph, make_float2(__shfl_xor_sync(0xffffffffu, ph.x, o), __shfl_xor_sync(0xffffffffu, ph.y, o)));
  if ((tid & 31) == 0) s_ph[tid >> 5] = ph;
  __syncthreads();
  if (tid == 0) {
    float2 q = s_ph[0];
    for (int i = 1; i < (int)(blockDim.x >> 5); ++i) q = cmul(q, s_ph[i]);
    phase[run] = q;
  }
  if (want_nin) {
    const float2 *in = a.psi_in + (a.istride ? run * a.istride : 0);
    float2 ni = make_float2(0.f, 0.f);
    for (int x = tid; x < (1 << a.n_in); x += blockDim.x) {
      const float2 v = in[x];
      two_sum_acc(ni.x, ni.y, v.x * v.x + v.y * v.y, 0.f);
    }
    const float2 tn = block_pair_sum(ni, s_red);
    if (tid == 0) nin[run] = (double)tn.x + (double)tn.y;
  }
}

__global__ void __launch_bounds__(kOutThreads) stream_out_write(StreamArgs a, OutDesc od, const float2 *part,
                                                       const float2 *phase, const double *nin, float2 *out,
                                                       int32_t lp_const, double *logprob, int32_t *status) {
  __shared__ float2 s_buf[1 << kOutLo];
  __shared__ float2 s_n2;
  __shared__ uint32_t s_w[64], s_y[64];
  const int64_t run = blockIdx.x >> od.nch_log;
  const uint32_t ch = blockIdx.x & ((1u << od.nch_log) - 1u);
  const int tid = threadIdx.x, nch = 1 << od.nch_log;
  if (tid < 64) {
    s_w[tid] = tid < 32 ? od.wlo[tid] : od.whi[tid - 32];
    s_y[tid] = tid < 32 ? od.ylo[tid] : od.yhi[tid - 32];
  }
  if (tid < 32) {  // the run's squared norm: its partials in a fixed order
    const float2 *pr = part + (run << od.nch_log);
    float2 n = make_float2(0.f, 0.f);
    for (int i = tid; i < nch; i += 32) two_sum_acc(n.x, n.y, pr[i].x, pr[i].y);
#pragma unroll
    for (int o = 16; o >= 1; o >>= 1)
      two_sum_acc(n.x, n.y, __shfl_xor_sync(0xffffffffu, n.x, o), __shfl_xor_sync(0xffffffffu, n.y, o));
    if (tid == 0) s_n2 = n;
  }
  __syncthreads();
  const float2 n2p = s_n2;
  const float n2 = n2p.x + n2p.y;
  const bool ok = (n2 > 0.f) && (n2 < 3.0e38f);
  float inv = rsqrtf(n2);
  inv = ok ? inv * (1.5f - 0.5f * n2 * inv * inv) : NAN;  // one Newton step
  const float2 ph = phase[run];
  const float2 sc = make_float2(ph.x * inv, ph.y * inv);
  const uint32_t y0 = ch << od.K;
  const float2 *st = a.state + (run << a.W) + chunk_window_base(od, a.n_out, y0);
  for (int l = tid; l < (1 << od.K); l += kOutThreads)
    s_buf[s_y[l & 31] | s_y[32 + (l >> 5)]] = cmul(st[s_w[l & 31] | s_w[32 + (l >> 5)]], sc);
  __syncthreads();
  float2 *o = out + (run << a.n_out) + y0;
  for (int j = tid; j < (1 << od.K); j += blockDim.x) o[j] = s_buf[j];
  if (ch == 0 && tid == 0) {
    if (status) status[run] = ok ? MBQC_RUN_OK : (isnan(n2) ? MBQC_RUN_NAN : MBQC_RUN_ZERO_NORM);
    if (logprob) {
      const double n2d = (double)n2p.x + (double)n2p.y;
      logprob[run] = log(n2d) - log(nin[run]) + 0.6931471805599453 * (2.0 * a.expo[run] + lp_const);
    }
  }
}

static OutDesc make_out_desc(const DevCircuit &hc) {
  OutDesc od{};
  const int n_out = hc.n_out, K = n_out < kOutLo ? n_out : kOutLo;
  od.K = K;
  od.nch_log = n_out - K;
  for (int j = 0; j < n_out; ++j) od.ywin[j] = hc.out_bits[n_out - 1 - j];  // output j is bit n_out-1-j of y
  // chunk-local index bits in window order: the window bits of y bits 0..K-1, sorted
  int order[kOutLo];
  for (int i = 0; i < K; ++i) order[i] = i;
  std::sort(order, order + K, [&](int p, int q) { return od.ywin[p] < od.ywin[q]; });
  for (int v = 0; v < 32; ++v) {
    uint32_t wl = 0, wh = 0;
    uint32_t yl = 0, yh = 0;
    for (int i = 0; i < 5; ++i) {
      if (!((v >> i) & 1)) continue;
      if (i < K) {
        wl |= 1u << od.ywin[order[i]];
        yl |= 1u << order[i];
      }
      if (i + 5 < K) {
        wh |= 1u << od.ywin[order[i + 5]];
        yh |= 1u << order[i + 5];
      }
    }
    od.wlo[v] = wl;
    od.whi[v] = wh;
    od.ylo[v] = (uint16_t)yl;
    od.yhi[v] = (uint16_t)yh;
  }
  return od;
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

// workspace: state [B][2^w] | norms [3][B] | expo [B] | (16-byte aligned)
// epilogue partials [B][2^(n_out - K)] | phases [B] | input norms [B]
static size_t stream_ws_head(int W, int64_t B) {
  const size_t h = (size_t)B * ((size_t)1 << W) * sizeof(float2) + (size_t)3 * B * sizeof(double) +
                   (size_t)B * sizeof(int32_t);
  return (h + 15) & ~(size_t)15;
}
static size_t stream_ws_bytes(const DevCircuit &hc, int64_t B) {
  const int K = hc.n_out < kOutLo ? hc.n_out : kOutLo;
  return stream_ws_head(hc.w, B) + ((size_t)B << (hc.n_out - K)) * sizeof(float2) + (size_t)B * sizeof(float2) +
         (size_t)B * sizeof(double) + 256;
}

}  // namespace mbqc

using namespace mbqc;

extern "C" {

int mbqc_sv_stream_workspace(const mbqc_plan *plan, int64_t batch, size_t *bytes) {
  if (!plan || !bytes || batch < 0) return fail(MBQC_E_INVALID, "stream_workspace: bad arguments");
  const DevCircuit &hc = host_circuit(plan, 0);
  if (hc.w < kStreamMinWindow)
    return fail(MBQC_E_UNSUPPORTED, "stream_workspace: window %d < %d", hc.w, kStreamMinWindow);
  *bytes = stream_ws_bytes(hc, batch);
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
  const bool gen = !hc.sv_planes_ok;  // XZ / YZ steps
  if (gen && !hc.sv_xz_ok)
    return fail(MBQC_E_UNSUPPORTED, "sv_forward_stream: statevector steps in XY, X, Y, XZ or YZ only");
  if (hc.n_angles > 0 && (!angles || angle_stride < hc.n_angles))
    return fail(MBQC_E_INVALID, "sv_forward_stream: bad angle array");
  if (in_stride != 0 && in_stride < ((int64_t)1 << hc.n_in))
    return fail(MBQC_E_INVALID, "sv_forward_stream: input stride too small");
  const size_t need = stream_ws_bytes(hc, batch);
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
  const InitDesc id = make_init_desc(hc);
  const int64_t chunks = batch << (hc.w - id.K);
  const int64_t blocks = std::min<int64_t>(std::max<int64_t>(chunks, (batch + 255) / 256), (int64_t)sm_count() * 8);
  stream_init<<<(int)blocks, kInitThreads, 0, s>>>(a, id);
  int rc = check_launch("stream_init");
  if (rc) return rc;
  // plain launches: as programmatic dependents these multi-wave passes ran
  // slower (the next pass's resident blocks idle through the last wave)
  if (hc.w >= 10) {
    // persistent grid: as many blocks as are resident at once
    const bool tma = (flags & MBQC_F_STREAM_TMA) != 0u;
    auto kmix = tma ? (gen ? stream_pass_mixed<true, true> : stream_pass_mixed<true, false>)
                    : (gen ? stream_pass_mixed<false, true> : stream_pass_mixed<false, false>);
    const size_t smem = (size_t)kMixWarps * 2 * (tma ? kMixBuf : 1024) * sizeof(float2);
    int occ = 0;
    rc = cuda_check(cudaFuncSetAttribute(kmix, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem),
                    "stream_pass_mixed smem");
    if (rc) return rc;
    rc = cuda_check(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, kmix, 32 * kMixWarps, smem),
                    "stream_pass_mixed occupancy");
    if (rc) return rc;
    const int64_t need = ((batch << (hc.w - 10)) + kMixWarps - 1) / kMixWarps;
    const int64_t nb = std::min<int64_t>(need, (int64_t)sm_count() * std::max(occ, 1));
    for (const MixDesc &d : make_mixed_passes(hc.w, hc.n_steps, host_steps(plan, 0))) {
      kmix<<<(int)nb, 32 * kMixWarps, smem, s>>>(a, d);
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
      high_pass_fn fn = low ? (gen ? stream_pass_low<true> : stream_pass_low<false>)
                            : (gen ? high_pass<true>(d.nsteps, d.npas) : high_pass<false>(d.nsteps, d.npas));
      if (!fn) return fail(MBQC_E_INVALID, "sv_forward_stream: pass shape %d+%d", d.nsteps, d.npas);
      fn<<<(int)nb, 128, 0, s>>>(a, d);
      rc = check_launch("stream_pass");
      if (rc) return rc;
    }
  }
  const OutDesc od = make_out_desc(hc);
  char *ep = ws + stream_ws_head(hc.w, batch);
  float2 *part = reinterpret_cast<float2 *>(ep);
  float2 *phase = part + ((size_t)batch << od.nch_log);
  double *nin = reinterpret_cast<double *>(phase + batch);
  const int64_t oblocks = batch << od.nch_log;
  if (oblocks > 0x7fffffff) return fail(MBQC_E_INVALID, "sv_forward_stream: batch too large");
  stream_out_norm<<<(int)oblocks, kOutThreads, 0, s>>>(a, od, flags, part, phase, nin, logprob != nullptr);
  rc = check_launch("stream_out_norm");
  if (rc) return rc;
  stream_out_write<<<(int)oblocks, kOutThreads, 0, s>>>(a, od, part, phase, nin, reinterpret_cast<float2 *>(psi_out),
                                                hc.lp_const, logprob, status);
  return check_launch("stream_out_write");
}

}  // extern "C"
