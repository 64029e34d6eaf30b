// Statevector sweep with sampled outcomes and flow byproduct corrections.
//
// The semantics of mentpy's PennyLane backend (pennylane_simulator.py:133-152):
// node i is measured in the XY plane at its angle; on outcome 1 an X acts on
// flow(i) and a Z on every neighbour of flow(i) measured after i.  Here the
// corrections are a Pauli frame: a pending X on a node flips the sign of its
// measurement angle, a pending Z adds pi (the same projections as applying
// the gates first); the frame left on the outputs is applied to the final
// state.  With a causal flow the output state does not depend on the drawn
// outcomes (up to a global phase).
//
// One warp per run, the window in shared memory (w <= 10): each step makes
// one pass to reduce S = sum conj(psi0) psi1 and T = sum |psi0|^2 + |psi1|^2
// over the pairs of the measured bit (the branch weights are T +- 2 Re(c S)),
// draws the outcome (SplitMix64 of seed, run, step), and one pass to apply
// the branch, renormalised.
#include <cuda_runtime.h>

#include "dispatch.h"

namespace mbqc {

struct SampledArgs {
  const DevStep *steps;
  const int2 *map;
  int64_t B;
  const double *angles;
  int64_t astride;
  const float2 *psi_in;
  int64_t istride;
  float2 *psi_out;
  int M, n_in, n_out;
  uint64_t seed;
  const int16_t *x_step;    // [M] step receiving this step's X, or -1
  const uint64_t *z_steps;  // [M][2] steps receiving a Z (bit set over steps)
  const uint32_t *x_out;    // [M] output-index bits receiving an X
  const uint32_t *z_out;    // [M] output-index bits receiving a Z
  int8_t *outcomes;         // [B, ostride]
  int64_t ostride;
  int32_t *status;
};

__device__ __forceinline__ uint64_t sm64(uint64_t z) {
  z += 0x9e3779b97f4a7c15ull;
  z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
  z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
  return z ^ (z >> 31);
}

__device__ __forceinline__ uint32_t insert_bit(uint32_t r, int p, uint32_t b) {
  return ((r >> p) << (p + 1)) | (b << p) | (r & ((1u << p) - 1u));
}

template <int W>
__global__ void __launch_bounds__(128) sv_sampled(SampledArgs a) {
  constexpr int D = 1 << W;
  extern __shared__ __align__(16) float2 smem_s[];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const int64_t run = (int64_t)blockIdx.x * (blockDim.x >> 5) + wid;
  if (run >= a.B) return;  // the whole warp leaves together
  const int M = a.M;
  float2 *s = smem_s + (size_t)wid * (D + M);
  float2 *coef = s + D;

  for (int k = lane; k < M; k += 32) {
    const DevStep st = a.steps[k];
    const double th = st.aidx >= 0 ? a.angles[run * a.astride + st.aidx] : st.fixed;
    float2 c, ph;
    sv_coef(st.plane, th, false, c, ph);
    coef[k] = c;
  }
  const float2 *in = a.psi_in + (a.istride ? run * a.istride : 0);
  for (int i = lane; i < D; i += 32) {
    const int2 m = a.map[i];
    s[i] = flip_sign(in[m.x & 0x7fffffff], (uint32_t)m.x & 0x80000000u);
  }
  __syncwarp();

  uint64_t fx0 = 0, fx1 = 0, fz0 = 0, fz1 = 0;  // pending X / Z per step
  uint32_t xo = 0, zo = 0;                      // pending X / Z on the outputs
  int32_t code = MBQC_RUN_OK;
  for (int k = 0; k < M; ++k) {
    const int p = k % W;
    const uint32_t mask = a.steps[k].mask;
    const bool dead = (mask & kDead) != 0u;
    float2 c = coef[k];
    const uint64_t fxw = k < 64 ? fx0 : fx1, fzw = k < 64 ? fz0 : fz1;
    if ((fxw >> (k & 63)) & 1ull) c.y = -c.y;            // X: angle -> -angle
    if ((fzw >> (k & 63)) & 1ull) c = make_float2(-c.x, -c.y);  // Z: angle -> angle + pi
    // branch weights
    float sr = 0.f, si = 0.f, t = 0.f;
    for (int q = lane; q < D / 2; q += 32) {
      const uint32_t i0 = insert_bit((uint32_t)q, p, 0u), i1 = i0 | (1u << p);
      const float2 u = s[i0], v = s[i1];
      sr += u.x * v.x + u.y * v.y;
      si += u.x * v.y - u.y * v.x;
      t += u.x * u.x + u.y * u.y + v.x * v.x + v.y * v.y;
    }
#pragma unroll
    for (int o = 16; o >= 1; o >>= 1) {
      sr += __shfl_xor_sync(0xffffffffu, sr, o);
      si += __shfl_xor_sync(0xffffffffu, si, o);
      t += __shfl_xor_sync(0xffffffffu, t, o);
    }
    const float re = c.x * sr - c.y * si;  // Re(c S)
    const float n0 = t + 2.f * re, n1 = t - 2.f * re;
    const uint64_t h = sm64(a.seed ^ sm64(((uint64_t)run << 20) ^ (uint64_t)k));
    const float u01 = (float)(h >> 40) * 5.9604644775390625e-08f;
    const int m = (u01 * (n0 + n1) >= n0) ? 1 : 0;
    const float nm = m ? n1 : n0;
    if (!(nm > 0.f) || isnan(nm) || isinf(nm)) {
      code = isnan(nm) ? MBQC_RUN_NAN : MBQC_RUN_ZERO_NORM;
      break;
    }
    const float g = rsqrtf(dead ? nm : 2.f * nm);
    const float2 ce = m ? make_float2(-c.x, -c.y) : c;
    for (int q = lane; q < D / 2; q += 32) {
      const uint32_t i0 = insert_bit((uint32_t)q, p, 0u), i1 = i0 | (1u << p);
      const float2 u = s[i0], v = s[i1];
      const float2 phi = make_float2(g * (u.x + ce.x * v.x - ce.y * v.y), g * (u.y + ce.x * v.y + ce.y * v.x));
      s[i0] = phi;
      s[i1] = dead ? make_float2(0.f, 0.f) : flip_sign(phi, (uint32_t)(__popc(i1 & mask) & 1u) << 31);
    }
    __syncwarp();
    if (lane == 0 && a.outcomes) a.outcomes[run * a.ostride + k] = (int8_t)m;
    if (m) {
      const int xt = a.x_step[k];
      if (xt >= 0) {
        if (xt < 64)
          fx0 ^= 1ull << xt;
        else
          fx1 ^= 1ull << (xt - 64);
      }
      fz0 ^= a.z_steps[2 * k];
      fz1 ^= a.z_steps[2 * k + 1];
      xo ^= a.x_out[k];
      zo ^= a.z_out[k];
    }
  }
  const int dout = 1 << a.n_out;
  float2 *out = a.psi_out + run * dout;
  for (int i = lane; i < D; i += 32) {
    const int y = a.map[i].y;
    if (y < 0) continue;
    const uint32_t yy = (uint32_t)y ^ xo;  // X on the outputs permutes the index
    const float2 v = code == MBQC_RUN_OK ? s[i] : make_float2(NAN, NAN);
    out[yy] = flip_sign(v, (uint32_t)(__popc(yy & zo) & 1u) << 31);  // then Z signs
  }
  if (lane == 0 && a.status) a.status[run] = code;
}

template <int W>
static int launch_sampled(const SampledArgs &a, cudaStream_t s) {
  const size_t smem = (size_t)4 * ((1 << W) + a.M) * sizeof(float2);
  auto k = sv_sampled<W>;
  int rc = cuda_check(cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem),
                      "sampled smem attribute");
  if (rc) return rc;
  const int64_t blocks = (a.B + 3) / 4;
  if (blocks > 0x7fffffff) return fail(MBQC_E_INVALID, "sv_forward_sampled: batch too large");
  k<<<(int)blocks, 128, smem, s>>>(a);
  return check_launch("sv_sampled");
}

}  // namespace mbqc

using namespace mbqc;

extern "C" int mbqc_sv_forward_sampled(const mbqc_plan *plan, int64_t batch, const double *angles,
                                       int64_t angle_stride, const float *psi_in, int64_t in_stride,
                                       float *psi_out, uint64_t seed, const mbqc_byproducts *corr,
                                       int8_t *outcomes, int64_t outcome_stride, int32_t *status,
                                       mbqc_stream_t stream) {
  if (!plan) return fail(MBQC_E_INVALID, "sv_forward_sampled: null plan");
  if (batch < 0) return fail(MBQC_E_INVALID, "sv_forward_sampled: negative batch");
  if (batch == 0) return MBQC_OK;
  const DevCircuit &hc = host_circuit(plan, 0);
  if (!psi_in || !psi_out || !corr) return fail(MBQC_E_INVALID, "sv_forward_sampled: null buffer");
  if (!hc.sv_planes_ok) return fail(MBQC_E_UNSUPPORTED, "sv_forward_sampled: steps in XY, X or Y only");
  if (hc.w > 10 || hc.map_off < 0) return fail(MBQC_E_UNSUPPORTED, "sv_forward_sampled: window %d > 10", hc.w);
  if (hc.n_steps > 128) return fail(MBQC_E_UNSUPPORTED, "sv_forward_sampled: %d steps > 128", hc.n_steps);
  if (hc.n_steps > 0 && (!corr->x_step || !corr->z_steps || !corr->x_out || !corr->z_out))
    return fail(MBQC_E_INVALID, "sv_forward_sampled: byproduct tables");
  if (hc.n_angles > 0 && (!angles || angle_stride < hc.n_angles))
    return fail(MBQC_E_INVALID, "sv_forward_sampled: bad angle array");
  if (in_stride != 0 && in_stride < ((int64_t)1 << hc.n_in))
    return fail(MBQC_E_INVALID, "sv_forward_sampled: input stride too small");
  if (outcomes && outcome_stride < hc.n_steps) return fail(MBQC_E_INVALID, "sv_forward_sampled: outcome stride");
  const PlanView v = view_of(plan);
  SampledArgs a;
  a.steps = v.d_steps + hc.step_off;
  a.map = v.d_map + hc.map_off;
  a.B = batch;
  a.angles = angles;
  a.astride = angle_stride;
  a.psi_in = reinterpret_cast<const float2 *>(psi_in);
  a.istride = in_stride;
  a.psi_out = reinterpret_cast<float2 *>(psi_out);
  a.M = hc.n_steps;
  a.n_in = hc.n_in;
  a.n_out = hc.n_out;
  a.seed = seed;
  a.x_step = corr->x_step;
  a.z_steps = corr->z_steps;
  a.x_out = corr->x_out;
  a.z_out = corr->z_out;
  a.outcomes = outcomes;
  a.ostride = outcome_stride;
  a.status = status;
  cudaStream_t s = (cudaStream_t)stream;
  switch (hc.w) {
    case 1: return launch_sampled<1>(a, s);
    case 2: return launch_sampled<2>(a, s);
    case 3: return launch_sampled<3>(a, s);
    case 4: return launch_sampled<4>(a, s);
    case 5: return launch_sampled<5>(a, s);
    case 6: return launch_sampled<6>(a, s);
    case 7: return launch_sampled<7>(a, s);
    case 8: return launch_sampled<8>(a, s);
    case 9: return launch_sampled<9>(a, s);
    default: return launch_sampled<10>(a, s);
  }
}
