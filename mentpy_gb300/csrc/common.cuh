// Shared device-side definitions of the windowed MBQC sweep kernels.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/mbqc_gb300.h"

namespace mbqc {

constexpr uint32_t kDead = MBQC_STEP_DEAD;
constexpr int kMaxWindow = 30;
constexpr int kMaxIn = 30;

// One step of a plan as the kernels read it (24 bytes).
struct DevStep {
  uint32_t mask;   // CZ partners of the entering qubit, or kDead
  int32_t aidx;    // angle-vector index, -1 = fixed
  int32_t plane;   // MBQC_PLANE_*
  int32_t pad;
  double fixed;    // fixed angle
};

// Per-circuit header of a device plan table.
struct DevCircuit {
  int32_t w, n_steps, n_in, n_out, n_angles, step_off, n_dead, lp_const;
  int64_t map_off;    // offset of this circuit's index map, -1 = none
  int8_t in_bits[32];
  int8_t out_bits[32];
  uint32_t init_cz[32];
  uint32_t out_mask;  // OR of (1 << out_bits[j])
  int32_t item_off;   // offset of this circuit's item table, -1 = none
  int8_t sv_planes_ok; // every step in XY, X or Y (the one-coefficient statevector step)
  int8_t has_z;        // some step measures in the Z basis (density matrix only)
  int8_t sv_xz_ok;     // every step in XY, X, Y, XZ or YZ (the general-plane statevector step)
  int8_t pad8;
  int32_t pad;
};

// Coefficient staging in item order: item i < n_angles is the step measured
// with angle i, the fixed-angle steps follow in step order.
struct DevItem {
  int32_t step;   // step index
  int32_t plane;  // MBQC_PLANE_*
  double fixed;   // angle of a fixed-angle step (unused for angle items)
};

// Index maps are precomputed for windows up to this size.
constexpr int kMapMaxWindow = 16;

// Host-side view of a plan (defined in plan.cu).
struct PlanView {
  const DevCircuit *d_circ;  // [n_circuits]
  const DevStep *d_steps;    // all steps
  const int2 *d_map;         // index maps (see SvArgs::map)
  const DevItem *d_items;    // item tables (see DevCircuit::item_off)
  int n_circuits;
  int max_w;
};

// ---------------------------------------------------------------- complex
template <typename T> struct C2;
template <> struct C2<float> { using type = float2; };
template <> struct C2<double> { using type = double2; };
template <typename T> using cplx = typename C2<T>::type;

template <typename T> __host__ __device__ __forceinline__ cplx<T> mk(T r, T i) {
  cplx<T> z; z.x = r; z.y = i; return z;
}

// flip the sign of both components when bit 31 of ``s`` is set (s is 0 or
// 0x80000000): one LOP per component for float
__device__ __forceinline__ float2 flip_sign(float2 z, uint32_t s) {
  return make_float2(__uint_as_float(__float_as_uint(z.x) ^ s),
                     __uint_as_float(__float_as_uint(z.y) ^ s));
}
__device__ __forceinline__ double2 flip_sign(double2 z, uint32_t s) {
  const unsigned long long m = (unsigned long long)s << 32;
  return make_double2(__longlong_as_double(__double_as_longlong(z.x) ^ m),
                      __longlong_as_double(__double_as_longlong(z.y) ^ m));
}

// Bit pattern whose bit j is bit q of j (j < 32): the truth table of
// "index bit q" over 32 register slots.
__host__ __device__ constexpr uint32_t bit_pattern(int q) {
  return q == 0 ? 0xAAAAAAAAu
       : q == 1 ? 0xCCCCCCCCu
       : q == 2 ? 0xF0F0F0F0u
       : q == 3 ? 0xFF00FF00u
       : 0xFFFF0000u;
}

// Parity table over the low ``rb`` index bits: bit j = parity(j & mask).
__device__ __forceinline__ uint32_t parity_table(uint32_t mask, int rb) {
  uint32_t t = 0;
#pragma unroll
  for (int q = 0; q < 5; ++q)
    if (q < rb && ((mask >> q) & 1u)) t ^= bit_pattern(q);
  return t;
}

// double -> float, round to nearest even, on the integer ALU: GB300's FP64
// pipe (which executes F2F.F32.F64) runs at a small fraction of the FP32
// rate and is shared by the SM's four schedulers.  Normal float range only:
// magnitudes below 2^-126 give +-0 and at or above 2^128 give +-inf.
__device__ __forceinline__ float f64_to_f32_rn(double d) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(d);
  const uint32_t hi = (uint32_t)(b >> 32), lo = (uint32_t)b;
  const uint32_t sign = hi & 0x80000000u;
  const int e = (int)((hi >> 20) & 0x7ffu) - 1023;
  const uint32_t m = ((hi & 0xfffffu) << 3) | (lo >> 29);  // top 23 mantissa bits
  const uint32_t rest = lo & 0x1fffffffu;                    // 29 dropped bits
  uint32_t f = sign | ((uint32_t)(e + 127) << 23) | m;
  f += (rest > 0x10000000u || (rest == 0x10000000u && (m & 1u))) ? 1u : 0u;  // carries into the exponent
  f = e < -126 ? sign : (e > 127 ? (sign | 0x7f800000u) : f);
  return __uint_as_float(f);
}

// programmatic dependent launch: wait for the previous kernel on the stream
// (a no-op when the launch did not ask for the overlap), and let the next one
// start its own prologue
__device__ __forceinline__ void griddep_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }
__device__ __forceinline__ void griddep_launch_dependents() { asm volatile("griddepcontrol.launch_dependents;" ::); }
__device__ __forceinline__ void prefetch_l2(const void *p) { asm volatile("prefetch.global.L2 [%0];" ::"l"(p)); }

// (hi, lo) += (oh, ol) for unevaluated float pairs: Knuth's two-sum makes
// the rounding error of hi + oh exact, so a sum of pairs keeps a ~48-bit
// significand (FP64-level accumulation on the FP32 pipe).  Commutative in its
// two operands bit for bit, so xor butterflies leave the same pair on every
// lane.
__device__ __forceinline__ void two_sum_acc(float &hi, float &lo, float oh, float ol) {
  const float s = hi + oh;
  const float bb = s - hi;
  const float err = (hi - (s - bb)) + (oh - bb);
  hi = s;
  lo = (lo + ol) + err;
}

// Sum of v over aligned groups of L lanes (xor butterfly), the same value on
// every lane of a group: float pairs for float, plain FP64 for double.
template <typename T, int L>
__device__ __forceinline__ T lane_group_sum(T v) {
  if constexpr (sizeof(T) == 4) {
    float hi = v, lo = 0.f;
#pragma unroll
    for (int o = 1; o < L; o <<= 1) {
      const float oh = __shfl_xor_sync(0xffffffffu, hi, o);
      const float ol = __shfl_xor_sync(0xffffffffu, lo, o);
      two_sum_acc(hi, lo, oh, ol);
    }
    return hi + lo;
  } else {
#pragma unroll
    for (int o = 1; o < L; o <<= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
  }
}

// The double reduction for huge angles and near +-pi, out of line: a call
// cannot be if-converted, so the FP64 instructions run only in warps where
// some lane needs them (inlined, the compiler predicates them into every
// lane's path).  Near the branch cut the side is taken from sin(theta) of the
// double angle, as the reference's double arithmetic sees it: atan2(sin, cos)
// is in [-pi, pi] with the sign of sin(theta).
static __device__ __noinline__ float reduce_angle_exact(double theta) {
  double s, c;
  sincos(theta, &s, &c);
  return (float)atan2(s, c);
}

// theta = t0 + t1 on the integer ALU: t0 holds the top 24 significand bits
// of theta (truncated, so exact) and t1 the remaining 29 bits rounded to
// float (relative error 2^-24 of a term below 2^-23 |theta|).  For
// 2^-74 <= |theta| < 2^128; below, t1 = 0 (and t0 = +-0 under 2^-126).
__device__ __forceinline__ void f64_split2(double d, float &t0, float &t1) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(d);
  const uint32_t hi = (uint32_t)(b >> 32), lo = (uint32_t)b;
  const uint32_t sign = hi & 0x80000000u;
  const int e = (int)((hi >> 20) & 0x7ffu) - 1023;
  const uint32_t m = ((hi & 0xfffffu) << 3) | (lo >> 29);  // top 23 stored bits
  const uint32_t rest = lo & 0x1fffffffu;                    // value rest * 2^(e-52)
  t0 = e < -126 ? __uint_as_float(sign) : __uint_as_float(sign | ((uint32_t)(e + 127) << 23) | m);
  const int sc = e + 75;  // biased float exponent of 2^(e-52)
  const float r1 = __uint2float_rn(rest) * __uint_as_float((uint32_t)(sc > 0 ? sc : 1) << 23);
  t1 = sc > 0 ? __uint_as_float(__float_as_uint(r1) | sign) : 0.f;
}

// Reduce a double angle to [-pi, pi] in float arithmetic with an error of a
// few float ulps of pi, whatever |theta| (the double is never rounded to float
// before the reduction): theta = t0 + t1 (f64_split2), k = rint(t0 / 2pi),
// r = (t0 - k C1) - k C2 + t1 with 2*pi = C1 + C2 in floats; t0 - k C1 is
// exact in the FMA (for k != 0 both are multiples of 2^-22 and the
// difference is below 4).  The first omitted term, k (2pi - C1 - C2), is
// below 5e-9 for |theta| < 2^22.  |theta| >= 2^22, and results within a few
// ulp of +-pi (where k may be
// off by one, or theta sits on the branch cut), take the double reduction
// out of line, so that theta = pi (as a double) maps to +pi exactly as the
// reference's double arithmetic sees it.
__device__ __forceinline__ float reduce_angle(double theta) {
  const uint32_t ehi = ((uint32_t)((unsigned long long)__double_as_longlong(theta) >> 52)) & 0x7ffu;
  if (ehi >= 1023u + 22u) return reduce_angle_exact(theta);
  float t0, t1;
  f64_split2(theta, t0, t1);
  const float inv2pi = 0.15915494309189535f;
  const float c1 = 6.28318548202514648f;      // float nearest 2*pi (ulp 2^-21)
  const float c2 = -1.7484555314695172e-07f;  // 2*pi - c1
  const float k = rintf(t0 * inv2pi);
  float r = fmaf(-k, c1, t0);
  r = fmaf(-k, c2, r);
  r += t1;
  if (fabsf(r) > 3.1415920f) r = reduce_angle_exact(theta);
  return r;
}

// sin and cos of h for |h| <= pi/2 (+ rounding): the Taylor series of both
// about 0 in Horner form in z = h^2, through h^13 for sin and h^12 for cos.
// The first omitted terms, h^15/15! and h^14/14!, are below 7e-10 and 7e-9
// at |h| = pi/2, so the result is accurate to float rounding; 14 FMAs, no
// branches and no range reduction (the caller's angle is already reduced).
__device__ __forceinline__ void sincos_taylor(float h, float &s, float &c) {
  const float z = h * h;
  float ps = 1.6059043836821613e-10f;         // 1/13!
  ps = fmaf(ps, z, -2.5052108385441720e-08f);  // -1/11!
  ps = fmaf(ps, z, 2.7557319223985893e-06f);   // 1/9!
  ps = fmaf(ps, z, -1.9841269841269841e-04f);  // -1/7!
  ps = fmaf(ps, z, 8.3333333333333333e-03f);   // 1/5!
  ps = fmaf(ps, z, -1.6666666666666667e-01f);  // -1/3!
  s = fmaf(ps * z, h, h);
  float pc = 2.0876756987868099e-09f;          // 1/12!
  pc = fmaf(pc, z, -2.7557319223985888e-07f);  // -1/10!
  pc = fmaf(pc, z, 2.4801587301587302e-05f);   // 1/8!
  pc = fmaf(pc, z, -1.3888888888888889e-03f);  // -1/6!
  pc = fmaf(pc, z, 4.1666666666666667e-02f);   // 1/4!
  pc = fmaf(pc, z, -0.5f);                     // -1/2!
  c = fmaf(pc, z, 1.0f);
}

// sin and cos of an angle reduced to [-pi, pi], by the half-angle series
__device__ __forceinline__ void sincos_reduced(float r, float &s, float &c) {
  float sh, ch;
  sincos_taylor(0.5f * r, sh, ch);
  s = 2.f * sh * ch;
  c = fmaf(ch, ch, -sh * sh);
}

// Coefficients of a statevector step.  The unnormalised contraction is
//   phi = psi[a=0] + c * psi[a=1],  c = e^{-i theta}  (= sqrt(2) <+_theta| psi),
// with theta = 0 for plane X and pi/2 for plane Y (ment.py:231-235).  ``ph``
// is the global phase the reference's summing partial trace (state_ops.py:69)
// attaches to the step, (v0 + v1)/|v0 + v1| = e^{i theta_r/2} for theta
// reduced to [-pi, pi]: 1 for X, e^{i pi/4} for Y.
__device__ __forceinline__ void sv_coef(int plane, double theta, bool want_phase, float2 &c,
                                        float2 &ph) {
  if (plane == MBQC_PLANE_X) {
    c = make_float2(1.f, 0.f);
    ph = make_float2(1.f, 0.f);
    return;
  }
  if (plane == MBQC_PLANE_Y) {
    c = make_float2(0.f, -1.f);
    ph = make_float2(0.70710678118654752f, 0.70710678118654752f);
    return;
  }
  // half-angle form: one series evaluation gives the step phase
  // e^{i r/2} and the coefficient e^{-i r} = conj(e^{i r/2})^2
  const float r = reduce_angle(theta);
  float sh, ch;
  sincos_taylor(0.5f * r, sh, ch);
  c = make_float2(fmaf(ch, ch, -sh * sh), -2.f * sh * ch);
  ph = want_phase ? make_float2(ch, sh) : make_float2(1.f, 0.f);
}
__device__ __forceinline__ void sv_coef(int plane, double theta, bool want_phase, double2 &c,
                                        double2 &ph) {
  if (plane == MBQC_PLANE_X) {
    c = make_double2(1.0, 0.0);
    ph = make_double2(1.0, 0.0);
    return;
  }
  if (plane == MBQC_PLANE_Y) {
    c = make_double2(0.0, -1.0);
    ph = make_double2(0.7071067811865476, 0.7071067811865476);
    return;
  }
  // sin and cos of the double angle itself (full-range reduction), so the
  // coefficient is the reference's e^{-i theta} to a few ulp for any theta;
  // the phase e^{i r/2} with r = atan2(sin, cos) in [-pi, pi]
  double s, co;
  sincos(theta, &s, &co);
  c = make_double2(co, -s);
  if (want_phase) {
    const double r = atan2(s, co);
    sincos(0.5 * r, &s, &co);
    ph = make_double2(co, s);
  } else {
    ph = make_double2(1.0, 0.0);
  }
}

// Coefficients of a step in any plane: the unnormalised contraction is
//   phi = amp * psi[a=0] + c * psi[a=1]  (= sqrt(2) <v|psi>, amp >= 0 real),
// v the outcome-0 eigenvector of the step's projector (ment.py:218-260).  XY,
// X and Y give amp = 1 and sv_coef's c.  With C = cos(r/2), S = sin(r/2) for
// the angle reduced to [-pi, pi]:
//   XZ (n = (cos, 0, sin)): amp = C + S, c = C - S,      ph = 1;
//   YZ (n = (0, cos, sin)): amp = C + S, c = -i (C - S), ph = (C + S + i (C - S)) / sqrt(2);
// ph is the phase (v0 + v1)/|v0 + v1| that the reference's summing partial
// trace (state_ops.py:69) attaches to the step.  The reference statevector
// simulator rejects these planes (np_simulator_sv.py:53-59); this is its
// algorithm applied to them, which its density-matrix simulator pins.
__device__ __forceinline__ void sv_coef_gen(int plane, double theta, bool want_phase, float2 &c, float &amp,
                                            float2 &ph) {
  if (plane != MBQC_PLANE_XZ && plane != MBQC_PLANE_YZ) {
    amp = 1.f;
    sv_coef(plane, theta, want_phase, c, ph);
    return;
  }
  float sh, ch;
  sincos_taylor(0.5f * reduce_angle(theta), sh, ch);
  amp = ch + sh;
  float d = ch - sh;
  // amp < 0: the reference's phase (v0 + v1)/|v0 + v1| carries the sign
  // (v0 = sqrt(P0[0,0]) >= 0); the contraction drops it and ph takes it, so
  // that the output without the phase is the reference's with its phase
  // divided out (what the adjoint differentiates) and with it, unchanged
  const float sg = amp < 0.f ? -1.f : 1.f;
  amp *= sg;
  d *= sg;
  if (plane == MBQC_PLANE_XZ) {
    c = make_float2(d, 0.f);
    ph = make_float2(sg, 0.f);
  } else {
    c = make_float2(0.f, -d);
    ph = want_phase ? make_float2(0.70710678118654752f * amp, 0.70710678118654752f * d) : make_float2(1.f, 0.f);
  }
}
__device__ __forceinline__ void sv_coef_gen(int plane, double theta, bool want_phase, double2 &c, double &amp,
                                            double2 &ph) {
  if (plane != MBQC_PLANE_XZ && plane != MBQC_PLANE_YZ) {
    amp = 1.0;
    sv_coef(plane, theta, want_phase, c, ph);
    return;
  }
  double s, co;
  sincos(theta, &s, &co);
  double sh, ch;
  sincos(0.5 * atan2(s, co), &sh, &ch);
  amp = ch + sh;
  double d = ch - sh;
  const double sg = amp < 0.0 ? -1.0 : 1.0;  // as in the float version
  amp *= sg;
  d *= sg;
  if (plane == MBQC_PLANE_XZ) {
    c = make_double2(d, 0.0);
    ph = make_double2(sg, 0.0);
  } else {
    c = make_double2(0.0, -d);
    ph = want_phase ? make_double2(0.7071067811865476 * amp, 0.7071067811865476 * d) : make_double2(1.0, 0.0);
  }
}

template <typename CT> __device__ __forceinline__ CT cmul(CT a, CT b) {
  CT z;
  z.x = a.x * b.x - a.y * b.y;
  z.y = a.x * b.y + a.y * b.x;
  return z;
}

__device__ __forceinline__ int gather_bits(uint32_t idx, const int8_t *bits, int n) {
  int x = 0;
  for (int i = 0; i < n; ++i) x = (x << 1) | ((idx >> bits[i]) & 1u);
  return x;
}

// parity of the initial CZ layer at index idx
__device__ __forceinline__ uint32_t init_parity(uint32_t idx, const uint32_t *init_cz, int w) {
  uint32_t p = 0;
  for (int q = 0; q < w; ++q) p ^= ((idx >> q) & 1u) & (__popc(idx & init_cz[q]) & 1u);
  return p;
}

}  // namespace mbqc
