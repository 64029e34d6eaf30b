// C ABI of libmbqc_gb300: plan upload, error reporting and kernel dispatch.
#include <cstdlib>
#include <cuda_runtime.h>

#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "common.cuh"
#include "dispatch.h"

struct mbqc_plan {
  int n_circuits = 0;
  int max_w = 0;
  int device = 0;
  std::vector<mbqc::DevCircuit> h_circ;
  std::vector<mbqc::DevStep> h_steps;
  std::vector<int2> h_map;
  mbqc::DevCircuit *d_circ = nullptr;
  mbqc::DevStep *d_steps = nullptr;
  int2 *d_map = nullptr;
  mbqc::DevItem *d_items = nullptr;
  int64_t n_steps_total = 0;
  int64_t map_total = 0;
};

namespace mbqc {

static thread_local std::string g_err;

int fail(int code, const char *fmt, ...) {
  char buf[1024];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  g_err = buf;
  return code;
}

int cuda_check(cudaError_t e, const char *what) {
  if (e == cudaSuccess) return MBQC_OK;
  return fail(MBQC_E_CUDA, "%s: %s", what, cudaGetErrorString(e));
}

int check_launch(const char *what) { return cuda_check(cudaGetLastError(), what); }

PlanView view_of(const mbqc_plan *p) {
  PlanView v;
  v.d_circ = p->d_circ;
  v.d_steps = p->d_steps;
  v.d_map = p->d_map;
  v.d_items = p->d_items;
  v.n_circuits = p->n_circuits;
  v.max_w = p->max_w;
  return v;
}

const DevCircuit &host_circuit(const mbqc_plan *p, int i) { return p->h_circ[i]; }

const int2 *host_map(const mbqc_plan *p, int i) {
  const int64_t off = p->h_circ[i].map_off;
  return off >= 0 ? p->h_map.data() + off : nullptr;
}

const DevStep *host_steps(const mbqc_plan *p, int i) { return p->h_steps.data() + p->h_circ[i].step_off; }

bool pdl_enabled() {
  static int on = -1;
  if (on < 0) {
    const char *e = getenv("MBQC_PDL");
    on = (e && e[0] == '0') ? 0 : 1;
  }
  return on != 0;
}

int sm_count() {
  static int sms = 0;
  if (!sms) {
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (sms <= 0) sms = 152;
  }
  return sms;
}

// Item table of one circuit (appended to out): angle items 0..A-1 in angle
// order, then the fixed-angle steps in step order.  Returns its offset, or -1
// when the angle indices are not a permutation of 0..A-1 (then kernels stage
// in step order).
static int32_t build_items(const mbqc_circuit_desc &d, std::vector<DevItem> &out) {
  const int M = d.n_steps, A = d.n_angles;
  std::vector<int> of_angle(A > 0 ? A : 1, -1);
  int seen = 0;
  for (int k = 0; k < M; ++k) {
    const int a = d.step_angle[k];
    if (a < 0) continue;
    if (a >= A || of_angle[a] != -1) return -1;
    of_angle[a] = k;
    ++seen;
  }
  if (seen != A) return -1;
  const int32_t off = (int32_t)out.size();
  for (int a = 0; a < A; ++a) {
    DevItem it;
    it.step = of_angle[a];
    it.plane = d.step_plane[it.step];
    it.fixed = 0.0;
    out.push_back(it);
  }
  for (int k = 0; k < M; ++k)
    if (d.step_angle[k] < 0) {
      DevItem it;
      it.step = k;
      it.plane = d.step_plane[k];
      it.fixed = d.step_fixed_angle[k];
      out.push_back(it);
    }
  return off;
}

static void build_map(const mbqc_circuit_desc &d, std::vector<int2> &out) {
  const int w = d.window;
  const uint32_t full = (w >= 32) ? 0xffffffffu : ((1u << w) - 1u);
  uint32_t omask = 0;
  for (int j = 0; j < d.n_out; ++j) omask |= 1u << d.out_bits[j];
  for (uint32_t idx = 0; idx < (1u << w); ++idx) {
    uint32_t x = 0;
    for (int i = 0; i < d.n_in; ++i) x = (x << 1) | ((idx >> d.in_bits[i]) & 1u);
    uint32_t par = 0;
    for (int q = 0; q < w; ++q)
      par ^= ((idx >> q) & 1u) & (__builtin_popcount(idx & d.init_cz[q]) & 1u);
    int y = -1;
    if ((idx & full & ~omask) == 0) {
      uint32_t yy = 0;
      for (int j = 0; j < d.n_out; ++j) yy = (yy << 1) | ((idx >> d.out_bits[j]) & 1u);
      y = (int)yy;
    }
    out.push_back(make_int2((int)(x | (par << 31)), y));
  }
}

}  // namespace mbqc

using namespace mbqc;

extern "C" {

int mbqc_abi_version(void) { return MBQC_ABI_VERSION; }

const char *mbqc_last_error(void) { return g_err.c_str(); }

int mbqc_device_sm_count(int32_t *sm_count) {
  int dev = 0;
  int rc = cuda_check(cudaGetDevice(&dev), "cudaGetDevice");
  if (rc) return rc;
  int v = 0;
  rc = cuda_check(cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev),
                  "cudaDeviceGetAttribute");
  if (rc) return rc;
  *sm_count = v;
  return MBQC_OK;
}

int mbqc_mapped_pointer(const void *host, void **device_ptr) {
  if (!host || !device_ptr) return fail(MBQC_E_INVALID, "mapped_pointer: null argument");
  cudaPointerAttributes at;
  const cudaError_t e = cudaPointerGetAttributes(&at, host);
  if (e != cudaSuccess) {
    cudaGetLastError();
    return fail(MBQC_E_INVALID, "mapped_pointer: %s", cudaGetErrorString(e));
  }
  if (at.type != cudaMemoryTypeHost || at.devicePointer == nullptr)
    return fail(MBQC_E_INVALID, "mapped_pointer: %p is not page-locked host memory mapped for the device",
                host);
  *device_ptr = at.devicePointer;
  return MBQC_OK;
}

int mbqc_plan_create(const mbqc_circuit_desc *circuits, int32_t n_circuits, mbqc_plan **plan) {
  if (!plan) return fail(MBQC_E_INVALID, "plan_create: null output pointer");
  *plan = nullptr;
  if (!circuits || n_circuits <= 0) return fail(MBQC_E_INVALID, "plan_create: no circuits");
  std::vector<DevCircuit> hc(n_circuits);
  std::vector<DevStep> hs;
  std::vector<int2> hm;
  std::vector<DevItem> hi;
  int max_w = 0;
  for (int c = 0; c < n_circuits; ++c) {
    const mbqc_circuit_desc &d = circuits[c];
    if (d.window < 1 || d.window > kMaxWindow)
      return fail(MBQC_E_UNSUPPORTED, "circuit %d: window %d outside 1..%d", c, d.window, kMaxWindow);
    if (d.n_in < 0 || d.n_in > d.window || d.n_out < 0 || d.n_out > d.window || d.n_steps < 0 ||
        d.n_angles < 0)
      return fail(MBQC_E_INVALID, "circuit %d: inconsistent sizes", c);
    if ((d.n_in && !d.in_bits) || (d.n_out && !d.out_bits) || !d.init_cz ||
        (d.n_steps && (!d.step_mask || !d.step_angle || !d.step_plane || !d.step_fixed_angle)))
      return fail(MBQC_E_INVALID, "circuit %d: missing table", c);
    DevCircuit &h = hc[c];
    std::memset(&h, 0, sizeof(h));
    h.w = d.window;
    h.n_steps = d.n_steps;
    h.n_in = d.n_in;
    h.n_out = d.n_out;
    h.n_angles = d.n_angles;
    h.step_off = (int32_t)hs.size();
    uint32_t seen = 0;
    for (int i = 0; i < d.n_in; ++i) {
      if (d.in_bits[i] < 0 || d.in_bits[i] >= d.window || ((seen >> d.in_bits[i]) & 1u))
        return fail(MBQC_E_INVALID, "circuit %d: bad input bit %d", c, d.in_bits[i]);
      seen |= 1u << d.in_bits[i];
      h.in_bits[i] = (int8_t)d.in_bits[i];
    }
    seen = 0;
    for (int j = 0; j < d.n_out; ++j) {
      if (d.out_bits[j] < 0 || d.out_bits[j] >= d.window || ((seen >> d.out_bits[j]) & 1u))
        return fail(MBQC_E_INVALID, "circuit %d: bad output bit %d", c, d.out_bits[j]);
      seen |= 1u << d.out_bits[j];
      h.out_bits[j] = (int8_t)d.out_bits[j];
    }
    h.out_mask = seen;
    const uint32_t full = (d.window >= 32) ? 0xffffffffu : ((1u << d.window) - 1u);
    for (int q = 0; q < d.window; ++q) {
      if (d.init_cz[q] & ~full) return fail(MBQC_E_INVALID, "circuit %d: bad initial CZ mask", c);
      h.init_cz[q] = d.init_cz[q];
    }
    int n_dead = 0;
    h.sv_planes_ok = 1;
    h.sv_xz_ok = 1;
    h.has_z = 0;
    for (int k = 0; k < d.n_steps; ++k) {
      DevStep s;
      s.mask = d.step_mask[k];
      if (s.mask & kDead) {
        s.mask = kDead;
        ++n_dead;
      } else if (s.mask & ~full) {
        return fail(MBQC_E_INVALID, "circuit %d step %d: CZ mask outside the window", c, k);
      } else if ((s.mask >> (k % d.window)) & 1u) {
        return fail(MBQC_E_INVALID, "circuit %d step %d: entering qubit linked to itself", c, k);
      }
      s.aidx = d.step_angle[k];
      if (s.aidx < -1 || s.aidx >= d.n_angles)
        return fail(MBQC_E_INVALID, "circuit %d step %d: angle index %d", c, k, s.aidx);
      s.plane = d.step_plane[k];
      if (s.plane < MBQC_PLANE_XY || s.plane > MBQC_PLANE_Z)
        return fail(MBQC_E_INVALID, "circuit %d step %d: plane %d", c, k, s.plane);
      if (s.plane > MBQC_PLANE_Y) h.sv_planes_ok = 0;
      if (s.plane == MBQC_PLANE_Z) h.has_z = 1, h.sv_xz_ok = 0;
      s.pad = 0;
      s.fixed = d.step_fixed_angle[k];
      hs.push_back(s);
    }
    // the window must shrink to exactly the outputs
    if (d.window - n_dead != d.n_out)
      return fail(MBQC_E_INVALID, "circuit %d: window %d with %d shrinking steps leaves %d qubits, "
                  "not %d outputs", c, d.window, n_dead, d.window - n_dead, d.n_out);
    h.n_dead = n_dead;
    h.lp_const = -(d.window - d.n_in) - 2 * (d.n_steps - n_dead) - n_dead;
    if (d.window <= kMapMaxWindow) {
      h.map_off = (int64_t)hm.size();
      build_map(d, hm);
    } else {
      h.map_off = -1;
    }
    h.item_off = build_items(d, hi);
    if (d.window > max_w) max_w = d.window;
  }

  mbqc_plan *p = new (std::nothrow) mbqc_plan();
  if (!p) return fail(MBQC_E_NOMEM, "plan_create: out of host memory");
  p->n_circuits = n_circuits;
  p->max_w = max_w;
  p->h_circ = hc;
  p->h_steps = hs;
  p->h_map = hm;
  p->n_steps_total = (int64_t)hs.size();
  p->map_total = (int64_t)hm.size();
  int rc = cuda_check(cudaGetDevice(&p->device), "cudaGetDevice");
  if (!rc) rc = cuda_check(cudaMalloc(&p->d_circ, sizeof(DevCircuit) * n_circuits), "cudaMalloc(plan)");
  if (!rc && !hs.empty())
    rc = cuda_check(cudaMalloc(&p->d_steps, sizeof(DevStep) * hs.size()), "cudaMalloc(steps)");
  if (!rc && !hm.empty())
    rc = cuda_check(cudaMalloc(&p->d_map, sizeof(int2) * hm.size()), "cudaMalloc(map)");
  if (!rc && !hi.empty())
    rc = cuda_check(cudaMalloc(&p->d_items, sizeof(DevItem) * hi.size()), "cudaMalloc(items)");
  if (!rc)
    rc = cuda_check(cudaMemcpy(p->d_circ, hc.data(), sizeof(DevCircuit) * n_circuits,
                               cudaMemcpyHostToDevice), "upload plan");
  if (!rc && !hs.empty())
    rc = cuda_check(cudaMemcpy(p->d_steps, hs.data(), sizeof(DevStep) * hs.size(),
                               cudaMemcpyHostToDevice), "upload steps");
  if (!rc && !hm.empty())
    rc = cuda_check(cudaMemcpy(p->d_map, hm.data(), sizeof(int2) * hm.size(), cudaMemcpyHostToDevice),
                    "upload map");
  if (!rc && !hi.empty())
    rc = cuda_check(cudaMemcpy(p->d_items, hi.data(), sizeof(DevItem) * hi.size(), cudaMemcpyHostToDevice),
                    "upload items");
  if (rc) {
    mbqc_plan_destroy(p);
    return rc;
  }
  *plan = p;
  return MBQC_OK;
}

int mbqc_plan_destroy(mbqc_plan *plan) {
  if (!plan) return MBQC_OK;
  cudaFree(plan->d_circ);
  cudaFree(plan->d_steps);
  cudaFree(plan->d_map);
  cudaFree(plan->d_items);
  delete plan;
  return MBQC_OK;
}

}  // extern "C"
