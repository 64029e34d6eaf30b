// Internal declarations shared by the translation units of libmbqc_gb300.
#pragma once

#include <utility>

#include "common.cuh"

namespace mbqc {

struct SvArgs;

int fail(int code, const char *fmt, ...);
int cuda_check(cudaError_t e, const char *what);
int check_launch(const char *what);
PlanView view_of(const mbqc_plan *p);
const DevCircuit &host_circuit(const mbqc_plan *p, int i);
const DevStep *host_steps(const mbqc_plan *p, int i);
// host copy of circuit i's index map (nullptr above the map's window limit)
const int2 *host_map(const mbqc_plan *p, int i);

// register-resident statevector kernels, one translation unit per window;
// the _gen launchers run plans with XZ / YZ steps (one lane layout each:
// sv_gen_ll for float, sv_f64_ll for double)
#define MBQC_DECL_SV(W)                                                                          \
  int launch_sv_reg_f32_w##W(int ll, const SvArgs &a, int blocks, int threads, cudaStream_t s);  \
  int launch_sv_reg_f64_w##W(int ll, const SvArgs &a, int blocks, int threads, cudaStream_t s);  \
  int launch_sv_reg_gen_f32_w##W(const SvArgs &a, int blocks, int threads, cudaStream_t s);      \
  int launch_sv_reg_gen_f64_w##W(const SvArgs &a, int blocks, int threads, cudaStream_t s);
MBQC_DECL_SV(1)
MBQC_DECL_SV(2)
MBQC_DECL_SV(3)
MBQC_DECL_SV(4)
MBQC_DECL_SV(5)
MBQC_DECL_SV(6)
MBQC_DECL_SV(7)
MBQC_DECL_SV(8)
MBQC_DECL_SV(9)
MBQC_DECL_SV(10)
#undef MBQC_DECL_SV

constexpr int kSvRegMaxWindow = 10;

// adjoint kernels (windows 1..8)
struct SvAdjArgs;
struct AdjLaunch {
  int blocks, threads;
  size_t smem;
  bool query;  // only report occupancy into *occ
  int *occ;
};
#define MBQC_DECL_ADJ(W)                                                               \
  int launch_sv_adj_f32_w##W(const SvAdjArgs &a, const AdjLaunch &l, cudaStream_t s); \
  int launch_sv_adj_f64_w##W(const SvAdjArgs &a, const AdjLaunch &l, cudaStream_t s);
MBQC_DECL_ADJ(1)
MBQC_DECL_ADJ(2)
MBQC_DECL_ADJ(3)
MBQC_DECL_ADJ(4)
MBQC_DECL_ADJ(5)
MBQC_DECL_ADJ(6)
MBQC_DECL_ADJ(7)
MBQC_DECL_ADJ(8)
#undef MBQC_DECL_ADJ

// adjoint kernels for windows 9..20 and general-plane plans (a block per run, sv_adj_wide.cu)
struct WideAdjGeom {
  int8_t in_bits[32];
  int8_t out_bits[32];
  uint32_t init_cz[32];
  uint32_t out_mask;
  int64_t slot_elems;  // complex64 elements of one run slot of the workspace
  int cluster;         // blocks sharing a run (1, 2 or 4; windows >= 15 only)
};
constexpr int kWideAdjMaxWindow = 20;
constexpr size_t kWideAdjMaxWorkspace = (size_t)16 << 30;
// gen: plans with XZ / YZ steps (any window up to kWideAdjMaxWindow)
int launch_sv_adj_wide(const SvAdjArgs &a, const WideAdjGeom &g, const AdjLaunch &l, cudaStream_t s, bool gen);
int wide_adj_threads(int w);
size_t wide_adj_smem(int w, int M, bool gen);

int sm_count();

// Programmatic dependent launch: a kernel launched this way may start while
// the previous kernel on its stream is still running; it must execute
// griddep_wait() before touching any memory that kernel could write (and
// before its own global writes).  MBQC_PDL=0 in the environment turns the
// attribute off.
bool pdl_enabled();
template <typename... P, typename... A>
inline cudaError_t launch_pdl(void (*k)(P...), dim3 grid, dim3 block, size_t smem, cudaStream_t s,
                              A &&...args) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = grid;
  cfg.blockDim = block;
  cfg.dynamicSmemBytes = smem;
  cfg.stream = s;
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  at[0].val.programmaticStreamSerializationAllowed = pdl_enabled() ? 1 : 0;
  cfg.attrs = at;
  cfg.numAttrs = 1;
  return cudaLaunchKernelEx(&cfg, k, std::forward<A>(args)...);
}

// log2(lanes per run) of the FP64 instantiation for window w
constexpr int sv_f64_ll(int w) { return w - 4 > 1 ? (w - 4 < 5 ? w - 4 : 5) : 1; }
// log2(lanes per run) of the general-plane float instantiation (16 amplitudes per lane at most)
constexpr int sv_gen_ll(int w) { return w - 4 > 0 ? (w - 4 < 5 ? w - 4 : 5) : 0; }

}  // namespace mbqc
