// Uneven density-matrix batches in one persistent launch.
//
// Thousands of circuits of different windows and depths (one run each) run
// in a single kernel launch: the host sorts the circuits into tiles (runs of
// one window that a 256-thread block executes together, TPR threads per
// run, the tile shape chosen per window by the caller's tuner), orders the
// tiles longest first, and every resident block claims the next tile with
// one atomicAdd until the list is exhausted.  No block waits on another:
// the last block to finish resets the claim counters for the next launch on
// the stream, so a captured CUDA graph can replay the launch.
//
// The per-run arithmetic is the factored density-matrix sweep (dm_fact.cuh)
// of NumpySimulatorDM.run (np_simulator_dm.py:218-346), one call per circuit
// in the reference.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>
#include <vector>

#include "dispatch.h"
#include "dm_fact.cuh"

namespace mbqc {

struct DmTile {
  int32_t w, tpr, first, count;  // window, threads per run, runs [first, first + count) of the run list
};

// (window, threads per run) pairs compiled into the persistent kernel
__host__ __device__ constexpr bool dm_tile_shape_ok(int w, int tpr) {
  return (w >= 2 && w <= 4 && tpr == 32) || (w == 5 && (tpr == 32 || tpr == 64)) ||
         (w == 6 && (tpr == 32 || tpr == 64 || tpr == 128)) ||
         (w == 7 && (tpr == 64 || tpr == 128 || tpr == 256)) || (w == 8 && tpr == 256);
}

template <int W, int TPR>
__device__ __forceinline__ void dm_tile_run(const DmArgs &A, const DmTile &t, unsigned char *smem) {
  const int group = threadIdx.x / TPR, tid = threadIdx.x % TPR;
  if (group < t.count)
    dm_fact_run<W, TPR>(A, (int64_t)t.first + group, tid, group,
                        smem + (size_t)group * dm_fact_slice_bytes<W>(A.maxm));
}

// A.run_circuit is the tile-ordered run list: slot s simulates circuit
// run_circuit[s] and every per-run array is indexed by that circuit.
__global__ void __launch_bounds__(256, 3) dm_fwd_persist(DmArgs A, const DmTile *tiles, int n_tiles,
                                                      int *counters) {
  extern __shared__ __align__(16) unsigned char smem_p[];
  __shared__ int s_tile;
  for (;;) {
    if (threadIdx.x == 0) s_tile = atomicAdd(&counters[0], 1);
    __syncthreads();
    const int ti = s_tile;
    __syncthreads();  // everyone has read the claim before the next one overwrites it
    if (ti >= n_tiles) break;
    const DmTile t = tiles[ti];
    switch (t.w * 512 + t.tpr) {
#define MBQC_TILE(W, TPR) \
  case W * 512 + TPR:     \
    dm_tile_run<W, TPR>(A, t, smem_p); \
    break;
      MBQC_TILE(2, 32)
      MBQC_TILE(3, 32)
      MBQC_TILE(4, 32)
      MBQC_TILE(5, 32)
      MBQC_TILE(5, 64)
      MBQC_TILE(6, 32)
      MBQC_TILE(6, 64)
      MBQC_TILE(6, 128)
      MBQC_TILE(7, 64)
      MBQC_TILE(7, 128)
      MBQC_TILE(7, 256)
      MBQC_TILE(8, 256)
#undef MBQC_TILE
      default:
        break;  // the host builds only compiled shapes
    }
    __syncthreads();  // the slice is reused by the next tile
  }
  // the last block out resets the claim counter for the next launch
  if (threadIdx.x == 0) {
    __threadfence();
    if (atomicAdd(&counters[1], 1) == (int)gridDim.x - 1) {
      counters[0] = 0;
      counters[1] = 0;
      __threadfence();
    }
  }
}

static size_t tile_smem(int w, int tpr, int maxm) {
  size_t slice = 0;
  switch (w) {
    case 2: slice = dm_fact_slice_bytes<2>(maxm); break;
    case 3: slice = dm_fact_slice_bytes<3>(maxm); break;
    case 4: slice = dm_fact_slice_bytes<4>(maxm); break;
    case 5: slice = dm_fact_slice_bytes<5>(maxm); break;
    case 6: slice = dm_fact_slice_bytes<6>(maxm); break;
    case 7: slice = dm_fact_slice_bytes<7>(maxm); break;
    case 8: slice = dm_fact_slice_bytes<8>(maxm); break;
    default: return 0;
  }
  return slice * (size_t)(256 / tpr);
}

static int default_tpr(int w) {
  switch (w) {
    case 2: return DmFactCfg<2>::TPR;
    case 3: return DmFactCfg<3>::TPR;
    case 4: return DmFactCfg<4>::TPR;
    case 5: return DmFactCfg<5>::TPR;
    case 6: return DmFactCfg<6>::TPR;
    case 7: return DmFactCfg<7>::TPR;
    default: return DmFactCfg<8>::TPR;
  }
}

}  // namespace mbqc

using namespace mbqc;

struct mbqc_dm_batch {
  const mbqc_plan *plan = nullptr;
  int n_runs = 0, n_tiles = 0, maxm = 1, max_in = 0, max_out = 0, max_a = 0;
  int blocks = 0;
  size_t smem = 0;
  int tpr[9] = {0};
  int32_t *d_runs = nullptr;
  DmTile *d_tiles = nullptr;
  int *d_counters = nullptr;
};

extern "C" int mbqc_dm_batch_destroy(mbqc_dm_batch *b) {
  if (!b) return MBQC_OK;
  cudaFree(b->d_runs);
  cudaFree(b->d_tiles);
  cudaFree(b->d_counters);
  delete b;
  return MBQC_OK;
}

extern "C" int mbqc_dm_batch_create_ex(const mbqc_plan *plan, int32_t n_circuits, const int32_t *tile_tpr,
                                       const int32_t *long_tpr, const int32_t *long_steps, int32_t blocks_per_sm,
                                       mbqc_dm_batch **out);

extern "C" int mbqc_dm_batch_create(const mbqc_plan *plan, int32_t n_circuits, const int32_t *tile_tpr,
                                    int32_t blocks_per_sm, mbqc_dm_batch **out) {
  return mbqc_dm_batch_create_ex(plan, n_circuits, tile_tpr, nullptr, nullptr, blocks_per_sm, out);
}

extern "C" int mbqc_dm_batch_create_ex(const mbqc_plan *plan, int32_t n_circuits, const int32_t *tile_tpr,
                                       const int32_t *long_tpr, const int32_t *long_steps, int32_t blocks_per_sm,
                                       mbqc_dm_batch **out) {
  if (!plan || !out) return fail(MBQC_E_INVALID, "dm_batch: null argument");
  *out = nullptr;
  const PlanView v = view_of(plan);
  if (n_circuits < 1 || n_circuits > v.n_circuits)
    return fail(MBQC_E_INVALID, "dm_batch: %d circuits of a %d-circuit plan", n_circuits, v.n_circuits);
  auto *b = new mbqc_dm_batch();
  b->plan = plan;
  b->n_runs = n_circuits;
  for (int w = 2; w <= 8; ++w) {
    const int t = tile_tpr ? tile_tpr[w] : 0;
    b->tpr[w] = t > 0 ? t : default_tpr(w);
    if (!dm_tile_shape_ok(w, b->tpr[w])) {
      mbqc_dm_batch_destroy(b);
      return fail(MBQC_E_INVALID, "dm_batch: no tile shape of %d threads per run at window %d", t, w);
    }
  }
  // circuits by window, longest first within a window; then tiles of the
  // window's runs per block, all tiles longest first
  std::vector<std::vector<int>> byw(9);
  for (int c = 0; c < n_circuits; ++c) {
    const DevCircuit &hc = host_circuit(plan, c);
    if (hc.w < 2 || hc.w > 8 || hc.n_steps < 1 || !(host_steps(plan, c)[hc.n_steps - 1].mask & kDead)) {
      mbqc_dm_batch_destroy(b);
      return fail(MBQC_E_UNSUPPORTED,
                  "dm_batch: circuit %d (window %d, %d steps) is outside the factored kernel (windows 2..8, "
                  "a last step that shrinks the window)", c, hc.w, hc.n_steps);
    }
    byw[hc.w].push_back(c);
    b->maxm = std::max(b->maxm, hc.n_steps);
    b->max_in = std::max(b->max_in, hc.n_in);
    b->max_out = std::max(b->max_out, hc.n_out);
    b->max_a = std::max(b->max_a, hc.n_angles);
  }
  struct HostTile {
    DmTile t;
    double cost;
  };
  std::vector<HostTile> tiles;
  std::vector<int32_t> runs;
  for (int w = 2; w <= 8; ++w) {
    auto &cs = byw[w];
    if (cs.empty()) continue;
    std::stable_sort(cs.begin(), cs.end(), [&](int x, int y) {
      return host_circuit(plan, x).n_steps > host_circuit(plan, y).n_steps;
    });
    // the circuits of at least long_steps[w] steps (the head of the sorted
    // list) may take their own tile shape: more threads per run shorten the
    // longest runs, which end the batch
    const int lt = (long_tpr && long_tpr[w] > 0) ? long_tpr[w] : b->tpr[w];
    if (!dm_tile_shape_ok(w, lt)) {
      mbqc_dm_batch_destroy(b);
      return fail(MBQC_E_INVALID, "dm_batch: no tile shape of %d threads per run at window %d", lt, w);
    }
    size_t nlong = 0;
    if (long_steps && long_steps[w] > 0)
      while (nlong < cs.size() && host_circuit(plan, cs[nlong]).n_steps >= long_steps[w]) ++nlong;
    b->smem = std::max(b->smem, tile_smem(w, b->tpr[w], b->maxm));
    if (nlong) b->smem = std::max(b->smem, tile_smem(w, lt, b->maxm));
    for (int part = 0; part < 2; ++part) {
      const int tpr = part == 0 ? lt : b->tpr[w];
      const size_t i0 = part == 0 ? 0 : nlong, i1 = part == 0 ? nlong : cs.size();
      const size_t g = (size_t)(256 / tpr);
      for (size_t i = i0; i < i1; i += g) {
        const int cnt = (int)std::min<size_t>(g, i1 - i);
        // time of a tile: its longest run, each step moving the 4^(w-1)-entry
        // matrix through shared memory, plus a fixed per-run part
        const double cost = (double)host_circuit(plan, cs[i]).n_steps * (double)(1u << (2 * (w - 1))) + 2048.0;
        tiles.push_back({DmTile{w, tpr, (int)i, cnt}, cost});  // first: within the window's list
      }
    }
  }
  std::stable_sort(tiles.begin(), tiles.end(), [](const HostTile &x, const HostTile &y) { return x.cost > y.cost; });
  std::vector<DmTile> dt;
  dt.reserve(tiles.size());
  for (auto &ht : tiles) {
    DmTile t = ht.t;
    const int off = (int)runs.size();
    for (int j = 0; j < t.count; ++j) runs.push_back(byw[t.w][t.first + j]);
    t.first = off;
    dt.push_back(t);
  }
  b->n_tiles = (int)dt.size();
  if (b->smem > (size_t)227 * 1024) {
    mbqc_dm_batch_destroy(b);
    return fail(MBQC_E_UNSUPPORTED, "dm_batch: %d steps need %zu bytes of shared memory per block", b->maxm,
                b->smem);
  }
  int rc = cuda_check(cudaFuncSetAttribute(dm_fwd_persist, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                           (int)b->smem),
                      "dm_batch smem attribute");
  if (!rc)
    rc = cuda_check(cudaFuncSetAttribute(dm_fwd_persist, cudaFuncAttributePreferredSharedMemoryCarveout,
                                         (int)cudaSharedmemCarveoutMaxShared),
                    "dm_batch carveout attribute");
  int occ = 0;
  if (!rc)
    rc = cuda_check(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, dm_fwd_persist, 256, b->smem),
                    "dm_batch occupancy");
  if (!rc && occ < 1) rc = fail(MBQC_E_UNSUPPORTED, "dm_batch: the persistent kernel does not fit on an SM");
  if (rc) {
    mbqc_dm_batch_destroy(b);
    return rc;
  }
  const int per_sm = blocks_per_sm > 0 ? std::min(blocks_per_sm, occ) : occ;
  b->blocks = std::max(1, std::min(sm_count() * per_sm, b->n_tiles));
  rc = cuda_check(cudaMalloc(&b->d_runs, sizeof(int32_t) * runs.size()), "cudaMalloc(dm_batch runs)");
  if (!rc) rc = cuda_check(cudaMalloc(&b->d_tiles, sizeof(DmTile) * dt.size()), "cudaMalloc(dm_batch tiles)");
  if (!rc) rc = cuda_check(cudaMalloc(&b->d_counters, 2 * sizeof(int)), "cudaMalloc(dm_batch counters)");
  if (!rc)
    rc = cuda_check(cudaMemcpy(b->d_runs, runs.data(), sizeof(int32_t) * runs.size(), cudaMemcpyHostToDevice),
                    "upload dm_batch runs");
  if (!rc)
    rc = cuda_check(cudaMemcpy(b->d_tiles, dt.data(), sizeof(DmTile) * dt.size(), cudaMemcpyHostToDevice),
                    "upload dm_batch tiles");
  if (!rc) rc = cuda_check(cudaMemset(b->d_counters, 0, 2 * sizeof(int)), "clear dm_batch counters");
  if (rc) {
    mbqc_dm_batch_destroy(b);
    return rc;
  }
  *out = b;
  return MBQC_OK;
}

extern "C" int mbqc_dm_batch_info(const mbqc_dm_batch *b, int32_t *info) {
  if (!b || !info) return fail(MBQC_E_INVALID, "dm_batch_info: null argument");
  info[0] = b->n_tiles;
  info[1] = b->blocks;
  info[2] = (int32_t)b->smem;
  for (int w = 2; w <= 8; ++w) info[1 + w] = b->tpr[w];
  return MBQC_OK;
}

extern "C" int mbqc_dm_batch_forward(const mbqc_dm_batch *b, const double *angles, int64_t angle_stride,
                                     const float *psi_in, int64_t in_stride, float *rho_out, int64_t out_stride,
                                     double noise, int8_t *outcomes, double *probs, int64_t outcome_stride,
                                     int32_t *status, uint32_t flags, uint64_t seed, mbqc_stream_t stream) {
  if (!b) return fail(MBQC_E_INVALID, "dm_batch_forward: null batch");
  if (!psi_in || !rho_out) return fail(MBQC_E_INVALID, "dm_batch_forward: null buffer");
  if (!(noise >= 0.0 && noise <= 1.0)) return fail(MBQC_E_INVALID, "dm_batch_forward: noise %g", noise);
  if (b->max_a > 0 && (!angles || angle_stride < b->max_a))
    return fail(MBQC_E_INVALID, "dm_batch_forward: angle stride %lld < %d", (long long)angle_stride, b->max_a);
  if (in_stride != 0 && in_stride < ((int64_t)1 << b->max_in))
    return fail(MBQC_E_INVALID, "dm_batch_forward: input stride too small");
  if (out_stride < ((int64_t)1 << (2 * b->max_out)))
    return fail(MBQC_E_INVALID, "dm_batch_forward: output stride too small");
  if ((outcomes || probs) && outcome_stride < b->maxm)
    return fail(MBQC_E_INVALID, "dm_batch_forward: outcome stride too small");
  const PlanView v = view_of(b->plan);
  DmArgs a{};
  a.circ = v.d_circ;
  a.steps = v.d_steps;
  a.maps = v.d_map;
  a.run_circuit = b->d_runs;
  a.B = b->n_runs;
  a.angles = angles;
  a.astride = angle_stride;
  a.psi_in = reinterpret_cast<const float2 *>(psi_in);
  a.istride = in_stride;
  a.rho_out = reinterpret_cast<float2 *>(rho_out);
  a.out_stride = out_stride;
  a.noise = noise;
  a.outcomes = outcomes;
  a.ostride = outcome_stride;
  a.probs = probs;
  a.status = status;
  a.maxm = b->maxm;
  a.flags = flags;
  a.seed = seed;
  dm_fwd_persist<<<b->blocks, 256, b->smem, (cudaStream_t)stream>>>(a, b->d_tiles, b->n_tiles, b->d_counters);
  return check_launch("dm_fwd_persist");
}
