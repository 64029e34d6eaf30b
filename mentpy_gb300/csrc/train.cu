// Device-side optimizer step for whole training runs on the GPU.
#include <cuda_runtime.h>

#include <cmath>

#include "dispatch.h"

namespace mbqc {

// Adam on n FP64 parameters (mentpy/optimizers/adam.py:54-66):
//   m = b1 m + (1 - b1) g,  v = b2 v + (1 - b2) g^2,
//   x -= lr * (m / c1) / (sqrt(v / c2) + eps),  c1 = 1 - b1^(i+1), c2 = 1 - b2^(i+1).
// c1, c2 come from the device state block, so that a captured graph can
// replay the step for every iteration.
__global__ void adam_kernel(int64_t n, double *__restrict__ x, const double *__restrict__ g,
                            double *__restrict__ m, double *__restrict__ v, const double *__restrict__ state,
                            double lr, double b1, double b2, double eps) {
  const double c1 = state[1], c2 = state[2];
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const double gi = g[i];
    const double mi = b1 * m[i] + (1.0 - b1) * gi;
    const double vi = b2 * v[i] + (1.0 - b2) * gi * gi;
    m[i] = mi;
    v[i] = vi;
    x[i] = x[i] - lr * (mi / c1) / (sqrt(vi / c2) + eps);
  }
}

// state = {i, 1 - b1^(i+1), 1 - b2^(i+1)} -> the same for i + 1
__global__ void adam_advance(double *state, double b1, double b2) {
  const double i = state[0] + 1.0;
  state[0] = i;
  state[1] = 1.0 - pow(b1, i + 1.0);
  state[2] = 1.0 - pow(b2, i + 1.0);
}

}  // namespace mbqc

using namespace mbqc;

extern "C" {

int mbqc_adam_state_init(double *state, double b1, double b2, mbqc_stream_t stream) {
  if (!state) return fail(MBQC_E_INVALID, "adam_state_init: null state");
  const double h[3] = {0.0, 1.0 - b1, 1.0 - b2};
  return cuda_check(cudaMemcpyAsync(state, h, sizeof(h), cudaMemcpyHostToDevice, (cudaStream_t)stream),
                    "adam_state_init");
}

int mbqc_adam_step(int64_t n, double *x, const double *g, double *m, double *v, double *state, double lr,
                   double b1, double b2, double eps, mbqc_stream_t stream) {
  if (n < 0 || (n > 0 && (!x || !g || !m || !v)) || !state) return fail(MBQC_E_INVALID, "adam_step: bad arguments");
  cudaStream_t s = (cudaStream_t)stream;
  if (n > 0) {
    int64_t blocks = (n + 255) / 256;
    const int64_t cap = (int64_t)sm_count() * 8;
    if (blocks > cap) blocks = cap;
    adam_kernel<<<(int)blocks, 256, 0, s>>>(n, x, g, m, v, state, lr, b1, b2, eps);
    const int rc = check_launch("adam_kernel");
    if (rc) return rc;
  }
  adam_advance<<<1, 1, 0, s>>>(state, b1, b2);
  return check_launch("adam_advance");
}

}  // extern "C"
