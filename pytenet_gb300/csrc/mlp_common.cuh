// Forward pass of the 12 -> 64 -> 64 -> 1 GELU MLP of the learned Lanczos depth,
// shared by the training kernels (mlp.cu) and the in-sweep predictor (krylov.cu).
#pragma once
#include <cuda_runtime.h>

namespace ptn {
namespace mlpdef {

constexpr int NI = 12, NH = 64;
constexpr int OFF_W1 = 0;
constexpr int OFF_B1 = OFF_W1 + NH * NI;
constexpr int OFF_W2 = OFF_B1 + NH;
constexpr int OFF_B2 = OFF_W2 + NH * NH;
constexpr int OFF_W3 = OFF_B2 + NH;
constexpr int OFF_B3 = OFF_W3 + NH;
constexpr int NPARAM = OFF_B3 + 1;

__device__ __forceinline__ float gelu(float x) {
  return 0.5f * x * (1.0f + erff(x * 0.70710678118654752f));
}

__device__ __forceinline__ float gelu_grad(float x) {
  const float cdf = 0.5f * (1.0f + erff(x * 0.70710678118654752f));
  const float pdf = 0.39894228040143268f * expf(-0.5f * x * x);
  return cdf + x * pdf;
}

// one warp, all lanes: returns the network output in every lane
__device__ __forceinline__ float forward_warp(const float* __restrict__ p, const float* x) {
  const int lane = threadIdx.x & 31;
  float h1[2], h2[2];
#pragma unroll
  for (int u = 0; u < 2; ++u) {
    const int j = lane + 32 * u;
    float s = p[OFF_B1 + j];
#pragma unroll
    for (int k = 0; k < NI; ++k) s = fmaf(p[OFF_W1 + j * NI + k], x[k], s);
    h1[u] = gelu(s);
  }
  float s2[2] = {p[OFF_B2 + lane], p[OFF_B2 + lane + 32]};
  for (int k = 0; k < NH; ++k) {
    const float hk = __shfl_sync(0xffffffffu, h1[k >> 5], k & 31);
    s2[0] = fmaf(p[OFF_W2 + lane * NH + k], hk, s2[0]);
    s2[1] = fmaf(p[OFF_W2 + (lane + 32) * NH + k], hk, s2[1]);
  }
  h2[0] = gelu(s2[0]);
  h2[1] = gelu(s2[1]);
  float y = p[OFF_W3 + lane] * h2[0] + p[OFF_W3 + lane + 32] * h2[1];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) y += __shfl_xor_sync(0xffffffffu, y, o);
  return y + p[OFF_B3];
}

}  // namespace mlpdef
}  // namespace ptn
