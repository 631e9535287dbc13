// Learned Lanczos depth: a 12 -> 64 -> 64 -> 1 FP32 MLP with GELU activations,
// trained and evaluated by these kernels only.
//
// Parameters are one contiguous FP32 vector:
//   W1[64][12], b1[64], W2[64][64], b2[64], W3[64], b3[1]     (5057 values)
// Training step (deterministic, no atomics):
//   1. per-sample kernel: forward pass, store z1, h1, z2, h2 and the output
//      derivative dL/dy of the mean-squared loss; back-propagate to dz2, dz1;
//   2. per-parameter kernel: one thread per parameter sums its gradient over the
//      batch in a fixed order (plus the loss);
//   3. Adam update.
// The predictor kernel runs one forward pass for the feature vector of the
// current local step and writes the Lanczos depth to use.
#include "ptn_common.cuh"
#include "mlp_common.cuh"
#include <algorithm>

namespace ptn {

void note_launches(int n);

namespace {

using namespace mlpdef;
constexpr int CACHE = 4 * NH + 1;   // per sample: h1, h2, dz1, dz2 (64 each) and dL/dy

__device__ float forward_one(const float* __restrict__ p, const float* __restrict__ x, float* z1,
                             float* h1, float* z2, float* h2) {
  for (int j = 0; j < NH; ++j) {
    float s = p[OFF_B1 + j];
#pragma unroll
    for (int k = 0; k < NI; ++k) s = fmaf(p[OFF_W1 + j * NI + k], x[k], s);
    z1[j] = s;
    h1[j] = gelu(s);
  }
  for (int j = 0; j < NH; ++j) {
    float s = p[OFF_B2 + j];
    for (int k = 0; k < NH; ++k) s = fmaf(p[OFF_W2 + j * NH + k], h1[k], s);
    z2[j] = s;
    h2[j] = gelu(s);
  }
  float y = p[OFF_B3];
  for (int k = 0; k < NH; ++k) y = fmaf(p[OFF_W3 + k], h2[k], y);
  return y;
}

__global__ void mlp_forward_kernel(const float* __restrict__ params, const float* __restrict__ X,
                                   int B, float* __restrict__ Y) {
  __shared__ float p[NPARAM];
  for (int i = threadIdx.x; i < NPARAM; i += blockDim.x) p[i] = params[i];
  __syncthreads();
  for (int b = blockIdx.x * blockDim.x + threadIdx.x; b < B; b += gridDim.x * blockDim.x) {
    float z1[NH], h1[NH], z2[NH], h2[NH];
    Y[b] = forward_one(p, X + (long)b * NI, z1, h1, z2, h2);
  }
}

// cache per sample: h1[64], h2[64], dz1[64], dz2[64], dy  -> 4*64+1 floats
__global__ void mlp_backprop_kernel(const float* __restrict__ params, const float* __restrict__ X,
                                    const float* __restrict__ T, int B, float* __restrict__ cache,
                                    float* __restrict__ sqerr) {
  __shared__ float p[NPARAM];
  for (int i = threadIdx.x; i < NPARAM; i += blockDim.x) p[i] = params[i];
  __syncthreads();
  for (int b = blockIdx.x * blockDim.x + threadIdx.x; b < B; b += gridDim.x * blockDim.x) {
    float z1[NH], h1[NH], z2[NH], h2[NH];
    const float y = forward_one(p, X + (long)b * NI, z1, h1, z2, h2);
    const float r = y - T[b];
    sqerr[b] = r * r;
    const float dy = 2.0f * r / (float)B;
    float* c = cache + (long)b * CACHE;
    float dz2[NH];
    for (int j = 0; j < NH; ++j) {
      dz2[j] = dy * p[OFF_W3 + j] * gelu_grad(z2[j]);
      c[j] = h1[j];
      c[NH + j] = h2[j];
      c[3 * NH + j] = dz2[j];
    }
    for (int k = 0; k < NH; ++k) {
      float s = 0.f;
      for (int j = 0; j < NH; ++j) s = fmaf(p[OFF_W2 + j * NH + k], dz2[j], s);
      c[2 * NH + k] = s * gelu_grad(z1[k]);
    }
    c[4 * NH] = dy;
  }
}

// one thread per parameter: gradient summed over the batch in sample order
__global__ void mlp_gradsum_kernel(const float* __restrict__ X, int B, const float* __restrict__ cache,
                                   const float* __restrict__ sqerr, float* __restrict__ grad,
                                   float* __restrict__ loss) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i > NPARAM) return;
  float s = 0.f;
  if (i == NPARAM) {   // loss = mean squared error
    for (int b = 0; b < B; ++b) s += sqerr[b];
    *loss = s / (float)B;
    return;
  }
  for (int b = 0; b < B; ++b) {
    const float* c = cache + (long)b * CACHE;
    const float* x = X + (long)b * NI;
    float g;
    if (i < OFF_B1) { const int j = i / NI, k = i % NI; g = c[2 * NH + j] * x[k]; }
    else if (i < OFF_W2) { g = c[2 * NH + (i - OFF_B1)]; }
    else if (i < OFF_B2) { const int t = i - OFF_W2, j = t / NH, k = t % NH; g = c[3 * NH + j] * c[k]; }
    else if (i < OFF_W3) { g = c[3 * NH + (i - OFF_B2)]; }
    else if (i < OFF_B3) { g = c[4 * NH] * c[NH + (i - OFF_W3)]; }
    else { g = c[4 * NH]; }
    s += g;
  }
  grad[i] = s;
}

__global__ void mlp_adam_kernel(float* __restrict__ params, const float* __restrict__ grad,
                                float* __restrict__ m, float* __restrict__ v, float lr, float b1,
                                float b2, float eps, int step) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= NPARAM) return;
  const float g = grad[i];
  const float mi = b1 * m[i] + (1.f - b1) * g;
  const float vi = b2 * v[i] + (1.f - b2) * g * g;
  m[i] = mi;
  v[i] = vi;
  const float mh = mi / (1.f - powf(b1, (float)step));
  const float vh = vi / (1.f - powf(b2, (float)step));
  params[i] -= lr * mh / (sqrtf(vh) + eps);
}

}  // namespace

int mlp_param_count() { return NPARAM; }
int mlp_cache_floats() { return CACHE; }

ptn_status mlp_forward(const float* params, const float* X, int B, float* Y, cudaStream_t st) {
  if (B <= 0) return PTN_OK;
  const int blocks = std::min((B + 127) / 128, 4 * num_sms());
  mlp_forward_kernel<<<blocks, 128, 0, st>>>(params, X, B, Y);
  PTN_LAUNCH_CHECK();
  note_launches(1);
  return PTN_OK;
}

size_t mlp_workspace_bytes(int B) { return ((size_t)B * CACHE + (size_t)B + 256) * sizeof(float); }

ptn_status mlp_grad(const float* params, const float* X, const float* T, int B, float* grad,
                    float* loss, void* ws, size_t ws_bytes, cudaStream_t st) {
  PTN_CHECK_ARG(B > 0 && ws_bytes >= mlp_workspace_bytes(B), "mlp: workspace too small");
  float* cache = static_cast<float*>(ws);
  float* sq = cache + (size_t)B * CACHE;
  const int blocks = std::min((B + 127) / 128, 4 * num_sms());
  mlp_backprop_kernel<<<blocks, 128, 0, st>>>(params, X, T, B, cache, sq);
  mlp_gradsum_kernel<<<(NPARAM + 1 + 127) / 128, 128, 0, st>>>(X, B, cache, sq, grad, loss);
  PTN_LAUNCH_CHECK();
  note_launches(2);
  return PTN_OK;
}

ptn_status mlp_adam(float* params, const float* grad, float* m, float* v, float lr, float b1,
                    float b2, float eps, int step, cudaStream_t st) {
  mlp_adam_kernel<<<(NPARAM + 127) / 128, 128, 0, st>>>(params, grad, m, v, lr, b1, b2, eps, step);
  PTN_LAUNCH_CHECK();
  note_launches(1);
  return PTN_OK;
}

}  // namespace ptn

using namespace ptn;

extern "C" {

int ptn_mlp_param_count(void) { return mlp_param_count(); }
size_t ptn_mlp_workspace_bytes(int batch) { return mlp_workspace_bytes(batch); }

ptn_status ptn_mlp_forward(const float* params, const float* X, int batch, float* Y, void* stream) {
  return mlp_forward(params, X, batch, Y, as_stream(stream));
}

ptn_status ptn_mlp_grad(const float* params, const float* X, const float* T, int batch, float* grad,
                        float* loss, void* ws, size_t ws_bytes, void* stream) {
  return mlp_grad(params, X, T, batch, grad, loss, ws, ws_bytes, as_stream(stream));
}

ptn_status ptn_mlp_adam(float* params, const float* grad, float* m, float* v, float lr, float beta1,
                        float beta2, float eps, int step, void* stream) {
  return mlp_adam(params, grad, m, v, lr, beta1, beta2, eps, step, as_stream(stream));
}

}  // extern "C"
