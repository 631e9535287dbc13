// Shared definitions for the GB300 single-site TDVP / DMRG engine.
// Complex128 values are stored as double2 {re, im}: the memory layout of
// numpy.complex128 / torch.complex128, so host arrays map 1:1 onto device buffers.
#pragma once

#include <cuda_runtime.h>
#include <cstdint>
#include <cstddef>

#include "../../include/pytenet_gb300.h"

namespace ptn {

// ---------------------------------------------------------------------------
// error plumbing: every C entry point returns a ptn_status; the message of the
// last failure is kept per host thread for ptn_last_error().
// ---------------------------------------------------------------------------
void set_error(const char* fmt, ...);

#define PTN_CHECK_ARG(cond, ...)                                   \
  do {                                                             \
    if (!(cond)) { ::ptn::set_error(__VA_ARGS__); return PTN_BAD_SHAPE; } \
  } while (0)

#define PTN_CUDA_TRY(expr)                                                        \
  do {                                                                            \
    cudaError_t _e = (expr);                                                      \
    if (_e != cudaSuccess) {                                                      \
      ::ptn::set_error("%s:%d %s: %s", __FILE__, __LINE__, #expr, cudaGetErrorString(_e)); \
      return PTN_CUDA_ERROR;                                                      \
    }                                                                             \
  } while (0)

#define PTN_LAUNCH_CHECK() PTN_CUDA_TRY(cudaGetLastError())

#define PTN_TRY(expr)                         \
  do {                                        \
    ptn_status _s = (expr);                   \
    if (_s != PTN_OK) return _s;              \
  } while (0)

inline cudaStream_t as_stream(void* s) { return reinterpret_cast<cudaStream_t>(s); }

int num_sms();
// tuning knob value (ptn_tune_set); key is one of the PTN_TUNE_* constants
int tune(int key);

// ---------------------------------------------------------------------------
// live kernel timing (off by default): launchers bracket a kernel of `kind`
// with CUDA events on its stream and record the algorithmic flops / bytes of
// the launch; ptn_prof_read sums the event intervals after a synchronise.
// Nothing is recorded while the stream is being captured into a graph.
// ---------------------------------------------------------------------------
enum ProfKind { PROF_ZGEMM_F64 = 0, PROF_TC_GEMM = 1, PROF_MPO_STAGE = 2, PROF_QR = 3,
                PROF_KRYLOV = 4, PROF_NKINDS = 5 };
int prof_begin(cudaStream_t st, int kind, double flops, double bytes);
void prof_end(cudaStream_t st, int slot);

// ---------------------------------------------------------------------------
// complex helpers
// ---------------------------------------------------------------------------
__host__ __device__ __forceinline__ double2 c2(double re, double im) { return make_double2(re, im); }
__host__ __device__ __forceinline__ double2 cadd(double2 a, double2 b) { return c2(a.x + b.x, a.y + b.y); }
__host__ __device__ __forceinline__ double2 csub(double2 a, double2 b) { return c2(a.x - b.x, a.y - b.y); }
__host__ __device__ __forceinline__ double2 cmul(double2 a, double2 b) {
  return c2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
__host__ __device__ __forceinline__ double2 cconj(double2 a) { return c2(a.x, -a.y); }
__host__ __device__ __forceinline__ double2 cscale(double2 a, double s) { return c2(a.x * s, a.y * s); }
// acc + a * b
__device__ __forceinline__ double2 cfma(double2 a, double2 b, double2 acc) {
  acc.x = fma(a.x, b.x, acc.x);
  acc.x = fma(-a.y, b.y, acc.x);
  acc.y = fma(a.x, b.y, acc.y);
  acc.y = fma(a.y, b.x, acc.y);
  return acc;
}

// ---------------------------------------------------------------------------
// block-level reductions (blockDim.x a multiple of 32, <= 1024)
// ---------------------------------------------------------------------------
__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// Sum over the block; result valid in every thread. `sh` needs 33 doubles.
__device__ __forceinline__ double block_sum(double v, double* sh) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
  v = warp_sum(v);
  __syncthreads();
  if (lane == 0) sh[wid] = v;
  __syncthreads();
  double t = (threadIdx.x < nw) ? sh[threadIdx.x] : 0.0;
  if (wid == 0) {
    t = warp_sum(t);
    if (lane == 0) sh[32] = t;
  }
  __syncthreads();
  return sh[32];
}

// ---------------------------------------------------------------------------
// complex GEMM (FP64): C = alpha * op(A) * op(B) + beta * C, row-major.
// op: 'N' plain, 'T' transpose, 'C' conjugate, 'H' conjugate transpose.
// Batched over `batch` with element strides sA/sB/sC. An optional device flag
// `skip` (non-null) makes the launch a no-op when *skip != 0; the Krylov loop
// uses it to retire iterations after a Lanczos breakdown without host syncs.
// ---------------------------------------------------------------------------
struct GemmArgs {
  int M, N, K;
  char opA, opB;
  double2 alpha, beta;
  const double2* A; long lda; long sA;
  const double2* B; long ldb; long sB;
  double2* C; long ldc; long sC;
  int batch;
  const int* skip;
};

// Workspace (bytes) a zgemm call may use for split-K partial sums.
size_t zgemm_workspace_bytes(int M, int N, int K, int batch);
ptn_status zgemm(const GemmArgs& g, void* ws, size_t ws_bytes, cudaStream_t st);

}  // namespace ptn
