// Householder QR of a complex128 matrix, the per-block kernel of block_sparse_qr
// (pytenet/block_sparse_util.py:106-180, which calls numpy.linalg.qr per block).
//
// Reflector convention: the one of LAPACK's zlarfg / zgeqr2 / zung2r, so that Q
// and R agree with numpy.linalg.qr(mode="reduced") column by column, including
// the signs (R has a real diagonal, beta = -sign(Re alpha) * |(alpha, x)|, and a
// column whose sub-diagonal part and imaginary diagonal part vanish gets tau = 0,
// H = I). This matters beyond cosmetics: for rank-deficient site tensors (the
// README workload clamps bonds) the completion of Q determines the later sweep.
//
// Structure (blocked, compact WY):  for each panel of NB columns
//   panel kernel  : one CTA factors the panel column by column and builds the
//                   NB x NB triangular factor T with H_1..H_nb = I - V T V^H;
//   block update  : A_trail -= V (T^H (V^H A_trail)), as two grid-wide passes
//                   (partial V^H A per 64-row tile, then reduce + apply);
// then Q = H_1 ... H_k [I; 0] is formed backwards with the same block update
// (using T instead of T^H).
#include "ptn_common.cuh"
#include <algorithm>

namespace ptn {

void note_launches(int n);

namespace {

constexpr int NB = 16;     // panel width
constexpr int PT = 512;    // panel kernel threads
constexpr int RT = 64;     // rows per block-update tile
constexpr int CTL = 32;    // columns per block-update tile

__device__ __forceinline__ double2 crecip(double2 a) {
  const double s = 1.0 / (a.x * a.x + a.y * a.y);
  return c2(a.x * s, -a.y * s);
}

// warp-reduce NB complex values, then across warps through shared memory;
// result in out[0..cnt) (valid after the trailing __syncthreads).
__device__ __forceinline__ void block_reduce_vec(double2 (&v)[NB], int cnt, double2 (*red)[NB],
                                                 double2* out) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
#pragma unroll
  for (int c = 0; c < NB; ++c) {
    if (c < cnt) {
      double x = v[c].x, y = v[c].y;
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) {
        x += __shfl_xor_sync(0xffffffffu, x, o);
        y += __shfl_xor_sync(0xffffffffu, y, o);
      }
      if (lane == 0) red[wid][c] = c2(x, y);
    }
  }
  __syncthreads();
  if (threadIdx.x < cnt) {
    double2 s = c2(0.0, 0.0);
    for (int w = 0; w < nw; ++w) s = cadd(s, red[w][threadIdx.x]);
    out[threadIdx.x] = s;
  }
  __syncthreads();
}

__global__ void __launch_bounds__(PT) qr_panel_kernel(double2* __restrict__ a, long lda, int m,
                                                      int j0, int jb, double2* __restrict__ Tout,
                                                      double2* __restrict__ V, long ldv) {
  __shared__ double sh[33];
  __shared__ double2 red[PT / 32][NB];
  __shared__ double2 wv[NB];
  __shared__ double2 taus[NB];
  __shared__ double2 sT[NB][NB];
  __shared__ double2 s_scal;
  __shared__ double s_beta;
  __shared__ int s_apply;
  const int tid = threadIdx.x;

  for (int jj = 0; jj < jb; ++jj) {
    const int col = j0 + jj;
    double acc = 0.0;
    for (int i = col + 1 + tid; i < m; i += PT) {
      const double2 v = a[(long)i * lda + col];
      acc = fma(v.x, v.x, acc);
      acc = fma(v.y, v.y, acc);
    }
    const double xn2 = block_sum(acc, sh);
    if (tid == 0) {
      const double2 alpha = a[(long)col * lda + col];
      if (xn2 == 0.0 && alpha.y == 0.0) {
        taus[jj] = c2(0.0, 0.0);
        s_apply = 0;
      } else {
        const double beta = -copysign(sqrt(alpha.x * alpha.x + alpha.y * alpha.y + xn2), alpha.x);
        taus[jj] = c2((beta - alpha.x) / beta, -alpha.y / beta);
        s_scal = crecip(c2(alpha.x - beta, alpha.y));
        s_beta = beta;
        s_apply = 1;
      }
    }
    __syncthreads();
    const int apply = s_apply;
    if (apply) {
      const double2 sc = s_scal;
      for (int i = col + 1 + tid; i < m; i += PT) {
        double2* p = a + (long)i * lda + col;
        *p = cmul(*p, sc);
      }
      if (tid == 0) a[(long)col * lda + col] = c2(s_beta, 0.0);
    }
    __syncthreads();
    const int nrem = j0 + jb - col - 1;
    if (apply && nrem > 0) {
      // w_c = v^H a_c for the remaining panel columns (v_col = 1)
      double2 part[NB];
#pragma unroll
      for (int c = 0; c < NB; ++c) part[c] = c2(0.0, 0.0);
      for (int i = col + tid; i < m; i += PT) {
        const double2 v = (i == col) ? c2(1.0, 0.0) : a[(long)i * lda + col];
        const double2 vc = cconj(v);
        const double2* row = a + (long)i * lda + col + 1;
#pragma unroll
        for (int c = 0; c < NB; ++c)
          if (c < nrem) part[c] = cfma(vc, row[c], part[c]);
      }
      block_reduce_vec(part, nrem, red, wv);
      const double2 ctau = cconj(taus[jj]);
      for (int i = col + tid; i < m; i += PT) {
        const double2 v = (i == col) ? c2(1.0, 0.0) : a[(long)i * lda + col];
        const double2 f = cmul(ctau, v);
        double2* row = a + (long)i * lda + col + 1;
#pragma unroll
        for (int c = 0; c < NB; ++c)
          if (c < nrem) row[c] = csub(row[c], cmul(f, wv[c]));
      }
    }
    __syncthreads();
  }

  // explicit V (unit lower trapezoidal) for the panel columns, rows j0..m-1
  for (int i = j0 + tid; i < m; i += PT) {
    for (int c = 0; c < jb; ++c) {
      const int col = j0 + c;
      V[(long)i * ldv + col] = (i < col) ? c2(0.0, 0.0)
                               : (i == col) ? c2(1.0, 0.0) : a[(long)i * lda + col];
    }
  }
  if (tid < NB * NB) sT[tid / NB][tid % NB] = c2(0.0, 0.0);
  __syncthreads();

  // T (zlarft, forward columnwise): T[c][c] = tau_c,
  // T[0:c, c] = -tau_c * T[0:c, 0:c] * (V[:, 0:c]^H v_c)
  for (int c = 0; c < jb; ++c) {
    if (c > 0) {
      double2 part[NB];
#pragma unroll
      for (int p = 0; p < NB; ++p) part[p] = c2(0.0, 0.0);
      for (int i = j0 + c + tid; i < m; i += PT) {
        const double2 vc = V[(long)i * ldv + j0 + c];
#pragma unroll
        for (int p = 0; p < NB; ++p)
          if (p < c) part[p] = cfma(cconj(V[(long)i * ldv + j0 + p]), vc, part[p]);
      }
      block_reduce_vec(part, c, red, wv);
    }
    if (tid == 0) {
      const double2 tc = taus[c];
      for (int p = 0; p < c; ++p) {
        double2 s = c2(0.0, 0.0);
        for (int q = p; q < c; ++q) s = cadd(s, cmul(sT[p][q], wv[q]));
        sT[p][c] = cmul(c2(-tc.x, -tc.y), s);
      }
      sT[c][c] = tc;
    }
    __syncthreads();
  }
  if (tid < NB * NB) Tout[tid] = sT[tid / NB][tid % NB];
}

// partial[rb][j][c] = sum_{rows r of tile rb} conj(V[r][v0 + j]) C[r][c0 + c]
// lane layout: tr = lane & 7 (row phase), 4 columns per warp, 8 warps -> 32 columns.
__global__ void __launch_bounds__(256) larfb_partial_kernel(const double2* __restrict__ C, long ldc,
                                                            const double2* __restrict__ V, long ldv,
                                                            int r0, int m, int c0, int nc, int v0,
                                                            int jb, double2* __restrict__ part) {
  __shared__ double2 sv[RT][NB];
  const int rb = blockIdx.y;
  const int rbase = r0 + rb * RT;
  for (int idx = threadIdx.x; idx < RT * NB; idx += blockDim.x) {
    const int rr = idx / NB, j = idx % NB;
    const int r = rbase + rr;
    sv[rr][j] = (r < m && j < jb) ? V[(long)r * ldv + v0 + j] : c2(0.0, 0.0);
  }
  __syncthreads();
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const int tr = lane & 7;
  const int cc = wid * 4 + (lane >> 3);
  const int c = c0 + blockIdx.x * CTL + cc;
  double2 acc[NB];
#pragma unroll
  for (int j = 0; j < NB; ++j) acc[j] = c2(0.0, 0.0);
  if (c < c0 + nc) {
    for (int rr = tr; rr < RT; rr += 8) {
      const int r = rbase + rr;
      if (r >= m) break;
      const double2 x = C[(long)r * ldc + c];
#pragma unroll
      for (int j = 0; j < NB; ++j)
        if (j < jb) acc[j] = cfma(cconj(sv[rr][j]), x, acc[j]);
    }
  }
#pragma unroll
  for (int j = 0; j < NB; ++j) {
#pragma unroll
    for (int o = 1; o < 8; o <<= 1) {
      acc[j].x += __shfl_xor_sync(0xffffffffu, acc[j].x, o);
      acc[j].y += __shfl_xor_sync(0xffffffffu, acc[j].y, o);
    }
  }
  if (tr == 0 && c < c0 + nc) {
#pragma unroll
    for (int j = 0; j < NB; ++j)
      if (j < jb) part[((long)rb * NB + j) * nc + (c - c0)] = acc[j];
  }
}

// W = sum_rb partial; W2 = op(T) W (op = T^H if conjT else T); C -= V W2 on this tile
__global__ void __launch_bounds__(256) larfb_update_kernel(double2* __restrict__ C, long ldc,
                                                           const double2* __restrict__ V, long ldv,
                                                           int r0, int m, int c0, int nc, int v0,
                                                           int jb, const double2* __restrict__ part,
                                                           int nrb, const double2* __restrict__ T,
                                                           int conjT) {
  __shared__ double2 sv[RT][NB];
  __shared__ double2 sw[NB][CTL];
  __shared__ double2 sw2[NB][CTL];
  __shared__ double2 sT[NB][NB];
  const int rb = blockIdx.y;
  const int rbase = r0 + rb * RT;
  for (int idx = threadIdx.x; idx < RT * NB; idx += blockDim.x) {
    const int rr = idx / NB, j = idx % NB;
    const int r = rbase + rr;
    sv[rr][j] = (r < m && j < jb) ? V[(long)r * ldv + v0 + j] : c2(0.0, 0.0);
  }
  if (threadIdx.x < NB * NB) sT[threadIdx.x / NB][threadIdx.x % NB] = T[threadIdx.x];
  for (int idx = threadIdx.x; idx < NB * CTL; idx += blockDim.x) {
    const int j = idx / CTL, cc = idx % CTL;
    const int c = blockIdx.x * CTL + cc;
    double2 s = c2(0.0, 0.0);
    if (j < jb && c < nc)
      for (int b = 0; b < nrb; ++b) s = cadd(s, part[((long)b * NB + j) * nc + c]);
    sw[j][cc] = s;
  }
  __syncthreads();
  for (int idx = threadIdx.x; idx < NB * CTL; idx += blockDim.x) {
    const int j = idx / CTL, cc = idx % CTL;
    double2 s = c2(0.0, 0.0);
    if (j < jb) {
      if (conjT) {
        for (int q = 0; q <= j; ++q) s = cadd(s, cmul(cconj(sT[q][j]), sw[q][cc]));
      } else {
        for (int q = j; q < jb; ++q) s = cadd(s, cmul(sT[j][q], sw[q][cc]));
      }
    }
    sw2[j][cc] = s;
  }
  __syncthreads();
  const int tc = threadIdx.x & 31, tr = threadIdx.x >> 5;
  const int c = c0 + blockIdx.x * CTL + tc;
  if (c >= c0 + nc) return;
  for (int rr = tr; rr < RT; rr += 8) {
    const int r = rbase + rr;
    if (r >= m) break;
    double2 x = C[(long)r * ldc + c];
#pragma unroll
    for (int j = 0; j < NB; ++j)
      if (j < jb) x = csub(x, cmul(sv[rr][j], sw2[j][tc]));
    C[(long)r * ldc + c] = x;
  }
}

__global__ void extract_r_kernel(const double2* __restrict__ a, long lda, int k, int n,
                                 double2* __restrict__ r, long ldr) {
  const long total = (long)k * n;
  for (long idx = blockIdx.x * (long)blockDim.x + threadIdx.x; idx < total;
       idx += (long)gridDim.x * blockDim.x) {
    const int i = (int)(idx / n), c = (int)(idx % n);
    r[(long)i * ldr + c] = (c >= i) ? a[(long)i * lda + c] : c2(0.0, 0.0);
  }
}

__global__ void eye_kernel(double2* __restrict__ q, long ldq, int m, int k) {
  const long total = (long)m * k;
  for (long idx = blockIdx.x * (long)blockDim.x + threadIdx.x; idx < total;
       idx += (long)gridDim.x * blockDim.x) {
    const int i = (int)(idx / k), c = (int)(idx % k);
    q[(long)i * ldq + c] = c2(i == c ? 1.0 : 0.0, 0.0);
  }
}

inline size_t al(size_t b) { return (b + 255) & ~size_t(255); }

struct QrWs {
  double2* V;
  double2* T;
  double2* part;
};

QrWs carve_qr(void* ws, int m, int n) {
  const int k = std::min(m, n);
  const int np = (k + NB - 1) / NB;
  char* p = static_cast<char*>(ws);
  QrWs w;
  w.V = reinterpret_cast<double2*>(p);
  p += al((size_t)m * k * sizeof(double2));
  w.T = reinterpret_cast<double2*>(p);
  p += al((size_t)np * NB * NB * sizeof(double2));
  w.part = reinterpret_cast<double2*>(p);
  return w;
}

ptn_status larfb(double2* C, long ldc, const double2* V, long ldv, int r0, int m, int c0, int nc,
                 int v0, int jb, const double2* T, bool conjT, double2* part, cudaStream_t st) {
  const int nrb = (m - r0 + RT - 1) / RT;
  dim3 grid((nc + CTL - 1) / CTL, nrb);
  larfb_partial_kernel<<<grid, 256, 0, st>>>(C, ldc, V, ldv, r0, m, c0, nc, v0, jb, part);
  larfb_update_kernel<<<grid, 256, 0, st>>>(C, ldc, V, ldv, r0, m, c0, nc, v0, jb, part, nrb, T,
                                            conjT ? 1 : 0);
  PTN_LAUNCH_CHECK();
  note_launches(2);
  return PTN_OK;
}

}  // namespace

size_t qr_workspace_bytes(int m, int n) {
  const int k = std::min(m, n);
  const int np = (k + NB - 1) / NB;
  const int nrb = (m + RT - 1) / RT;
  return al((size_t)m * k * sizeof(double2)) + al((size_t)np * NB * NB * sizeof(double2)) +
         al((size_t)nrb * NB * std::max(n, k) * sizeof(double2));
}

ptn_status qr(double2* a, int m, int n, double2* q, long ldq, double2* r, long ldr, void* ws,
              size_t ws_bytes, cudaStream_t st) {
  PTN_CHECK_ARG(m > 0 && n > 0, "qr: empty matrix (%d x %d)", m, n);
  PTN_CHECK_ARG(ws_bytes >= qr_workspace_bytes(m, n), "qr: workspace too small");
  const int k = std::min(m, n);
  QrWs w = carve_qr(ws, m, n);
  const long lda = n;
  // LAPACK flop count of zgeqrf + zungqr (4 real flops per complex op)
  const double fq = 8.0 * ((double)m * n * k - (double)(m + n) * k * k / 2.0 + (double)k * k * k / 3.0);
  const int prof = prof_begin(st, PROF_QR, 2.0 * fq, 16.0 * 3.0 * m * n);
  for (int j0 = 0, p = 0; j0 < k; j0 += NB, ++p) {
    const int jb = std::min(NB, k - j0);
    qr_panel_kernel<<<1, PT, 0, st>>>(a, lda, m, j0, jb, w.T + (long)p * NB * NB, w.V, k);
    PTN_LAUNCH_CHECK();
    note_launches(1);
    const int nc = n - j0 - jb;
    if (nc > 0)
      PTN_TRY(larfb(a, lda, w.V, k, j0, m, j0 + jb, nc, j0, jb, w.T + (long)p * NB * NB, true,
                    w.part, st));
  }
  const int blocks = std::max(1, std::min(4 * num_sms(), (int)(((long)k * n + 255) / 256)));
  extract_r_kernel<<<blocks, 256, 0, st>>>(a, lda, k, n, r, ldr);
  const int qblocks = std::max(1, std::min(4 * num_sms(), (int)(((long)m * k + 255) / 256)));
  eye_kernel<<<qblocks, 256, 0, st>>>(q, ldq, m, k);
  PTN_LAUNCH_CHECK();
  note_launches(2);
  const int np = (k + NB - 1) / NB;
  for (int p = np - 1; p >= 0; --p) {
    const int j0 = p * NB;
    const int jb = std::min(NB, k - j0);
    PTN_TRY(larfb(q, ldq, w.V, k, j0, m, j0, k - j0, j0, jb, w.T + (long)p * NB * NB, false,
                  w.part, st));
  }
  prof_end(st, prof);
  return PTN_OK;
}

}  // namespace ptn

extern "C" {

size_t ptn_qr_workspace_bytes(int m, int n) { return ptn::qr_workspace_bytes(m, n); }

ptn_status ptn_qr(ptn_c128* a, int m, int n, ptn_c128* q, long ldq, ptn_c128* r, long ldr,
                  void* ws, size_t ws_bytes, void* stream) {
  return ptn::qr(reinterpret_cast<double2*>(a), m, n, reinterpret_cast<double2*>(q), ldq,
                 reinterpret_cast<double2*>(r), ldr, ws, ws_bytes, ptn::as_stream(stream));
}

}  // extern "C"
