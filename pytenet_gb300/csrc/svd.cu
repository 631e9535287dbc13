// Thin singular value decomposition of a complex128 matrix: the per-block kernel of
// block_sparse_svd (pytenet/block_sparse_util.py:244-330, which calls
// numpy.linalg.svd(full_matrices=False) per quantum-number block) and so of the
// two-site splits (pytenet/bond_ops.py:41-53, pytenet/mps.py:538-568).
//
// Method: one-sided Jacobi (Hestenes) in FP64. The columns of W (A, or A^H when A
// is wide, so that W is p x r with p >= r) are orthogonalised pairwise: for a pair
// (j, k) with Gram entries a = |w_j|^2, b = |w_k|^2, c = w_j^H w_k = |c| e^{i phi},
// w_k is first turned by e^{-i phi} (which makes the pair's Gram entry real) and
// then the real Jacobi rotation with zeta = (b - a) / (2 |c|),
// t = sign(zeta) / (|zeta| + sqrt(1 + zeta^2)), cs = 1 / sqrt(1 + t^2), sn = cs t
// zeroes it: w_j <- cs w_j - sn w_k, w_k <- sn w_j + cs w_k. The same unitary column
// operations accumulate in V (r x r, starting at I). Pairs follow the round-robin
// (circle) order, r/2 disjoint pairs per round, one warp per pair; a sweep is
// r - 1 rounds; sweeps repeat until no pair has |c| > tol sqrt(a b)
// (tol = p * eps), at most MAX_SWEEPS of them. Then s_j = |w_j|, the columns are
// sorted by decreasing s (ties by index, LAPACK's order), U = W / s, and
// A = U diag(s) V^H (for a wide A the roles of U and V swap).
//
// Singular vectors of one singular value are unique only up to a phase (or a
// unitary mix for repeated values): they need not equal LAPACK's, while the
// singular values, the products U diag(s) V^H and every quantity built from a
// truncated split agree to rounding.
//
// One CTA per matrix: for the block sizes of quantum-number blocks and of the
// two-site steps at moderate bond dimension (hundreds); larger dense blocks take
// O(r^2 p) FP64 work per sweep on a single SM.
#include "ptn_common.cuh"
#include <algorithm>

namespace ptn {

void note_launches(int n);

namespace {

constexpr int ST = 256;           // threads per CTA
constexpr int NWARP = ST / 32;
constexpr int MAX_SWEEPS = 60;

__device__ __forceinline__ double warp_sum(double x) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
  return x;
}

// W (p x r) and V (r x r) are column-major scratch; u, vh row-major outputs.
__global__ void __launch_bounds__(ST) svd_jacobi_kernel(const double2* __restrict__ a, int m, int n,
                                                       long lda, double2* __restrict__ W,
                                                       double2* __restrict__ V,
                                                       double* __restrict__ sig,
                                                       int* __restrict__ pos, double2* __restrict__ u,
                                                       long ldu, double* __restrict__ s,
                                                       double2* __restrict__ vh, long ldvh,
                                                       int* __restrict__ sweeps_out) {
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const bool wide = m < n;
  const int p = wide ? n : m, r = wide ? m : n;
  for (long e = tid; e < (long)p * r; e += ST) {
    const int j = (int)(e / p), i = (int)(e % p);
    W[e] = wide ? cconj(a[(long)j * lda + i]) : a[(long)i * lda + j];
  }
  for (long e = tid; e < (long)r * r; e += ST) V[e] = c2((e / r == e % r) ? 1.0 : 0.0, 0.0);
  __shared__ int s_rot;
  __syncthreads();
  const double tol = (double)p * 2.220446049250313e-16;
  const int rr = r + (r & 1);   // an odd count plays against an absent column
  int sweep = 0;
  for (; sweep < MAX_SWEEPS; ++sweep) {
    if (tid == 0) s_rot = 0;
    __syncthreads();
    for (int q = 0; q < rr - 1; ++q) {
      for (int t = warp; t < rr / 2; t += NWARP) {
        int j, k;
        if (t == 0) {
          j = 0;
          k = 1 + q;
        } else {
          j = 1 + (q + t) % (rr - 1);
          k = 1 + (q + rr - 1 - t) % (rr - 1);
        }
        if (j > k) {
          const int x = j;
          j = k;
          k = x;
        }
        if (k >= r) continue;
        double2* wj = W + (long)j * p;
        double2* wk = W + (long)k * p;
        double aa = 0.0, bb = 0.0, cr = 0.0, ci = 0.0;
        for (int i = lane; i < p; i += 32) {
          const double2 x = wj[i], y = wk[i];
          aa = fma(x.x, x.x, fma(x.y, x.y, aa));
          bb = fma(y.x, y.x, fma(y.y, y.y, bb));
          cr = fma(x.x, y.x, fma(x.y, y.y, cr));   // conj(x) y
          ci = fma(x.x, y.y, fma(-x.y, y.x, ci));
        }
        aa = warp_sum(aa);
        bb = warp_sum(bb);
        cr = warp_sum(cr);
        ci = warp_sum(ci);
        const double ac = sqrt(cr * cr + ci * ci);
        if (!(ac > 0.0) || !(ac > tol * sqrt(aa) * sqrt(bb))) continue;
        const double2 ph = c2(cr / ac, -ci / ac);   // e^{-i phi}
        const double zeta = (bb - aa) / (2.0 * ac);
        const double tt = copysign(1.0, zeta) / (fabs(zeta) + sqrt(1.0 + zeta * zeta));
        const double cs = 1.0 / sqrt(1.0 + tt * tt), sn = cs * tt;
        for (int i = lane; i < p; i += 32) {
          const double2 x = wj[i], y = cmul(wk[i], ph);
          wj[i] = c2(cs * x.x - sn * y.x, cs * x.y - sn * y.y);
          wk[i] = c2(sn * x.x + cs * y.x, sn * x.y + cs * y.y);
        }
        double2* vj = V + (long)j * r;
        double2* vk = V + (long)k * r;
        for (int i = lane; i < r; i += 32) {
          const double2 x = vj[i], y = cmul(vk[i], ph);
          vj[i] = c2(cs * x.x - sn * y.x, cs * x.y - sn * y.y);
          vk[i] = c2(sn * x.x + cs * y.x, sn * x.y + cs * y.y);
        }
        if (lane == 0) atomicAdd(&s_rot, 1);
      }
      __syncthreads();
    }
    const int rot = s_rot;
    __syncthreads();
    if (rot == 0) break;
  }
  // singular values, their order, the outputs
  for (int j = warp; j < r; j += NWARP) {
    const double2* wj = W + (long)j * p;
    double acc = 0.0;
    for (int i = lane; i < p; i += 32) acc = fma(wj[i].x, wj[i].x, fma(wj[i].y, wj[i].y, acc));
    acc = warp_sum(acc);
    if (lane == 0) sig[j] = sqrt(acc);
  }
  __syncthreads();
  for (int j = tid; j < r; j += ST) {
    const double sj = sig[j];
    int c = 0;
    for (int i = 0; i < r; ++i) c += (sig[i] > sj || (sig[i] == sj && i < j)) ? 1 : 0;
    pos[j] = c;
    s[c] = sj;
  }
  __syncthreads();
  if (!wide) {
    // U[i][pos j] = w_j[i] / s_j (i < m), Vh[pos j][c] = conj(V[c][j]) (c < n)
    for (long e = tid; e < (long)r * p; e += ST) {
      const int j = (int)(e / p), i = (int)(e % p);
      const double sj = sig[j];
      const double inv = sj > 0.0 ? 1.0 / sj : 0.0;
      const double2 x = W[e];
      u[(long)i * ldu + pos[j]] = c2(x.x * inv, x.y * inv);
    }
    for (long e = tid; e < (long)r * r; e += ST) {
      const int j = (int)(e / r), c = (int)(e % r);
      vh[(long)pos[j] * ldvh + c] = cconj(V[e]);
    }
  } else {
    // A^H = W-side U_w diag(s) V^H: U[i][pos j] = V[i][j] (i < m), Vh[pos j][c] = conj(w_j[c]) / s_j
    for (long e = tid; e < (long)r * r; e += ST) {
      const int j = (int)(e / r), i = (int)(e % r);
      u[(long)i * ldu + pos[j]] = V[e];
    }
    for (long e = tid; e < (long)r * p; e += ST) {
      const int j = (int)(e / p), c = (int)(e % p);
      const double sj = sig[j];
      const double inv = sj > 0.0 ? 1.0 / sj : 0.0;
      const double2 x = W[e];
      vh[(long)pos[j] * ldvh + c] = c2(x.x * inv, -x.y * inv);
    }
  }
  if (tid == 0 && sweeps_out != nullptr) *sweeps_out = sweep + (sweep == MAX_SWEEPS ? 1 : 0);
}

// a[i][j] *= s[j] (side 0: columns) or s[i] (side 1: rows), row-major with ld
__global__ void diag_scale_kernel(double2* __restrict__ a, long rows, long cols, long ld,
                                  const double* __restrict__ s, int side) {
  const long total = rows * cols;
  for (long e = blockIdx.x * (long)blockDim.x + threadIdx.x; e < total;
       e += (long)gridDim.x * blockDim.x) {
    const long i = e / cols, j = e % cols;
    const double f = s[side == 0 ? j : i];
    double2* x = a + i * ld + j;
    *x = c2(x->x * f, x->y * f);
  }
}

inline size_t al(size_t b) { return (b + 255) & ~size_t(255); }

}  // namespace

size_t svd_workspace_bytes(int m, int n) {
  const long p = std::max(m, n), r = std::min(m, n);
  return al((size_t)p * r * sizeof(double2)) + al((size_t)r * r * sizeof(double2)) +
         al((size_t)r * sizeof(double)) + al((size_t)r * sizeof(int));
}

ptn_status svd(const double2* a, int m, int n, long lda, double2* u, long ldu, double* s,
               double2* vh, long ldvh, int* sweeps, void* ws, size_t ws_bytes, cudaStream_t st) {
  PTN_CHECK_ARG(m > 0 && n > 0, "svd: empty matrix (%d x %d)", m, n);
  PTN_CHECK_ARG(lda >= n && ldu >= std::min(m, n) && ldvh >= n, "svd: bad leading dimensions");
  PTN_CHECK_ARG(ws_bytes >= svd_workspace_bytes(m, n), "svd: workspace too small");
  const long p = std::max(m, n), r = std::min(m, n);
  char* c = static_cast<char*>(ws);
  double2* W = reinterpret_cast<double2*>(c);
  c += al((size_t)p * r * sizeof(double2));
  double2* V = reinterpret_cast<double2*>(c);
  c += al((size_t)r * r * sizeof(double2));
  double* sig = reinterpret_cast<double*>(c);
  c += al((size_t)r * sizeof(double));
  int* pos = reinterpret_cast<int*>(c);
  svd_jacobi_kernel<<<1, ST, 0, st>>>(a, m, n, lda, W, V, sig, pos, u, ldu, s, vh, ldvh, sweeps);
  PTN_LAUNCH_CHECK();
  note_launches(1);
  return PTN_OK;
}

}  // namespace ptn

extern "C" {

size_t ptn_svd_workspace_bytes(int m, int n) { return ptn::svd_workspace_bytes(m, n); }

ptn_status ptn_svd(const ptn_c128* a, int m, int n, long lda, ptn_c128* u, long ldu, double* s,
                   ptn_c128* vh, long ldvh, int* sweeps, void* ws, size_t ws_bytes,
                   void* stream) {
  return ptn::svd(reinterpret_cast<const double2*>(a), m, n, lda, reinterpret_cast<double2*>(u),
                  ldu, s, reinterpret_cast<double2*>(vh), ldvh, sweeps, ws, ws_bytes,
                  ptn::as_stream(stream));
}

ptn_status ptn_diag_scale(ptn_c128* a, long rows, long cols, long ld, const double* s, int side,
                          void* stream) {
  PTN_CHECK_ARG(rows >= 0 && cols >= 0 && ld >= cols && (side == 0 || side == 1),
                "diag_scale: bad arguments");
  if (rows == 0 || cols == 0) return PTN_OK;
  cudaStream_t st = ptn::as_stream(stream);
  const long total = rows * cols;
  const int blocks = (int)std::max(1L, std::min((total + 255) / 256, 8L * ptn::num_sms()));
  ptn::diag_scale_kernel<<<blocks, 256, 0, st>>>(reinterpret_cast<double2*>(a), rows, cols, ld,
                                                 s, side);
  PTN_LAUNCH_CHECK();
  ptn::note_launches(1);
  return PTN_OK;
}

}  // extern "C"
