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
//   panel kernel  : a cluster of up to 16 CTAs factors the panel column by
//                   column -- each CTA owns a slice of the rows, the column norm
//                   and the reflector dot products are reduced across the
//                   cluster through distributed shared memory (two cluster
//                   barriers per column) -- and builds the NB x NB triangular
//                   factor T with H_1..H_nb = I - V T V^H;
//   block update  : A_trail -= V (T^H (V^H A_trail)), as two grid-wide passes
//                   (partial V^H A per 64-row tile, then reduce + apply);
// then Q = H_1 ... H_k [I; 0] is formed backwards with the same block update
// (using T instead of T^H).
#include "ptn_common.cuh"
#include <cooperative_groups.h>
#include <algorithm>
#include <mutex>

namespace cg = cooperative_groups;

namespace ptn {

void note_launches(int n);

namespace {

constexpr int NB = 16;     // panel width
constexpr int PT = 512;    // panel kernel threads

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

// Cluster version of the panel factorisation: CTA `rank` of the cluster owns rows
// [j0 + rank * chunk, j0 + (rank + 1) * chunk). All reductions sum the per-CTA
// partials in rank order, so every CTA derives identical reflectors.
constexpr int CPT = 256;   // threads per cluster CTA

__global__ void __launch_bounds__(CPT) qr_panel_cluster_kernel(double2* __restrict__ a, long lda,
                                                               int m, int j0, int jb,
                                                               double2* __restrict__ Tout,
                                                               double2* __restrict__ V, long ldv) {
  cg::cluster_group cluster = cg::this_cluster();
  const int rank = (int)cluster.block_rank();
  const int cs = (int)cluster.num_blocks();
  const int tid = threadIdx.x;
  __shared__ double sh[33];
  __shared__ double2 red[CPT / 32][NB];
  __shared__ double s_nrm;
  __shared__ double2 s_alpha;
  __shared__ double2 s_w[NB];       // this CTA's partial vector (read remotely)
  __shared__ double2 gath[16][NB];  // all CTAs' partial vectors (cluster size <= 16)
  __shared__ double2 wv[NB];        // cluster-reduced vector
  __shared__ double2 taus[NB];
  __shared__ double2 sT[NB][NB];
  __shared__ double2 s_scal;
  __shared__ double s_beta;
  __shared__ int s_apply;

  const int mp = m - j0;
  const int chunk = (mp + cs - 1) / cs;
  const int rb = j0 + rank * chunk;
  const int re = min(m, rb + chunk);

  for (int jj = 0; jj < jb; ++jj) {
    const int col = j0 + jj;
    const int owner = jj / chunk;            // CTA holding row col
    double acc = 0.0;
    for (int i = max(rb, col + 1) + tid; i < re; i += CPT) {
      const double2 v = a[(long)i * lda + col];
      acc = fma(v.x, v.x, acc);
      acc = fma(v.y, v.y, acc);
    }
    acc = block_sum(acc, sh);
    if (tid == 0) {
      s_nrm = acc;
      if (rank == owner) s_alpha = a[(long)col * lda + col];
    }
    cluster.sync();
    if (tid < 32) {
      // one remote load per lane, then a fixed-order tree: identical in every CTA
      double v = (tid < cs) ? *cluster.map_shared_rank(&s_nrm, tid) : 0.0;
      const double2 alpha_l = (tid == 0) ? *cluster.map_shared_rank(&s_alpha, owner) : c2(0.0, 0.0);
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
      const double xn2 = v;
      const double2 alpha = alpha_l;
      if (tid == 0) {
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
    }
    __syncthreads();
    const int apply = s_apply;
    if (apply) {
      const double2 sc = s_scal;
      for (int i = max(rb, col + 1) + tid; i < re; i += CPT) {
        double2* p = a + (long)i * lda + col;
        *p = cmul(*p, sc);
      }
      if (tid == 0 && rank == owner) a[(long)col * lda + col] = c2(s_beta, 0.0);
    }
    __syncthreads();
    const int nrem = j0 + jb - col - 1;
    // every CTA takes part in the barrier below, also when there is nothing to apply
    double2 part[NB];
#pragma unroll
    for (int c = 0; c < NB; ++c) part[c] = c2(0.0, 0.0);
    if (apply && nrem > 0) {
      for (int i = max(rb, col) + tid; i < re; i += CPT) {
        const double2 v = (i == col) ? c2(1.0, 0.0) : a[(long)i * lda + col];
        const double2 vc = cconj(v);
        const double2* row = a + (long)i * lda + col + 1;
#pragma unroll
        for (int c = 0; c < NB; ++c)
          if (c < nrem) part[c] = cfma(vc, row[c], part[c]);
      }
    }
    block_reduce_vec(part, NB, red, s_w);
    cluster.sync();
    // gather all CTAs' partial vectors with one remote load per thread, then sum in rank order
    if (tid < cs * NB) gath[tid / NB][tid % NB] = cluster.map_shared_rank(s_w, tid / NB)[tid % NB];
    __syncthreads();
    if (tid < NB) {
      double2 sacc = c2(0.0, 0.0);
      for (int r = 0; r < cs; ++r) sacc = cadd(sacc, gath[r][tid]);
      wv[tid] = sacc;
    }
    __syncthreads();
    if (apply && nrem > 0) {
      const double2 ctau = cconj(taus[jj]);
      for (int i = max(rb, col) + tid; i < re; i += CPT) {
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

  // explicit V for the panel columns on this CTA's rows
  for (int i = rb + tid; i < re; i += CPT) {
    for (int c = 0; c < jb; ++c) {
      const int col = j0 + c;
      V[(long)i * ldv + col] = (i < col) ? c2(0.0, 0.0)
                               : (i == col) ? c2(1.0, 0.0) : a[(long)i * lda + col];
    }
  }
  // partial Gram G[p][c] = v_p^H v_c (p < c) over this CTA's rows -> s_G
  __shared__ double2 s_G[NB][NB];
  if (tid < NB * NB) s_G[tid / NB][tid % NB] = c2(0.0, 0.0);
  __syncthreads();
  for (int c = 1; c < jb; ++c) {
    double2 pp[NB];
#pragma unroll
    for (int p = 0; p < NB; ++p) pp[p] = c2(0.0, 0.0);
    for (int i = max(rb, j0 + c) + tid; i < re; i += CPT) {
      const double2 vc = (i == j0 + c) ? c2(1.0, 0.0) : a[(long)i * lda + j0 + c];
#pragma unroll
      for (int p = 0; p < NB; ++p)
        if (p < c) {
          const double2 vp = (i == j0 + p) ? c2(1.0, 0.0) : a[(long)i * lda + j0 + p];
          pp[p] = cfma(cconj(vp), vc, pp[p]);
        }
    }
    block_reduce_vec(pp, c, red, wv);
    if (tid < c) s_G[tid][c] = wv[tid];
    __syncthreads();
  }
  cluster.sync();
  if (rank == 0) {
    // sum the Gram partials of all CTAs (rank order), then T as in zlarft
    if (tid < NB * NB) {
      const int p = tid / NB, c = tid % NB;
      double2 g = c2(0.0, 0.0);
      for (int r = 0; r < cs; ++r) g = cadd(g, cluster.map_shared_rank(&s_G[0][0], r)[p * NB + c]);
      sT[p][c] = g;   // the summed Gram (upper part)
    }
    __syncthreads();
    // T column by column (zlarft); column c needs only columns < c of T
    if (tid < NB * NB) s_G[tid / NB][tid % NB] = c2(0.0, 0.0);   // now holds T
    __syncthreads();
    for (int c = 0; c < jb; ++c) {
      if (tid < c) {
        const int p = tid;
        double2 acc2 = c2(0.0, 0.0);
        for (int q = p; q < c; ++q) acc2 = cadd(acc2, cmul(s_G[p][q], sT[q][c]));
        s_G[p][c] = cmul(c2(-taus[c].x, -taus[c].y), acc2);
      }
      if (tid == 0) s_G[c][c] = taus[c];
      __syncthreads();
    }
    if (tid < NB * NB) Tout[tid] = s_G[tid / NB][tid % NB];
  }
  cluster.sync();   // no CTA leaves while its shared memory may still be read
}

// Panel factorisation for GB300's FP64 budget: a cluster of CTAs of 1..4 warps,
// one panel row per thread. Per column: norm and dot products are reduced inside
// each warp by reduce-scatter (lane l ends up with the warp sum of one value),
// across the warps through shared memory and across the cluster through
// distributed shared memory, with two cluster barriers. The reflector scalars are
// computed by every warp from the gathered partials (no broadcast). The dot
// products of the new reflector with the previous ones (for T) ride along in the
// same reduction.
constexpr int QW = 4;   // warps per CTA

// 16 complex values per lane -> lane l holds the warp sum of value qv(l)
__device__ __forceinline__ double2 reduce_scatter16(double2 (&v)[NB], int lane) {
#pragma unroll
  for (int lvl = 0, half = 8, mask = 16; lvl < 4; ++lvl, half >>= 1, mask >>= 1) {
    const bool up = (lane & mask) != 0;
#pragma unroll
    for (int i = 0; i < 8; ++i) {
      if (i < half) {
        const double2 send = up ? v[i] : v[i + half];
        const double2 keep = up ? v[i + half] : v[i];
        const double2 got = c2(__shfl_xor_sync(0xffffffffu, send.x, mask),
                               __shfl_xor_sync(0xffffffffu, send.y, mask));
        v[i] = cadd(keep, got);
      }
    }
  }
  const double2 r = v[0];
  return cadd(r, c2(__shfl_xor_sync(0xffffffffu, r.x, 1), __shfl_xor_sync(0xffffffffu, r.y, 1)));
}

// value index held by lane after reduce_scatter16
__device__ __forceinline__ int rs_index(int lane) {
  return ((lane >> 4) & 1) * 8 + ((lane >> 3) & 1) * 4 + ((lane >> 2) & 1) * 2 + ((lane >> 1) & 1);
}

// Panel on a cluster, one row per thread, 1..QW warps per CTA (as many as the row
// chunk needs: idle warps would spend the scarce FP64 issue slots on zeros). The
// CTA's rows live in shared memory column-major (xs[c][thread]: conflict-free)
// and the column loop stays rolled, so one small loop body serves every column
// (a fully unrolled body stalled on instruction fetch). Per column: the norm
// (one cluster barrier, partials read through DSMEM), the reflector, one
// reduce-scatter of w_c = v^H a_c (c > jj) and of the Gram column g_p = v_p^H v
// (p < jj) (second barrier), the rank-1 update of the remaining panel columns.
__global__ void __launch_bounds__(QW * 32) qr_panel4_kernel(double2* __restrict__ a, long lda, int m,
                                                            int j0, int jb,
                                                            double2* __restrict__ Tout,
                                                            double2* __restrict__ V, long ldv) {
  cg::cluster_group cluster = cg::this_cluster();
  const int rank = (int)cluster.block_rank();
  const int cs = (int)cluster.num_blocks();
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int nw = (int)(blockDim.x >> 5);
  __shared__ double2 xs[NB][QW * 32];     // this CTA's panel rows, column-major
  __shared__ double s_wn[QW];             // per-warp norm partials
  __shared__ double2 s_wv[QW][NB];        // per-warp vector partials
  __shared__ double s_nrm;                // CTA partial norm (read remotely)
  __shared__ double2 s_alpha;
  __shared__ double2 s_vec[NB];           // CTA partial vectors (read remotely)
  __shared__ double2 s_tau[NB];
  __shared__ double2 s_G[NB][NB];         // Gram entries v_p^H v_c, p < c (rank 0)

  const int mp = m - j0;
  const int chunk = (mp + cs - 1) / cs;
  const int rb = j0 + rank * chunk;
  const int re = min(m, rb + chunk);
  const int i = rb + tid;                 // this thread's row
  const bool mine = i < re;

#pragma unroll
  for (int c = 0; c < NB; ++c) xs[c][tid] = (mine && c < jb) ? a[(long)i * lda + j0 + c] : c2(0.0, 0.0);
  for (int e = tid; e < NB * NB; e += blockDim.x) s_G[e / NB][e % NB] = c2(0.0, 0.0);

#pragma unroll 1
  for (int jj = 0; jj < jb; ++jj) {
    const int col = j0 + jj;
    const int owner = jj / chunk;
    // ---- norm of the part below the diagonal
    const double2 xj = xs[jj][tid];
    double acc = (mine && i > col) ? fma(xj.x, xj.x, xj.y * xj.y) : 0.0;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    if (lane == 0) s_wn[warp] = acc;
    if (i == col) s_alpha = xj;
    __syncthreads();
    if (tid == 0) {
      const double h0 = s_wn[0] + ((nw > 1) ? s_wn[1] : 0.0);
      const double h1 = (nw > 2) ? s_wn[2] + ((nw > 3) ? s_wn[3] : 0.0) : 0.0;
      s_nrm = h0 + h1;
    }
    cluster.sync();
    double v = (lane < cs) ? *cluster.map_shared_rank(&s_nrm, lane) : 0.0;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    const double xn2 = v;
    const double2 alpha = *cluster.map_shared_rank(&s_alpha, owner);
    double2 tau = c2(0.0, 0.0), scal = c2(0.0, 0.0);
    double beta = 0.0;
    const bool apply = !(xn2 == 0.0 && alpha.y == 0.0);
    if (apply) {
      beta = -copysign(sqrt(alpha.x * alpha.x + alpha.y * alpha.y + xn2), alpha.x);
      const double ib = 1.0 / beta;
      tau = c2((beta - alpha.x) * ib, -alpha.y * ib);
      scal = crecip(c2(alpha.x - beta, alpha.y));
    }
    if (tid == 0) s_tau[jj] = tau;
    double2 xjn = xj;
    if (apply && mine && i > col) xjn = cmul(xj, scal);
    if (apply && i == col) xjn = c2(beta, 0.0);
    xs[jj][tid] = xjn;
    // ---- one reduction: w_c = v^H a_c (c > jj) and g_p = v_p^H v (p < jj)
    const double2 vcur = (mine && i >= col) ? ((i == col) ? c2(1.0, 0.0) : xjn) : c2(0.0, 0.0);
    double2 q[NB];
#pragma unroll
    for (int c = 0; c < NB; ++c) {
      const double2 xc = xs[c][tid];
      if (c > jj) {
        q[c] = cmul(cconj(vcur), xc);
      } else if (c < jj) {
        const double2 vp = (mine && i >= j0 + c) ? ((i == j0 + c) ? c2(1.0, 0.0) : xc) : c2(0.0, 0.0);
        q[c] = cmul(cconj(vp), vcur);
      } else {
        q[c] = c2(0.0, 0.0);
      }
    }
    const double2 ws = reduce_scatter16(q, lane);
    const int qi = rs_index(lane);
    if ((lane & 1) == 0) s_wv[warp][qi] = ws;
    __syncthreads();
    if (tid < NB) {
      const double2 h0 = (nw > 1) ? cadd(s_wv[0][tid], s_wv[1][tid]) : s_wv[0][tid];
      const double2 h1 = (nw > 2) ? ((nw > 3) ? cadd(s_wv[2][tid], s_wv[3][tid]) : s_wv[2][tid])
                                  : c2(0.0, 0.0);
      s_vec[tid] = (nw > 2) ? cadd(h0, h1) : h0;
    }
    cluster.sync();
    // ---- gather: lane c (< NB) of every warp sums rank by rank (tree, same order everywhere)
    double2 tot = c2(0.0, 0.0);
    if (lane < NB) {
      double2 vals[16];
#pragma unroll
      for (int r = 0; r < 16; ++r)
        vals[r] = (r < cs) ? cluster.map_shared_rank(s_vec, r)[lane] : c2(0.0, 0.0);
#pragma unroll
      for (int h = 8; h > 0; h >>= 1)
#pragma unroll
        for (int r = 0; r < h; ++r) vals[r] = cadd(vals[r], vals[r + h]);
      tot = vals[0];
    }
    if (rank == 0 && warp == 0 && lane < jj) s_G[lane][jj] = tot;
    // ---- rank-1 update of this thread's row: x_c -= v conj(tau) w_c, with the
    // scalar conj(tau) w_c formed once per column (lane c) and broadcast
    const double2 sc = (lane < NB) ? cmul(cconj(tau), tot) : c2(0.0, 0.0);
#pragma unroll
    for (int c = 0; c < NB; ++c) {
      const double2 s = c2(__shfl_sync(0xffffffffu, sc.x, c), __shfl_sync(0xffffffffu, sc.y, c));
      if (c > jj && apply && mine && i >= col) xs[c][tid] = csub(xs[c][tid], cmul(vcur, s));
    }
  }

  // ---- write the panel back and the explicit V
  if (mine) {
#pragma unroll
    for (int c = 0; c < NB; ++c) {
      if (c < jb) {
        const int col = j0 + c;
        const double2 x = xs[c][tid];
        a[(long)i * lda + col] = x;
        V[(long)i * ldv + col] = (i < col) ? c2(0.0, 0.0) : (i == col) ? c2(1.0, 0.0) : x;
      }
    }
  }
  // ---- T (zlarft) on rank 0 from the Gram entries
  if (rank == 0) {
    __syncthreads();
    if (warp == 0) {
      double2 T[NB];   // lane p holds row p of T
#pragma unroll
      for (int c = 0; c < NB; ++c) T[c] = c2(0.0, 0.0);
#pragma unroll
      for (int c = 0; c < NB; ++c) {
        if (c < jb) {
          double2 acc2 = c2(0.0, 0.0);
#pragma unroll
          for (int qq = 0; qq < NB; ++qq)
            if (qq < c && lane <= qq) acc2 = cfma(T[qq], s_G[qq][c], acc2);
          const double2 tc = s_tau[c];
          if (lane < c) T[c] = cmul(c2(-tc.x, -tc.y), acc2);
          if (lane == c) T[c] = tc;
        }
      }
      if (lane < NB)
#pragma unroll
        for (int c = 0; c < NB; ++c) Tout[lane * NB + c] = T[c];
    }
  }
  cluster.sync();   // no CTA leaves while its shared memory may still be read
}

// Panel for GB300's FP64 budget, second form: the same row-per-thread layout and
// the same two cluster barriers per column as qr_panel4_kernel, with fewer FP64
// instructions per column on each SM (the FP64 pipe is shared by all of the SM's
// warps, so work duplicated in every warp is paid once per warp):
//  - the norm partials of all warps of all CTAs are read directly through DSMEM by
//    warp 0, which alone forms beta, tau and the scaling (both reciprocals in one
//    division sequence, on two lanes) and hands them over in shared memory;
//  - warp 0 alone gathers the reduced vector (all 32 lanes: 16 values x two halves
//    of the ranks), forms the update scalars conj(tau) w_c (zero for c <= jj) and
//    keeps the Gram entries;
//  - the rank-1 update loops only over the columns right of the pivot, reading the
//    rows from shared memory.
__global__ void __launch_bounds__(QW * 32) qr_panel5_kernel(double2* __restrict__ a, long lda, int m,
                                                            int j0, int jb,
                                                            double2* __restrict__ Tout,
                                                            double2* __restrict__ V, long ldv) {
  cg::cluster_group cluster = cg::this_cluster();
  const int rank = (int)cluster.block_rank();
  const int cs = (int)cluster.num_blocks();
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int nw = (int)(blockDim.x >> 5);
  __shared__ double2 xs[NB][QW * 32];     // this CTA's panel rows, column-major
  __shared__ double s_wn[QW];             // per-warp norm partials (read remotely)
  __shared__ double2 s_wv[QW][NB];        // per-warp vector partials
  __shared__ double2 s_alpha;
  __shared__ double2 s_vec[NB];           // CTA partial vectors (read remotely)
  __shared__ double2 s_tau[NB];
  __shared__ double2 s_scal;              // 1 / (alpha - beta)
  __shared__ double s_beta;
  __shared__ int s_apply;
  __shared__ double2 s_upd[NB];           // conj(tau) w_c for c > jj, else 0
  __shared__ double2 s_G[NB][NB];         // Gram entries v_p^H v_c, p < c (rank 0)

  const int mp = m - j0;
  const int chunk = (mp + cs - 1) / cs;
  const int rb = j0 + rank * chunk;
  const int re = min(m, rb + chunk);
  const int i = rb + tid;                 // this thread's row
  const bool mine = i < re;

#pragma unroll
  for (int c = 0; c < NB; ++c) xs[c][tid] = (mine && c < jb) ? a[(long)i * lda + j0 + c] : c2(0.0, 0.0);
  for (int e = tid; e < NB * NB; e += blockDim.x) s_G[e / NB][e % NB] = c2(0.0, 0.0);

#pragma unroll 1
  for (int jj = 0; jj < jb; ++jj) {
    const int col = j0 + jj;
    const int owner = jj / chunk;
    // ---- norm partials of the part below the diagonal, one per warp
    const double2 xj = xs[jj][tid];
    double acc = (mine && i > col) ? fma(xj.x, xj.x, xj.y * xj.y) : 0.0;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    if (lane == 0) s_wn[warp] = acc;
    if (i == col) s_alpha = xj;
    cluster.sync();
    // ---- warp 0: the reflector scalars from every warp's partial (fixed order)
    if (warp == 0) {
      const int np = cs * nw;              // <= 64
      double v = 0.0;
      if (lane < np) v = cluster.map_shared_rank(s_wn, lane / nw)[lane % nw];
      if (lane + 32 < np) v += cluster.map_shared_rank(s_wn, (lane + 32) / nw)[(lane + 32) % nw];
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
      const double xn2 = v;
      const double2 alpha = *cluster.map_shared_rank(&s_alpha, owner);
      const bool apply = !(xn2 == 0.0 && alpha.y == 0.0);
      double beta = 0.0, dx = 0.0, d2 = 1.0;
      if (apply) {
        beta = -copysign(sqrt(alpha.x * alpha.x + alpha.y * alpha.y + xn2), alpha.x);
        dx = alpha.x - beta;
        d2 = dx * dx + alpha.y * alpha.y;   // |alpha - beta|^2 > 0
      }
      // the two reciprocals in one division sequence: lane 0 1 / beta, lane 1 1 / d2
      const double rec = 1.0 / ((lane == 0) ? (apply ? beta : 1.0) : d2);
      const double ib = __shfl_sync(0xffffffffu, rec, 0);
      const double id2 = __shfl_sync(0xffffffffu, rec, 1);
      if (lane == 0) {
        double2 tau = c2(0.0, 0.0), scal = c2(0.0, 0.0);
        if (apply) {
          tau = c2((beta - alpha.x) * ib, -alpha.y * ib);
          scal = c2(dx * id2, -alpha.y * id2);
        }
        s_tau[jj] = tau;
        s_scal = scal;
        s_beta = beta;
        s_apply = apply ? 1 : 0;
      }
    }
    __syncthreads();
    const bool apply = s_apply != 0;
    const double2 scal = s_scal;
    double2 xjn = xj;
    if (apply && mine && i > col) xjn = cmul(xj, scal);
    if (apply && i == col) xjn = c2(s_beta, 0.0);
    xs[jj][tid] = xjn;
    // ---- one reduction: w_c = v^H a_c (c > jj) and g_p = v_p^H v (p < jj)
    const double2 vcur = (mine && i >= col) ? ((i == col) ? c2(1.0, 0.0) : xjn) : c2(0.0, 0.0);
    double2 q[NB];
#pragma unroll
    for (int c = 0; c < NB; ++c) {
      const double2 xc = xs[c][tid];
      if (c > jj) {
        q[c] = cmul(cconj(vcur), xc);
      } else if (c < jj) {
        const double2 vp = (mine && i >= j0 + c) ? ((i == j0 + c) ? c2(1.0, 0.0) : xc) : c2(0.0, 0.0);
        q[c] = cmul(cconj(vp), vcur);
      } else {
        q[c] = c2(0.0, 0.0);
      }
    }
    const double2 ws = reduce_scatter16(q, lane);
    const int qi = rs_index(lane);
    if ((lane & 1) == 0) s_wv[warp][qi] = ws;
    __syncthreads();
    if (tid < NB) {
      const double2 h0 = (nw > 1) ? cadd(s_wv[0][tid], s_wv[1][tid]) : s_wv[0][tid];
      const double2 h1 = (nw > 2) ? ((nw > 3) ? cadd(s_wv[2][tid], s_wv[3][tid]) : s_wv[2][tid])
                                  : c2(0.0, 0.0);
      s_vec[tid] = (nw > 2) ? cadd(h0, h1) : h0;
    }
    cluster.sync();
    // ---- warp 0: lane (c, half) sums the ranks of its half, then the two halves
    if (warp == 0) {
      const int c = lane & 15, h = lane >> 4;
      double2 vals[8];
#pragma unroll
      for (int r = 0; r < 8; ++r) {
        const int rr = h * 8 + r;
        vals[r] = (rr < cs) ? cluster.map_shared_rank(s_vec, rr)[c] : c2(0.0, 0.0);
      }
#pragma unroll
      for (int hh = 4; hh > 0; hh >>= 1)
#pragma unroll
        for (int r = 0; r < hh; ++r) vals[r] = cadd(vals[r], vals[r + hh]);
      double2 tot = vals[0];
      tot = cadd(tot, c2(__shfl_xor_sync(0xffffffffu, tot.x, 16),
                         __shfl_xor_sync(0xffffffffu, tot.y, 16)));
      if (h == 0) {
        if (rank == 0 && c < jj) s_G[c][jj] = tot;
        s_upd[c] = (apply && c > jj) ? cmul(cconj(s_tau[jj]), tot) : c2(0.0, 0.0);
      }
    }
    __syncthreads();
    // ---- rank-1 update of this thread's row on the columns right of the pivot:
    // x_c -= v conj(tau) w_c (v = 0 on the rows above the pivot and past the end)
#pragma unroll 1
    for (int c = jj + 1; c < jb; ++c) {
      const double2 s = s_upd[c];
      double2 x = xs[c][tid];
      x.x = fma(-vcur.x, s.x, x.x);
      x.x = fma(vcur.y, s.y, x.x);
      x.y = fma(-vcur.x, s.y, x.y);
      x.y = fma(-vcur.y, s.x, x.y);
      xs[c][tid] = x;
    }
  }

  // ---- write the panel back and the explicit V
  if (mine) {
#pragma unroll
    for (int c = 0; c < NB; ++c) {
      if (c < jb) {
        const int col = j0 + c;
        const double2 x = xs[c][tid];
        a[(long)i * lda + col] = x;
        V[(long)i * ldv + col] = (i < col) ? c2(0.0, 0.0) : (i == col) ? c2(1.0, 0.0) : x;
      }
    }
  }
  // ---- T (zlarft) on rank 0 from the Gram entries
  if (rank == 0) {
    __syncthreads();
    if (warp == 0) {
      double2 T[NB];   // lane p holds row p of T
#pragma unroll
      for (int c = 0; c < NB; ++c) T[c] = c2(0.0, 0.0);
#pragma unroll
      for (int c = 0; c < NB; ++c) {
        if (c < jb) {
          double2 acc2 = c2(0.0, 0.0);
#pragma unroll
          for (int qq = 0; qq < NB; ++qq)
            if (qq < c && lane <= qq) acc2 = cfma(T[qq], s_G[qq][c], acc2);
          const double2 tc = s_tau[c];
          if (lane < c) T[c] = cmul(c2(-tc.x, -tc.y), acc2);
          if (lane == c) T[c] = tc;
        }
      }
      if (lane < NB)
#pragma unroll
        for (int c = 0; c < NB; ++c) Tout[lane * NB + c] = T[c];
    }
  }
  cluster.sync();   // no CTA leaves while its shared memory may still be read
}

// 8 complex values per lane -> lane l holds the warp sum of value rs8_index(l)
__device__ __forceinline__ double2 reduce_scatter8(double2 (&v)[8], int lane) {
#pragma unroll
  for (int lvl = 0, half = 4, mask = 16; lvl < 3; ++lvl, half >>= 1, mask >>= 1) {
    const bool up = (lane & mask) != 0;
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      if (i < half) {
        const double2 send = up ? v[i] : v[i + half];
        const double2 keep = up ? v[i + half] : v[i];
        const double2 got = c2(__shfl_xor_sync(0xffffffffu, send.x, mask),
                               __shfl_xor_sync(0xffffffffu, send.y, mask));
        v[i] = cadd(keep, got);
      }
    }
  }
  double2 r = v[0];
  r = cadd(r, c2(__shfl_xor_sync(0xffffffffu, r.x, 2), __shfl_xor_sync(0xffffffffu, r.y, 2)));
  return cadd(r, c2(__shfl_xor_sync(0xffffffffu, r.x, 1), __shfl_xor_sync(0xffffffffu, r.y, 1)));
}

__device__ __forceinline__ int rs8_index(int lane) {
  return ((lane >> 4) & 1) * 4 + ((lane >> 3) & 1) * 2 + ((lane >> 2) & 1);
}

// Panel, third form: a 32-row group of the CTA is shared by two warps, one per
// column set (even / odd columns), so a CTA of 64 rows runs four warps, one on
// each SM sub-partition, and each warp issues the FP64 work of 8 columns per pivot
// (dot products, Gram entries, reduction, rank-1 update); interleaving the sets
// balances the columns right of the pivot between them. Two cluster barriers per
// column as before; the reflector scalars come from warp 0, the gathered vector
// from the two warps of row group 0 (one per set).
constexpr int P6W = 8;   // up to 4 row groups x 2 column sets
__global__ void __launch_bounds__(P6W * 32) qr_panel6_kernel(double2* __restrict__ a, long lda, int m,
                                                             int j0, int jb,
                                                             double2* __restrict__ Tout,
                                                             double2* __restrict__ V, long ldv) {
  cg::cluster_group cluster = cg::this_cluster();
  const int rank = (int)cluster.block_rank();
  const int cs = (int)cluster.num_blocks();
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int ng = (int)(blockDim.x >> 6);  // row groups
  const int ch = warp & 1, rg = warp >> 1;
  __shared__ double2 xs[NB][P6W / 2 * 32];  // this CTA's panel rows, column-major
  __shared__ double s_wn[P6W / 2];          // norm partials per row group (read remotely)
  __shared__ double2 s_wv[P6W / 2][NB];     // vector partials per row group
  __shared__ double2 s_alpha;
  __shared__ double2 s_vec[NB];             // CTA partial vectors (read remotely)
  __shared__ double2 s_tau[NB];
  __shared__ double2 s_scal;
  __shared__ double s_beta;
  __shared__ int s_apply;
  __shared__ double2 s_upd[NB];             // conj(tau) w_c for c > jj, else 0
  __shared__ double2 s_G[NB][NB];           // Gram entries v_p^H v_c, p < c (rank 0)

  const int mp = m - j0;
  const int chunk = (mp + cs - 1) / cs;
  const int rb = j0 + rank * chunk;
  const int re = min(m, rb + chunk);
  const int lr = rg * 32 + lane;            // this thread's row within the CTA
  const int i = rb + lr;
  const bool mine = i < re;

#pragma unroll
  for (int t = 0; t < NB / 2; ++t) {
    const int c = 2 * t + ch;
    xs[c][lr] = (mine && c < jb) ? a[(long)i * lda + j0 + c] : c2(0.0, 0.0);
  }
  for (int e = tid; e < NB * NB; e += blockDim.x) s_G[e / NB][e % NB] = c2(0.0, 0.0);

#pragma unroll 1
  for (int jj = 0; jj < jb; ++jj) {
    const int col = j0 + jj;
    const int owner = jj / chunk;
    const int oh = jj & 1;                  // column set holding the pivot
    // ---- norm partials below the diagonal (the pivot's set), one per row group
    if (ch == oh) {
      const double2 xj = xs[jj][lr];
      double acc = (mine && i > col) ? fma(xj.x, xj.x, xj.y * xj.y) : 0.0;
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
      if (lane == 0) s_wn[rg] = acc;
      if (i == col) s_alpha = xj;
    }
    cluster.sync();
    // ---- warp 0: the reflector scalars from every row group's partial (fixed order)
    if (warp == 0) {
      const int np = cs * ng;               // <= 64
      double v = 0.0;
      if (lane < np) v = cluster.map_shared_rank(s_wn, lane / ng)[lane % ng];
      if (lane + 32 < np) v += cluster.map_shared_rank(s_wn, (lane + 32) / ng)[(lane + 32) % ng];
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
      const double xn2 = v;
      const double2 alpha = *cluster.map_shared_rank(&s_alpha, owner);
      const bool apply = !(xn2 == 0.0 && alpha.y == 0.0);
      double beta = 0.0, dx = 0.0, d2 = 1.0;
      if (apply) {
        beta = -copysign(sqrt(alpha.x * alpha.x + alpha.y * alpha.y + xn2), alpha.x);
        dx = alpha.x - beta;
        d2 = dx * dx + alpha.y * alpha.y;
      }
      // the two reciprocals in one division sequence: lane 0 1 / beta, lane 1 1 / d2
      const double rec = 1.0 / ((lane == 0) ? (apply ? beta : 1.0) : d2);
      const double ib = __shfl_sync(0xffffffffu, rec, 0);
      const double id2 = __shfl_sync(0xffffffffu, rec, 1);
      if (lane == 0) {
        double2 tau = c2(0.0, 0.0), scal = c2(0.0, 0.0);
        if (apply) {
          tau = c2((beta - alpha.x) * ib, -alpha.y * ib);
          scal = c2(dx * id2, -alpha.y * id2);
        }
        s_tau[jj] = tau;
        s_scal = scal;
        s_beta = beta;
        s_apply = apply ? 1 : 0;
      }
    }
    __syncthreads();
    const bool apply = s_apply != 0;
    // the pivot column as updated by the previous pivot (visible after the barriers)
    const double2 xj = xs[jj][lr];
    double2 xjn = xj;
    if (apply && mine && i > col) xjn = cmul(xj, s_scal);
    if (apply && i == col) xjn = c2(s_beta, 0.0);
    // ---- one reduction: w_c = v^H a_c (c > jj) and g_p = v_p^H v (p < jj), own set
    const double2 vcur = (mine && i >= col) ? ((i == col) ? c2(1.0, 0.0) : xjn) : c2(0.0, 0.0);
    double2 q[NB / 2];
#pragma unroll
    for (int t = 0; t < NB / 2; ++t) {
      const int c = 2 * t + ch;
      const double2 xc = xs[c][lr];
      if (c > jj) {
        q[t] = cmul(cconj(vcur), xc);
      } else if (c < jj) {
        const double2 vp = (mine && i >= j0 + c) ? ((i == j0 + c) ? c2(1.0, 0.0) : xc) : c2(0.0, 0.0);
        q[t] = cmul(cconj(vp), vcur);
      } else {
        q[t] = c2(0.0, 0.0);
      }
    }
    const double2 ws = reduce_scatter8(q, lane);
    if ((lane & 3) == 0) s_wv[rg][2 * rs8_index(lane) + ch] = ws;
    __syncthreads();
    if (tid < NB) {
      double2 s = s_wv[0][tid];
      if (ng > 1) s = cadd(s, s_wv[1][tid]);
      if (ng > 2) s = cadd(s, (ng > 3) ? cadd(s_wv[2][tid], s_wv[3][tid]) : s_wv[2][tid]);
      s_vec[tid] = s;
    }
    cluster.sync();
    // ---- row group 0, one warp per set: lane (t, quarter) sums four ranks, then
    // the quarters (fixed order, identical in every CTA)
    if (rg == 0) {
      const int t = lane & 7, rq = lane >> 3;
      const int c = 2 * t + ch;
      double2 vals[4];
#pragma unroll
      for (int k = 0; k < 4; ++k) {
        const int rr = rq * 4 + k;
        vals[k] = (rr < cs) ? cluster.map_shared_rank(s_vec, rr)[c] : c2(0.0, 0.0);
      }
      double2 tot = cadd(cadd(vals[0], vals[1]), cadd(vals[2], vals[3]));
      tot = cadd(tot, c2(__shfl_xor_sync(0xffffffffu, tot.x, 8), __shfl_xor_sync(0xffffffffu, tot.y, 8)));
      tot = cadd(tot, c2(__shfl_xor_sync(0xffffffffu, tot.x, 16), __shfl_xor_sync(0xffffffffu, tot.y, 16)));
      if (rq == 0) {
        if (rank == 0 && c < jj) s_G[c][jj] = tot;
        s_upd[c] = (apply && c > jj) ? cmul(cconj(s_tau[jj]), tot) : c2(0.0, 0.0);
      }
    }
    __syncthreads();
    // ---- rank-1 update of this thread's row on its set's columns right of the pivot
#pragma unroll 1
    for (int t = (jj + 2 - ch) >> 1; 2 * t + ch < jb; ++t) {
      const int c = 2 * t + ch;
      const double2 s = s_upd[c];
      double2 x = xs[c][lr];
      x.x = fma(-vcur.x, s.x, x.x);
      x.x = fma(vcur.y, s.y, x.x);
      x.y = fma(-vcur.x, s.y, x.y);
      x.y = fma(-vcur.y, s.x, x.y);
      xs[c][lr] = x;
    }
    // the pivot column takes its reflector (every warp has read xj by now)
    if (ch == oh) xs[jj][lr] = xjn;
  }

  // ---- write the panel back and the explicit V
  if (mine) {
#pragma unroll
    for (int t = 0; t < NB / 2; ++t) {
      const int c = 2 * t + ch;
      if (c < jb) {
        const int col = j0 + c;
        const double2 x = xs[c][lr];
        a[(long)i * lda + col] = x;
        V[(long)i * ldv + col] = (i < col) ? c2(0.0, 0.0) : (i == col) ? c2(1.0, 0.0) : x;
      }
    }
  }
  // ---- T (zlarft) on rank 0 from the Gram entries
  if (rank == 0) {
    __syncthreads();
    if (warp == 0) {
      double2 T[NB];   // lane p holds row p of T
#pragma unroll
      for (int c = 0; c < NB; ++c) T[c] = c2(0.0, 0.0);
#pragma unroll
      for (int c = 0; c < NB; ++c) {
        if (c < jb) {
          double2 acc2 = c2(0.0, 0.0);
#pragma unroll
          for (int qq = 0; qq < NB; ++qq)
            if (qq < c && lane <= qq) acc2 = cfma(T[qq], s_G[qq][c], acc2);
          const double2 tc = s_tau[c];
          if (lane < c) T[c] = cmul(c2(-tc.x, -tc.y), acc2);
          if (lane == c) T[c] = tc;
        }
      }
      if (lane < NB)
#pragma unroll
        for (int c = 0; c < NB; ++c) Tout[lane * NB + c] = T[c];
    }
  }
  cluster.sync();   // no CTA leaves while its shared memory may still be read
}

__device__ __forceinline__ void cluster_arrive() {
  asm volatile("barrier.cluster.arrive.release;" ::: "memory");
}
__device__ __forceinline__ void cluster_wait() {
  asm volatile("barrier.cluster.wait.acquire;" ::: "memory");
}

// Panel, fourth form (default): the layout of qr_panel6_kernel (two warps per 32-row
// group, even / odd columns) with a shorter instruction path per column:
//  - one product per row and column, conj(v) x_c, for every column: on the rows
//    where a masked operand would differ, v is zero, so the dot products (c > jj)
//    and the conjugated Gram entries (c < jj) come out of the same select-free loop;
//  - the products go to shared memory (rows x 17 complex, conflict-free) and
//    thread (column, 8-row block) sums them: one pass instead of a shuffle
//    reduce-scatter with selects;
//  - after the gather, the next pivot column is updated first and its norm partial
//    published; the cluster barrier that guards it is split (arrive now, wait at the
//    next pivot), so the other updates run while the barrier completes.
// Dynamic shared memory: xs[NB][R] and the product buffer [R][17], R = 32 x row groups.
__global__ void __launch_bounds__(P6W * 32) qr_panel7_kernel(double2* __restrict__ a, long lda, int m,
                                                             int j0, int jb,
                                                             double2* __restrict__ Tout,
                                                             double2* __restrict__ V, long ldv) {
  cg::cluster_group cluster = cg::this_cluster();
  const int rank = (int)cluster.block_rank();
  const int cs = (int)cluster.num_blocks();
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int ng = (int)(blockDim.x >> 6);   // row groups
  const int nw = 2 * ng;
  const int R = 32 * ng;                   // rows held by this CTA
  const int ch = warp & 1, rg = warp >> 1;
  extern __shared__ double2 dyn[];
  double2* xs = dyn;                       // xs[c * R + row]
  double2* qs = dyn + NB * R;              // qs[row * 17 + c]
  __shared__ double s_wn[P6W / 2];
  __shared__ double2 s_wv[P6W][NB];        // per-warp column sums
  __shared__ double2 s_alpha;
  __shared__ double2 s_vec[NB];            // CTA column sums (read remotely)
  __shared__ double2 s_tau[NB];
  __shared__ double2 s_scal;
  __shared__ double s_beta;
  __shared__ int s_apply;
  __shared__ double2 s_upd[NB];
  __shared__ double2 s_G[NB][NB];

  const int mp = m - j0;
  const int chunk = (mp + cs - 1) / cs;
  const int rb = j0 + rank * chunk;
  const int re = min(m, rb + chunk);
  const int lr = rg * 32 + lane;
  const int i = rb + lr;
  const bool mine = i < re;

#pragma unroll
  for (int t = 0; t < NB / 2; ++t) {
    const int c = 2 * t + ch;
    xs[c * R + lr] = (mine && c < jb) ? a[(long)i * lda + j0 + c] : c2(0.0, 0.0);
  }
  for (int e = tid; e < NB * NB; e += blockDim.x) s_G[e / NB][e % NB] = c2(0.0, 0.0);

  // norm partial of pivot column p (its set's warps) and the pivot entry
  auto publish_norm = [&](int p) {
    if (ch == (p & 1)) {
      const double2 x = xs[p * R + lr];
      double acc = (mine && i > j0 + p) ? fma(x.x, x.x, x.y * x.y) : 0.0;
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
      if (lane == 0) s_wn[rg] = acc;
      if (i == j0 + p) s_alpha = x;
    }
  };
  publish_norm(0);
  cluster_arrive();

#pragma unroll 1
  for (int jj = 0; jj < jb; ++jj) {
    const int col = j0 + jj;
    const int owner = jj / chunk;
    const int oh = jj & 1;
    cluster_wait();
    // ---- warp 0: the reflector scalars (fixed summation order)
    if (warp == 0) {
      const int np = cs * ng;
      double v = 0.0;
      if (lane < np) v = cluster.map_shared_rank(s_wn, lane / ng)[lane % ng];
      if (lane + 32 < np) v += cluster.map_shared_rank(s_wn, (lane + 32) / ng)[(lane + 32) % ng];
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
      const double xn2 = v;
      const double2 alpha = *cluster.map_shared_rank(&s_alpha, owner);
      const bool apply = !(xn2 == 0.0 && alpha.y == 0.0);
      double beta = 0.0, dx = 0.0, d2 = 1.0;
      if (apply) {
        beta = -copysign(sqrt(alpha.x * alpha.x + alpha.y * alpha.y + xn2), alpha.x);
        dx = alpha.x - beta;
        d2 = dx * dx + alpha.y * alpha.y;
      }
      const double rec = 1.0 / ((lane == 0) ? (apply ? beta : 1.0) : d2);
      const double ib = __shfl_sync(0xffffffffu, rec, 0);
      const double id2 = __shfl_sync(0xffffffffu, rec, 1);
      if (lane == 0) {
        double2 tau = c2(0.0, 0.0), scal = c2(0.0, 0.0);
        if (apply) {
          tau = c2((beta - alpha.x) * ib, -alpha.y * ib);
          scal = c2(dx * id2, -alpha.y * id2);
        }
        s_tau[jj] = tau;
        s_scal = scal;
        s_beta = beta;
        s_apply = apply ? 1 : 0;
      }
    }
    __syncthreads();
    const bool apply = s_apply != 0;
    const double2 xj = xs[jj * R + lr];
    double2 xjn = xj;
    if (apply && mine && i > col) xjn = cmul(xj, s_scal);
    if (apply && i == col) xjn = c2(s_beta, 0.0);
    const double2 vcur = (mine && i >= col) ? ((i == col) ? c2(1.0, 0.0) : xjn) : c2(0.0, 0.0);
    const double2 vc = cconj(vcur);
    // ---- products conj(v) x_c of this row, own set
#pragma unroll
    for (int t = 0; t < NB / 2; ++t) {
      const int c = 2 * t + ch;
      qs[lr * 17 + c] = cmul(vc, xs[c * R + lr]);
    }
    __syncthreads();
    // ---- column sums: thread (c, 8-row block), the two blocks of a warp, per warp
    {
      const int c = tid & 15, p = tid >> 4;
      const double2* src = qs + (8 * p) * 17 + c;
      double2 s01 = cadd(src[0 * 17], src[1 * 17]), s23 = cadd(src[2 * 17], src[3 * 17]);
      double2 s45 = cadd(src[4 * 17], src[5 * 17]), s67 = cadd(src[6 * 17], src[7 * 17]);
      double2 s = cadd(cadd(s01, s23), cadd(s45, s67));
      s = cadd(s, c2(__shfl_xor_sync(0xffffffffu, s.x, 16), __shfl_xor_sync(0xffffffffu, s.y, 16)));
      if (lane < 16) s_wv[warp][c] = s;
    }
    __syncthreads();
    if (tid < NB) {
      double2 s = s_wv[0][tid];
      for (int w = 1; w < nw; ++w) s = cadd(s, s_wv[w][tid]);
      s_vec[tid] = s;
    }
    cluster.sync();
    // ---- row group 0, one warp per set: gather four ranks per lane, then the quarters
    if (rg == 0) {
      const int t = lane & 7, rq = lane >> 3;
      const int c = 2 * t + ch;
      double2 vals[4];
#pragma unroll
      for (int k = 0; k < 4; ++k) {
        const int rr = rq * 4 + k;
        vals[k] = (rr < cs) ? cluster.map_shared_rank(s_vec, rr)[c] : c2(0.0, 0.0);
      }
      double2 tot = cadd(cadd(vals[0], vals[1]), cadd(vals[2], vals[3]));
      tot = cadd(tot, c2(__shfl_xor_sync(0xffffffffu, tot.x, 8), __shfl_xor_sync(0xffffffffu, tot.y, 8)));
      tot = cadd(tot, c2(__shfl_xor_sync(0xffffffffu, tot.x, 16), __shfl_xor_sync(0xffffffffu, tot.y, 16)));
      if (rq == 0) {
        if (rank == 0 && c < jj) s_G[c][jj] = cconj(tot);   // v_c^H v_jj
        s_upd[c] = (apply && c > jj) ? cmul(cconj(s_tau[jj]), tot) : c2(0.0, 0.0);
      }
    }
    __syncthreads();
    // ---- next pivot first: update, publish its norm, arrive; then the rest
    auto upd = [&](int c) {
      const double2 s = s_upd[c];
      double2 x = xs[c * R + lr];
      x.x = fma(-vcur.x, s.x, x.x);
      x.x = fma(vcur.y, s.y, x.x);
      x.y = fma(-vcur.x, s.y, x.y);
      x.y = fma(-vcur.y, s.x, x.y);
      xs[c * R + lr] = x;
    };
    if (ch == oh) xs[jj * R + lr] = xjn;   // the pivot column takes its reflector
    if (jj + 1 < jb) {
      if (ch != oh) upd(jj + 1);
      publish_norm(jj + 1);
      cluster_arrive();
    }
#pragma unroll 1
    for (int t = (jj + 3 - ch) >> 1; 2 * t + ch < jb; ++t) upd(2 * t + ch);
  }

  // ---- write the panel back and the explicit V
  if (mine) {
#pragma unroll
    for (int t = 0; t < NB / 2; ++t) {
      const int c = 2 * t + ch;
      if (c < jb) {
        const int colc = j0 + c;
        const double2 x = xs[c * R + lr];
        a[(long)i * lda + colc] = x;
        V[(long)i * ldv + colc] = (i < colc) ? c2(0.0, 0.0) : (i == colc) ? c2(1.0, 0.0) : x;
      }
    }
  }
  // ---- T (zlarft) on rank 0 from the Gram entries
  if (rank == 0) {
    __syncthreads();
    if (warp == 0) {
      double2 T[NB];
#pragma unroll
      for (int c = 0; c < NB; ++c) T[c] = c2(0.0, 0.0);
#pragma unroll
      for (int c = 0; c < NB; ++c) {
        if (c < jb) {
          double2 acc2 = c2(0.0, 0.0);
#pragma unroll
          for (int qq = 0; qq < NB; ++qq)
            if (qq < c && lane <= qq) acc2 = cfma(T[qq], s_G[qq][c], acc2);
          const double2 tc = s_tau[c];
          if (lane < c) T[c] = cmul(c2(-tc.x, -tc.y), acc2);
          if (lane == c) T[c] = tc;
        }
      }
      if (lane < NB)
#pragma unroll
        for (int c = 0; c < NB; ++c) Tout[lane * NB + c] = T[c];
    }
  }
  cluster.sync();   // no CTA leaves while its shared memory may still be read
}

size_t panel7_smem_bytes(int ng) { return (size_t)(NB * 32 * ng + 32 * ng * 17) * sizeof(double2); }

// partial[rb][j][c] = sum_{rows r of tile rb} conj(V[r][v0 + j]) C[r][c0 + c]
// lane layout: tr = lane & 7 (row phase), 4 columns per warp, 8 warps -> 32 columns.
template <int RTT, int CTT>
__global__ void __launch_bounds__(256) larfb_partial_kernel(const double2* __restrict__ C, long ldc,
                                                            const double2* __restrict__ V, long ldv,
                                                            int r0, int m, int c0, int nc, int v0,
                                                            int jb, double2* __restrict__ part) {
  __shared__ double2 sv[RTT][NB];
  const int rb = blockIdx.y;
  const int rbase = r0 + rb * RTT;
  for (int idx = threadIdx.x; idx < RTT * NB; idx += blockDim.x) {
    const int rr = idx / NB, j = idx % NB;
    const int r = rbase + rr;
    sv[rr][j] = (r < m && j < jb) ? V[(long)r * ldv + v0 + j] : c2(0.0, 0.0);
  }
  __syncthreads();
  constexpr int CPW = CTT / 8;             // columns per warp
  constexpr int RPH = 32 / CPW;            // row phases per column
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const int tr = lane % RPH;
  const int cc = wid * CPW + lane / RPH;
  const int c = c0 + blockIdx.x * CTT + cc;
  double2 acc[NB];
#pragma unroll
  for (int j = 0; j < NB; ++j) acc[j] = c2(0.0, 0.0);
  if (c < c0 + nc) {
    for (int rr = tr; rr < RTT; rr += RPH) {
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
    for (int o = 1; o < RPH; o <<= 1) {
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

// W = sum_rb partial; W2 = op(T) W (op = T^H if conjT else T), once per column
// tile; W2 overwrites block 0 of the partials (each CTA owns its columns).
template <int CTT>
__global__ void __launch_bounds__(256) larfb_w2_kernel(double2* __restrict__ part, int nc, int jb,
                                                       int nrb, const double2* __restrict__ T,
                                                       int conjT) {
  __shared__ double2 sw[NB][CTT];
  __shared__ double2 sT[NB][NB];
  if (threadIdx.x < NB * NB) sT[threadIdx.x / NB][threadIdx.x % NB] = T[threadIdx.x];
  for (int idx = threadIdx.x; idx < NB * CTT; idx += blockDim.x) {
    const int j = idx / CTT, cc = idx % CTT;
    const int c = blockIdx.x * CTT + cc;
    double2 s = c2(0.0, 0.0);
    if (j < jb && c < nc)
      for (int b = 0; b < nrb; ++b) s = cadd(s, part[((long)b * NB + j) * nc + c]);
    sw[j][cc] = s;
  }
  __syncthreads();
  for (int idx = threadIdx.x; idx < NB * CTT; idx += blockDim.x) {
    const int j = idx / CTT, cc = idx % CTT;
    const int c = blockIdx.x * CTT + cc;
    double2 s = c2(0.0, 0.0);
    if (j < jb) {
      if (conjT) {
        for (int q = 0; q <= j; ++q) s = cadd(s, cmul(cconj(sT[q][j]), sw[q][cc]));
      } else {
        for (int q = j; q < jb; ++q) s = cadd(s, cmul(sT[j][q], sw[q][cc]));
      }
    }
    if (c < nc) part[(long)j * nc + c] = s;
  }
}

// C -= V W2 on this tile (W2 from larfb_w2_kernel)
template <int RTT, int CTT>
__global__ void __launch_bounds__(256) larfb_update_kernel(double2* __restrict__ C, long ldc,
                                                           const double2* __restrict__ V, long ldv,
                                                           int r0, int m, int c0, int nc, int v0,
                                                           int jb, const double2* __restrict__ W2) {
  __shared__ double2 sv[RTT][NB];
  __shared__ double2 sw2[NB][CTT];
  const int rb = blockIdx.y;
  const int rbase = r0 + rb * RTT;
  for (int idx = threadIdx.x; idx < RTT * NB; idx += blockDim.x) {
    const int rr = idx / NB, j = idx % NB;
    const int r = rbase + rr;
    sv[rr][j] = (r < m && j < jb) ? V[(long)r * ldv + v0 + j] : c2(0.0, 0.0);
  }
  for (int idx = threadIdx.x; idx < NB * CTT; idx += blockDim.x) {
    const int j = idx / CTT, cc = idx % CTT;
    const int c = blockIdx.x * CTT + cc;
    sw2[j][cc] = (j < jb && c < nc) ? W2[(long)j * nc + c] : c2(0.0, 0.0);
  }
  __syncthreads();
  const int tc = threadIdx.x % CTT, tr = threadIdx.x / CTT;
  const int c = c0 + blockIdx.x * CTT + tc;
  if (c >= c0 + nc) return;
  for (int rr = tr; rr < RTT; rr += 256 / CTT) {
    const int r = rbase + rr;
    if (r >= m) break;
    double2 x = C[(long)r * ldc + c];
#pragma unroll
    for (int j = 0; j < NB; ++j)
      if (j < jb) x = csub(x, cmul(sv[rr][j], sw2[j][tc]));
    C[(long)r * ldc + c] = x;
  }
}

// ---------------------------------------------------------------------------
// Register-tiled block reflector application (the default block update):
//   C <- (I - V op(T) V^H) C   on rows [r0, m), columns [c0, c0 + nc)
// as three launches
//   larfb_vhc_kernel   : W_s = V_s^H C_s per (column tile, row split s): one column
//                        per lane (TC = 32), or per half-warp with two row phases
//                        (TC = 16, the narrow look-ahead update), the split's rows
//                        over LW warps, summed over warps and phases in shared memory;
//   larfb_tw1_kernel   : W2 = op(T) sum_s W_s per column, the splits summed in a
//                        fixed order;
//   larfb_apply_kernel : C -= V W2, one column per lane with its W2 column in registers.
// On GB300 every FP64 instruction takes a warp slot of the SM's small FP64 pipe, so
// the inner loops are FMA only (no cross-lane reductions inside the row loop) and
// the columns past jb are zero rather than predicated off.
constexpr int LW = 4;   // warps per CTA of the block-update kernels

template <int RPW, int TC>
__global__ void __launch_bounds__(LW * 32) larfb_vhc_kernel(const double2* __restrict__ C, long ldc,
                                                            const double2* __restrict__ V, long ldv,
                                                            int r0, int m, int c0, int nc, int v0,
                                                            int jb, double2* __restrict__ part) {
  constexpr int PH = 32 / TC;             // row phases per warp
  constexpr int RS = LW * RPW * PH;       // rows of one split
  constexpr int NRED = LW * PH;           // partials per output inside the CTA
  static_assert(RS * NB <= NRED * NB * TC, "shared buffer sized by the reduction");
  __shared__ double2 sm[NRED * NB * TC];  // V rows of the split, then the partials
  const int s = blockIdx.y;
  const int rbase = r0 + s * RS;
  for (int idx = threadIdx.x; idx < RS * NB; idx += LW * 32) {
    const int rr = idx / NB, j = idx % NB;
    const int r = rbase + rr;
    sm[idx] = (r < m && j < jb) ? V[(long)r * ldv + v0 + j] : c2(0.0, 0.0);
  }
  __syncthreads();
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int col = lane % TC, ph = lane / TC;
  const int cl = blockIdx.x * TC + col;
  const bool live = cl < nc;
  double2 acc[NB];
#pragma unroll
  for (int j = 0; j < NB; ++j) acc[j] = c2(0.0, 0.0);
  const int rw = warp * RPW * PH + ph;
#pragma unroll 2
  for (int i = 0; i < RPW; ++i) {
    const int rr = rw + i * PH;
    const int r = rbase + rr;
    if (r >= m) break;
    const double2 x = live ? C[(long)r * ldc + c0 + cl] : c2(0.0, 0.0);
    const double2* vr = sm + rr * NB;
#pragma unroll
    for (int j = 0; j < NB; ++j) {
      const double2 v = vr[j];
      acc[j].x = fma(v.x, x.x, acc[j].x);
      acc[j].x = fma(v.y, x.y, acc[j].x);
      acc[j].y = fma(v.x, x.y, acc[j].y);
      acc[j].y = fma(-v.y, x.x, acc[j].y);
    }
  }
  __syncthreads();   // the V rows are no longer needed: reuse the buffer for the partials
  const int p = warp * PH + ph;
#pragma unroll
  for (int j = 0; j < NB; ++j) sm[(p * NB + j) * TC + col] = acc[j];
  __syncthreads();
  for (int o = threadIdx.x; o < NB * TC; o += LW * 32) {
    const int j = o / TC, cc = o % TC;
    double2 t = sm[o];
#pragma unroll
    for (int q = 1; q < NRED; ++q) t = cadd(t, sm[q * NB * TC + o]);
    const int c = blockIdx.x * TC + cc;
    if (c < nc) part[((long)s * NB + j) * nc + c] = t;
  }
}

// W2 = op(T) sum_s W_s, one column per CTA (W2 replaces split 0 of the partials;
// every CTA reads and writes only its own column). On GB300 each of an SM's four
// sub-partitions issues one FP64 warp instruction per ~64 cycles, so the split
// sums and the triangular product are spread over as many SMs as there are
// columns. Thread
// (j, part) sums the splits s = part (mod 8) of W[j]; three tree levels combine the
// parts; thread (j, part) then forms two terms of (op(T) W)[j], combined the same way.
__global__ void __launch_bounds__(128) larfb_tw1_kernel(double2* __restrict__ part, int nsplit,
                                                        int nc, int jb,
                                                        const double2* __restrict__ T,
                                                        int conjT) {
  __shared__ double2 sT[NB][NB];
  __shared__ double2 sp[8][NB];
  __shared__ double2 sw[NB];
  const int c = blockIdx.x;
  const int j = threadIdx.x & 15, pp = threadIdx.x >> 4;
  for (int e = threadIdx.x; e < NB * NB; e += 128) sT[e / NB][e % NB] = T[e];
  double2 s0 = c2(0.0, 0.0);
  if (j < jb) {
    const double2* src = part + (long)j * nc + c;
    const long st = (long)NB * nc;
    // eight independent loads in flight per round, summed as a tree
    for (int base = pp; base < nsplit; base += 64) {
      double2 v[8];
#pragma unroll
      for (int u = 0; u < 8; ++u) {
        const int s = base + 8 * u;
        v[u] = (s < nsplit) ? src[(long)s * st] : c2(0.0, 0.0);
      }
      s0 = cadd(s0, cadd(cadd(cadd(v[0], v[1]), cadd(v[2], v[3])),
                         cadd(cadd(v[4], v[5]), cadd(v[6], v[7]))));
    }
  }
  sp[pp][j] = s0;
  __syncthreads();
  if (pp < 4) sp[pp][j] = cadd(sp[pp][j], sp[pp + 4][j]);
  __syncthreads();
  if (pp < 2) sp[pp][j] = cadd(sp[pp][j], sp[pp + 2][j]);
  __syncthreads();
  if (pp == 0) sw[j] = cadd(sp[0][j], sp[1][j]);
  __syncthreads();
  // (op(T) W)[j] = sum_q op(T)[j][q] W[q]; thread (j, pp) takes q = pp and pp + 8
  double2 acc = c2(0.0, 0.0);
  if (j < jb) {
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      const int q = pp + 8 * h;
      const double2 t = conjT ? cconj(sT[q][j]) : sT[j][q];
      const bool tri = conjT ? (q <= j) : (q >= j && q < jb);
      if (tri) acc = cfma(t, sw[q], acc);
    }
  }
  sp[pp][j] = acc;
  __syncthreads();
  if (pp < 4) sp[pp][j] = cadd(sp[pp][j], sp[pp + 4][j]);
  __syncthreads();
  if (pp < 2) sp[pp][j] = cadd(sp[pp][j], sp[pp + 2][j]);
  __syncthreads();
  if (pp == 0) part[(long)j * nc + c] = cadd(sp[0][j], sp[1][j]);
}

template <int RPW, int TC>
__global__ void __launch_bounds__(LW * 32) larfb_apply_kernel(double2* __restrict__ C, long ldc,
                                                              const double2* __restrict__ V, long ldv,
                                                              int r0, int m, int c0, int nc, int v0,
                                                              int jb, const double2* __restrict__ W2) {
  constexpr int PH = 32 / TC;
  constexpr int RT = LW * RPW * PH;       // rows of one CTA
  __shared__ double2 sv[RT * NB];
  const int rbase = r0 + blockIdx.y * RT;
  for (int idx = threadIdx.x; idx < RT * NB; idx += LW * 32) {
    const int rr = idx / NB, j = idx % NB;
    const int r = rbase + rr;
    sv[idx] = (r < m && j < jb) ? V[(long)r * ldv + v0 + j] : c2(0.0, 0.0);
  }
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int col = lane % TC, ph = lane / TC;
  const int cl = blockIdx.x * TC + col;
  const bool live = cl < nc;
  double2 w[NB];
#pragma unroll
  for (int j = 0; j < NB; ++j) w[j] = live ? W2[(long)j * nc + cl] : c2(0.0, 0.0);
  __syncthreads();
  if (!live) return;
  const int rw = warp * RPW * PH + ph;
#pragma unroll 2
  for (int i = 0; i < RPW; ++i) {
    const int rr = rw + i * PH;
    const int r = rbase + rr;
    if (r >= m) break;
    double2* px = C + (long)r * ldc + c0 + cl;
    double2 x = *px;
    const double2* vr = sv + rr * NB;
#pragma unroll
    for (int j = 0; j < NB; ++j) {
      const double2 v = vr[j];
      x.x = fma(-v.x, w[j].x, x.x);
      x.x = fma(v.y, w[j].y, x.x);
      x.y = fma(-v.x, w[j].y, x.y);
      x.y = fma(-v.y, w[j].x, x.y);
    }
    *px = x;
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
  double2* part;    // block-update partials (the narrow and the look-ahead update never overlap)
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

template <int RTT, int CTT>
ptn_status larfb_t(double2* C, long ldc, const double2* V, long ldv, int r0, int m, int c0, int nc,
                   int v0, int jb, const double2* T, bool conjT, double2* part, cudaStream_t st) {
  const int nrb = (m - r0 + RTT - 1) / RTT;
  dim3 grid((nc + CTT - 1) / CTT, nrb);
  larfb_partial_kernel<RTT, CTT><<<grid, 256, 0, st>>>(C, ldc, V, ldv, r0, m, c0, nc, v0, jb, part);
  larfb_w2_kernel<CTT><<<grid.x, 256, 0, st>>>(part, nc, jb, nrb, T, conjT ? 1 : 0);
  larfb_update_kernel<RTT, CTT><<<grid, 256, 0, st>>>(C, ldc, V, ldv, r0, m, c0, nc, v0, jb, part);
  PTN_LAUNCH_CHECK();
  note_launches(3);
  return PTN_OK;
}

// register-tiled form: rows per warp chosen so that the launch has about two CTAs
// per SM (every SM's FP64 pipe busy) while a split keeps at least 8 rows (the
// workspace holds (m + 7) / 8 splits)
template <int TC>
ptn_status larfb_rt(double2* C, long ldc, const double2* V, long ldv, int r0, int m, int c0, int nc,
                    int v0, int jb, const double2* T, bool conjT, double2* part, cudaStream_t st) {
  constexpr int PH = 32 / TC;
  const long rows = m - r0;
  const long ctiles = (nc + TC - 1) / TC;
  const long want = 2L * num_sms();
  auto splits = [&](int rpw) { return (rows + LW * rpw * PH - 1) / (LW * rpw * PH); };
  auto choose = [&](int lo) {
    for (int rpw = 16; rpw > lo; rpw >>= 1)
      if (ctiles * splits(rpw) >= want) return rpw;
    return lo;
  };
  const int rp = choose(2 / PH);      // partial pass: at least 8 rows per split
  const int ra = choose(1);           // apply pass
  const int nsplit = (int)splits(rp);
  const dim3 gp((unsigned)ctiles, (unsigned)nsplit);
  switch (rp) {
    case 16: larfb_vhc_kernel<16, TC><<<gp, LW * 32, 0, st>>>(C, ldc, V, ldv, r0, m, c0, nc, v0, jb, part); break;
    case 8: larfb_vhc_kernel<8, TC><<<gp, LW * 32, 0, st>>>(C, ldc, V, ldv, r0, m, c0, nc, v0, jb, part); break;
    case 4: larfb_vhc_kernel<4, TC><<<gp, LW * 32, 0, st>>>(C, ldc, V, ldv, r0, m, c0, nc, v0, jb, part); break;
    case 2: larfb_vhc_kernel<2, TC><<<gp, LW * 32, 0, st>>>(C, ldc, V, ldv, r0, m, c0, nc, v0, jb, part); break;
    default: larfb_vhc_kernel<1, TC><<<gp, LW * 32, 0, st>>>(C, ldc, V, ldv, r0, m, c0, nc, v0, jb, part); break;
  }
  larfb_tw1_kernel<<<nc, 128, 0, st>>>(part, nsplit, nc, jb, T, conjT ? 1 : 0);
  const dim3 ga((unsigned)ctiles, (unsigned)splits(ra));
  switch (ra) {
    case 16: larfb_apply_kernel<16, TC><<<ga, LW * 32, 0, st>>>(C, ldc, V, ldv, r0, m, c0, nc, v0, jb, part); break;
    case 8: larfb_apply_kernel<8, TC><<<ga, LW * 32, 0, st>>>(C, ldc, V, ldv, r0, m, c0, nc, v0, jb, part); break;
    case 4: larfb_apply_kernel<4, TC><<<ga, LW * 32, 0, st>>>(C, ldc, V, ldv, r0, m, c0, nc, v0, jb, part); break;
    case 2: larfb_apply_kernel<2, TC><<<ga, LW * 32, 0, st>>>(C, ldc, V, ldv, r0, m, c0, nc, v0, jb, part); break;
    default: larfb_apply_kernel<1, TC><<<ga, LW * 32, 0, st>>>(C, ldc, V, ldv, r0, m, c0, nc, v0, jb, part); break;
  }
  PTN_LAUNCH_CHECK();
  note_launches(3);
  return PTN_OK;
}

// PTN_TUNE_LARFB_TILE 0: the register-tiled form (16-column tiles for narrow
// updates); 1..4 the earlier three-pass kernels with a fixed tile; 5 those kernels
// with the tile chosen per call so that shrinking trailing matrices still launch
// enough CTAs to keep every SM's FP64 pipes busy
ptn_status larfb(double2* C, long ldc, const double2* V, long ldv, int r0, int m, int c0, int nc,
                 int v0, int jb, const double2* T, bool conjT, double2* part, cudaStream_t st) {
  switch (tune(PTN_TUNE_LARFB_TILE)) {
    case 0:
      if (nc <= 16) return larfb_rt<16>(C, ldc, V, ldv, r0, m, c0, nc, v0, jb, T, conjT, part, st);
      return larfb_rt<32>(C, ldc, V, ldv, r0, m, c0, nc, v0, jb, T, conjT, part, st);
    case 1: return larfb_t<16, 16>(C, ldc, V, ldv, r0, m, c0, nc, v0, jb, T, conjT, part, st);
    case 2: return larfb_t<32, 16>(C, ldc, V, ldv, r0, m, c0, nc, v0, jb, T, conjT, part, st);
    case 3: return larfb_t<32, 32>(C, ldc, V, ldv, r0, m, c0, nc, v0, jb, T, conjT, part, st);
    case 4: return larfb_t<64, 32>(C, ldc, V, ldv, r0, m, c0, nc, v0, jb, T, conjT, part, st);
    default: break;
  }
  const long rows = m - r0;
  const long want = 2L * num_sms();
  auto ctas = [&](long rt, long ct) { return ((rows + rt - 1) / rt) * ((nc + ct - 1) / ct); };
  if (ctas(64, 32) >= want) return larfb_t<64, 32>(C, ldc, V, ldv, r0, m, c0, nc, v0, jb, T, conjT, part, st);
  if (ctas(32, 32) >= want) return larfb_t<32, 32>(C, ldc, V, ldv, r0, m, c0, nc, v0, jb, T, conjT, part, st);
  if (ctas(32, 16) >= want) return larfb_t<32, 16>(C, ldc, V, ldv, r0, m, c0, nc, v0, jb, T, conjT, part, st);
  return larfb_t<16, 16>(C, ldc, V, ldv, r0, m, c0, nc, v0, jb, T, conjT, part, st);
}

}  // namespace

namespace {

// Largest cluster the panel kernel can be launched with on this device (16, else 8,
// else 1 = the single-CTA kernel); decided once.
int panel_cluster_size() {
  static int cs = 0;
  if (cs != 0) return cs;
  cs = 1;
  if (cudaFuncSetAttribute(qr_panel_cluster_kernel, cudaFuncAttributeNonPortableClusterSizeAllowed,
                           1) != cudaSuccess)
    cudaGetLastError();
  if (cudaFuncSetAttribute(qr_panel4_kernel, cudaFuncAttributeNonPortableClusterSizeAllowed, 1) !=
      cudaSuccess)
    cudaGetLastError();
  if (cudaFuncSetAttribute(qr_panel5_kernel, cudaFuncAttributeNonPortableClusterSizeAllowed, 1) !=
      cudaSuccess)
    cudaGetLastError();
  if (cudaFuncSetAttribute(qr_panel6_kernel, cudaFuncAttributeNonPortableClusterSizeAllowed, 1) !=
      cudaSuccess)
    cudaGetLastError();
  if (cudaFuncSetAttribute(qr_panel7_kernel, cudaFuncAttributeNonPortableClusterSizeAllowed, 1) !=
      cudaSuccess)
    cudaGetLastError();
  if (cudaFuncSetAttribute(qr_panel7_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                           (int)panel7_smem_bytes(P6W / 2)) != cudaSuccess)
    cudaGetLastError();
  for (int c : {16, 8}) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(c);
    cfg.blockDim = dim3(CPT);
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = c;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    int nclusters = 0;
    if (cudaOccupancyMaxActiveClusters(&nclusters, qr_panel_cluster_kernel, &cfg) == cudaSuccess &&
        nclusters > 0) {
      cs = c;
      break;
    }
    cudaGetLastError();
  }
  return cs;
}

}  // namespace

// Side streams for the look-ahead of the factorisation: a small fixed pool, created
// at the first QR (which runs eagerly, before any graph capture), lowest priority so
// that the panel on the caller's stream gets its SMs first; a caller's stream maps
// to one of them by its handle. Fork / join events are per side stream; every use is
// issued from one host thread in order, so reusing them is safe (a wait takes the
// event's latest record at the time of the call).
struct SideStreams {
  static constexpr int N = 8;
  cudaStream_t s[N] = {};
  cudaEvent_t fork[N] = {}, join[N] = {};
  int device = -1;   // the device they belong to (the look-ahead is off on others)
  bool ok = false;
};

SideStreams& side_streams() {
  static SideStreams ss;
  static std::once_flag once;
  std::call_once(once, [] {
    int least = 0, greatest = 0;
    if (cudaDeviceGetStreamPriorityRange(&least, &greatest) != cudaSuccess) least = 0;
    bool good = true;
    for (int i = 0; i < SideStreams::N && good; ++i) {
      good = cudaStreamCreateWithPriority(&ss.s[i], cudaStreamNonBlocking, least) == cudaSuccess &&
             cudaEventCreateWithFlags(&ss.fork[i], cudaEventDisableTiming) == cudaSuccess &&
             cudaEventCreateWithFlags(&ss.join[i], cudaEventDisableTiming) == cudaSuccess;
    }
    if (!good) cudaGetLastError();
    if (cudaGetDevice(&ss.device) != cudaSuccess) good = false;
    ss.ok = good;
  });
  return ss;
}

int side_index(cudaStream_t st) {
  const uintptr_t h = reinterpret_cast<uintptr_t>(st);
  return (int)((h >> 4) % SideStreams::N);
}

size_t qr_workspace_bytes(int m, int n) {
  const int k = std::min(m, n);
  const int np = (k + NB - 1) / NB;
  const int nrb = (m + 7) / 8;     // most row splits of a block update
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
  const int cs_max = panel_cluster_size();
  const int cap = tune(PTN_TUNE_QR_CLUSTER);
  auto panel = [&](int j0, int p) -> ptn_status {
    const int jb = std::min(NB, k - j0);
    // cluster of the panel: at least 32 rows per CTA (power of two), at most the
    // device's largest cluster and the tuning cap; small panels take few CTAs and so
    // leave the other SMs of the GPC to concurrent work
    int cs = 1;
    while (cs < cs_max && cs * 32 < m - j0) cs *= 2;
    if (cap > 0) cs = std::min(cs, cap);
    const int chunk = cs > 1 ? (m - j0 + cs - 1) / cs : m - j0;
    if (chunk <= QW * 32) {   // a cluster of one CTA is the single-CTA case
      cudaLaunchConfig_t cfg = {};
      const int form = tune(PTN_TUNE_QR_PANEL);
      const int ngroups = (chunk + 31) / 32;
      cfg.gridDim = dim3(cs);
      // warps the row chunk needs (two per 32-row group for the two-set panels)
      cfg.blockDim = dim3((form == 0 || form == 3 ? 64 : 32) * ngroups);
      cfg.dynamicSmemBytes = form == 0 ? panel7_smem_bytes(ngroups) : 0;
      cfg.stream = st;
      cudaLaunchAttribute attr[1];
      attr[0].id = cudaLaunchAttributeClusterDimension;
      attr[0].val.clusterDim.x = cs;
      attr[0].val.clusterDim.y = 1;
      attr[0].val.clusterDim.z = 1;
      cfg.attrs = attr;
      cfg.numAttrs = 1;
      if (form == 0)
        PTN_CUDA_TRY(cudaLaunchKernelEx(&cfg, qr_panel7_kernel, a, lda, m, j0, jb,
                                        w.T + (long)p * NB * NB, w.V, (long)k));
      else if (form == 3)
        PTN_CUDA_TRY(cudaLaunchKernelEx(&cfg, qr_panel6_kernel, a, lda, m, j0, jb,
                                        w.T + (long)p * NB * NB, w.V, (long)k));
      else if (form == 2)
        PTN_CUDA_TRY(cudaLaunchKernelEx(&cfg, qr_panel5_kernel, a, lda, m, j0, jb,
                                        w.T + (long)p * NB * NB, w.V, (long)k));
      else
        PTN_CUDA_TRY(cudaLaunchKernelEx(&cfg, qr_panel4_kernel, a, lda, m, j0, jb,
                                        w.T + (long)p * NB * NB, w.V, (long)k));
    } else if (cs > 1) {
      cudaLaunchConfig_t cfg = {};
      cfg.gridDim = dim3(cs);
      cfg.blockDim = dim3(CPT);
      cfg.dynamicSmemBytes = 0;
      cfg.stream = st;
      cudaLaunchAttribute attr[1];
      attr[0].id = cudaLaunchAttributeClusterDimension;
      attr[0].val.clusterDim.x = cs;
      attr[0].val.clusterDim.y = 1;
      attr[0].val.clusterDim.z = 1;
      cfg.attrs = attr;
      cfg.numAttrs = 1;
      PTN_CUDA_TRY(cudaLaunchKernelEx(&cfg, qr_panel_cluster_kernel, a, lda, m, j0, jb,
                                      w.T + (long)p * NB * NB, w.V, (long)k));
    } else {
      qr_panel_kernel<<<1, PT, 0, st>>>(a, lda, m, j0, jb, w.T + (long)p * NB * NB, w.V, k);
    }
    PTN_LAUNCH_CHECK();
    note_launches(1);
    return PTN_OK;
  };
  // Look-ahead: after panel p, reflector p is applied first to the columns of panel
  // p + 1 only (caller's stream), then to the remaining trailing columns on a side
  // stream while panel p + 1 is factorised on the caller's stream: the latency-bound
  // panel (one cluster) overlaps the throughput-bound update (the other SMs). The
  // column ranges are disjoint; the side stream joins back before the next narrow
  // update (whose columns it has just updated) and at the end. Same kernels and the
  // same arithmetic as without look-ahead.
  SideStreams& ss = side_streams();
  const int si = side_index(st);
  int dev = -1;
  PTN_CUDA_TRY(cudaGetDevice(&dev));
  const bool look_ahead = ss.ok && ss.device == dev && k > NB;
  bool pending = false;   // side-stream work not yet joined
  PTN_TRY(panel(0, 0));
  for (int j0 = 0, p = 0; j0 < k; j0 += NB, ++p) {
    const int jb = std::min(NB, k - j0);
    const int nc = n - j0 - jb;                               // trailing columns
    const int jn = std::min(NB, std::max(0, k - (j0 + jb)));  // next panel's columns
    if (pending) {
      PTN_CUDA_TRY(cudaStreamWaitEvent(st, ss.join[si], 0));
      pending = false;
    }
    if (!look_ahead) {
      if (nc > 0)
        PTN_TRY(larfb(a, lda, w.V, k, j0, m, j0 + jb, nc, j0, jb, w.T + (long)p * NB * NB, true,
                      w.part, st));
      if (jn > 0) PTN_TRY(panel(j0 + jb, p + 1));
      continue;
    }
    if (jn > 0)
      PTN_TRY(larfb(a, lda, w.V, k, j0, m, j0 + jb, jn, j0, jb, w.T + (long)p * NB * NB, true,
                    w.part, st));
    const int rest = nc - jn;
    if (rest > 0) {
      PTN_CUDA_TRY(cudaEventRecord(ss.fork[si], st));
      PTN_CUDA_TRY(cudaStreamWaitEvent(ss.s[si], ss.fork[si], 0));
      PTN_TRY(larfb(a, lda, w.V, k, j0, m, j0 + jb + jn, rest, j0, jb, w.T + (long)p * NB * NB,
                    true, w.part, ss.s[si]));
      PTN_CUDA_TRY(cudaEventRecord(ss.join[si], ss.s[si]));
      pending = true;
    }
    if (jn > 0) PTN_TRY(panel(j0 + jb, p + 1));
  }
  if (pending) PTN_CUDA_TRY(cudaStreamWaitEvent(st, ss.join[si], 0));
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
