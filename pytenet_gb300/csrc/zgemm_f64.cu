// Complex128 GEMM on the FP64 DMMA tensor-core path (mma.sync m8n8k4 f64).
//
// C = alpha op(A) op(B) + beta C, all row-major, op in {N, T, C, H}. This is the
// contraction engine of the plain (all-FP64) form: every tensordot of
// pytenet/chain_ops.py (apply_local_hamiltonian, the environment steps, the bond
// contraction) and of the sweep (pytenet/tdvp.py:84,112) becomes one call.
//
// Tiling: 64x64 output tile per CTA of 8 warps (2 x 4), warp tile 32x16 = 4x2
// DMMA fragments; K advances in slabs of 16 complex values staged through shared
// memory as separate re/im planes (pitch 68 doubles: the 16-lane halves of a
// fragment load hit 16 distinct 8-byte banks). A complex fragment product is four
// real DMMAs: re += ar*br - ai*bi, im += ar*bi + ai*br.
// Transposition and conjugation are folded into the global->shared load, so no
// operand is ever materialised transposed. Skinny problems (fewer tiles than SMs)
// split K across CTAs and reduce the FP64 partials in a second, deterministic pass.
//
// Block sparsity: a K slab whose A part (64 x 16) or B part (16 x 64) of this tile is
// entirely zero contributes nothing and its DMMAs are skipped (the barrier after the
// shared-memory store votes on it). Tensors with quantum numbers hold zero blocks
// (pytenet/block_sparse_util.py:47-64), and after the first block QR every bond is
// ordered by quantum number, so their blocks line up with tiles and slabs; dense data
// pays two barrier votes per slab.
#include "ptn_common.cuh"
#include <algorithm>

namespace ptn {
namespace {

constexpr int BM = 64, BN = 64, BK = 16;
constexpr int PITCH = 68;
constexpr int THREADS = 256;

enum { OP_N = 0, OP_T = 1, OP_C = 2, OP_H = 3 };

__device__ __forceinline__ void dmma(double& d0, double& d1, double a, double b) {
  asm volatile("mma.sync.aligned.m8n8k4.row.col.f64.f64.f64.f64 {%0,%1}, {%2}, {%3}, {%0,%1};\n"
               : "+d"(d0), "+d"(d1)
               : "d"(a), "d"(b));
}

template <int OP>
struct OpTraits {
  static constexpr bool trans = (OP == OP_T || OP == OP_H);
  static constexpr bool conj = (OP == OP_C || OP == OP_H);
};

// whether any of a thread's four loaded entries is non-zero
__device__ __forceinline__ bool nonzero4(const double2 (&r)[4]) {
  bool nz = false;
#pragma unroll
  for (int i = 0; i < 4; ++i) nz |= (r[i].x != 0.0) | (r[i].y != 0.0);
  return nz;
}

// Load op(A)[m0 + m][k0 + k] for the 64x16 tile into registers.
template <int OA>
__device__ __forceinline__ void load_a(double2 (&ra)[4], const double2* __restrict__ A, long lda,
                                       int M, int m0, int k0, int kend) {
  const int tid = threadIdx.x;
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    int m, k;
    if (!OpTraits<OA>::trans) { k = tid & 15; m = (tid >> 4) + 16 * i; }
    else                      { m = tid & 63; k = (tid >> 6) + 4 * i; }
    const int gm = m0 + m, gk = k0 + k;
    double2 v = make_double2(0.0, 0.0);
    if (gm < M && gk < kend)
      v = OpTraits<OA>::trans ? A[(long)gk * lda + gm] : A[(long)gm * lda + gk];
    if (OpTraits<OA>::conj) v.y = -v.y;
    ra[i] = v;
  }
}

template <int OA>
__device__ __forceinline__ void store_a(const double2 (&ra)[4], double (*sre)[PITCH],
                                        double (*sim)[PITCH]) {
  const int tid = threadIdx.x;
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    int m, k;
    if (!OpTraits<OA>::trans) { k = tid & 15; m = (tid >> 4) + 16 * i; }
    else                      { m = tid & 63; k = (tid >> 6) + 4 * i; }
    sre[k][m] = ra[i].x;
    sim[k][m] = ra[i].y;
  }
}

// Load op(B)[k0 + k][n0 + n] for the 16x64 tile.
template <int OB>
__device__ __forceinline__ void load_b(double2 (&rb)[4], const double2* __restrict__ B, long ldb,
                                       int N, int n0, int k0, int kend) {
  const int tid = threadIdx.x;
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    int n, k;
    if (!OpTraits<OB>::trans) { n = tid & 63; k = (tid >> 6) + 4 * i; }
    else                      { k = tid & 15; n = (tid >> 4) + 16 * i; }
    const int gn = n0 + n, gk = k0 + k;
    double2 v = make_double2(0.0, 0.0);
    if (gn < N && gk < kend)
      v = OpTraits<OB>::trans ? B[(long)gn * ldb + gk] : B[(long)gk * ldb + gn];
    if (OpTraits<OB>::conj) v.y = -v.y;
    rb[i] = v;
  }
}

template <int OB>
__device__ __forceinline__ void store_b(const double2 (&rb)[4], double (*sre)[PITCH],
                                        double (*sim)[PITCH]) {
  const int tid = threadIdx.x;
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    int n, k;
    if (!OpTraits<OB>::trans) { n = tid & 63; k = (tid >> 6) + 4 * i; }
    else                      { k = tid & 15; n = (tid >> 4) + 16 * i; }
    sre[k][n] = rb[i].x;
    sim[k][n] = rb[i].y;
  }
}

struct KArgs {
  int M, N, K, batch, splits, kchunk;
  double2 alpha, beta;
  const double2* A; long lda, sA;
  const double2* B; long ldb, sB;
  double2* C; long ldc, sC;
  double2* part;   // split-K partials [batch][splits][M][N], or null
  const int* skip;
};

template <int OA, int OB>
__global__ void __launch_bounds__(THREADS) zgemm_dmma_kernel(const KArgs p) {
  if (p.skip != nullptr && *p.skip != 0) return;
  __shared__ __align__(16) double sa_re[BK][PITCH];
  __shared__ __align__(16) double sa_im[BK][PITCH];
  __shared__ __align__(16) double sb_re[BK][PITCH];
  __shared__ __align__(16) double sb_im[BK][PITCH];

  const int bz = blockIdx.z;
  const int b = bz / p.splits, split = bz % p.splits;
  const int m0 = blockIdx.y * BM, n0 = blockIdx.x * BN;
  const int kbeg = split * p.kchunk;
  const int kend = min(p.K, kbeg + p.kchunk);
  const double2* A = p.A + (long)b * p.sA;
  const double2* B = p.B + (long)b * p.sB;

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int wm = (warp >> 2) * 32, wn = (warp & 3) * 16;
  const int fr = lane >> 2, fc = lane & 3;

  double acc[4][2][4];
#pragma unroll
  for (int i = 0; i < 4; ++i)
#pragma unroll
    for (int j = 0; j < 2; ++j)
#pragma unroll
      for (int t = 0; t < 4; ++t) acc[i][j][t] = 0.0;

  double2 ra[4], rb[4];
  if (kbeg < kend) {
    load_a<OA>(ra, A, p.lda, p.M, m0, kbeg, kend);
    load_b<OB>(rb, B, p.ldb, p.N, n0, kbeg, kend);
  }
  for (int k0 = kbeg; k0 < kend; k0 += BK) {
    __syncthreads();
    store_a<OA>(ra, sa_re, sa_im);
    store_b<OB>(rb, sb_re, sb_im);
    // barrier with a vote: does this slab have a non-zero entry in A's and in B's part
    const int live_a = __syncthreads_or(nonzero4(ra));
    const int live_b = __syncthreads_or(nonzero4(rb));
    const bool live = live_a != 0 && live_b != 0;
    if (k0 + BK < kend) {
      load_a<OA>(ra, A, p.lda, p.M, m0, k0 + BK, kend);
      load_b<OB>(rb, B, p.ldb, p.N, n0, k0 + BK, kend);
    }
    if (!live) continue;
#pragma unroll
    for (int kk = 0; kk < BK; kk += 4) {
      double are[4], aim[4], bre[2], bim[2];
#pragma unroll
      for (int i = 0; i < 4; ++i) {
        are[i] = sa_re[kk + fc][wm + i * 8 + fr];
        aim[i] = sa_im[kk + fc][wm + i * 8 + fr];
      }
#pragma unroll
      for (int j = 0; j < 2; ++j) {
        bre[j] = sb_re[kk + fc][wn + j * 8 + fr];
        bim[j] = sb_im[kk + fc][wn + j * 8 + fr];
      }
#pragma unroll
      for (int i = 0; i < 4; ++i) {
        const double naim = -aim[i];
#pragma unroll
        for (int j = 0; j < 2; ++j) {
          dmma(acc[i][j][0], acc[i][j][1], are[i], bre[j]);
          dmma(acc[i][j][0], acc[i][j][1], naim, bim[j]);
          dmma(acc[i][j][2], acc[i][j][3], are[i], bim[j]);
          dmma(acc[i][j][2], acc[i][j][3], aim[i], bre[j]);
        }
      }
    }
  }

  // epilogue: fragment element (fr, 2*fc + e)
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    const int gm = m0 + wm + i * 8 + fr;
    if (gm >= p.M) continue;
#pragma unroll
    for (int j = 0; j < 2; ++j) {
#pragma unroll
      for (int e = 0; e < 2; ++e) {
        const int gn = n0 + wn + j * 8 + 2 * fc + e;
        if (gn >= p.N) continue;
        const double2 v = make_double2(acc[i][j][e], acc[i][j][2 + e]);
        if (p.part != nullptr) {
          p.part[(((long)b * p.splits + split) * p.M + gm) * p.N + gn] = v;
        } else {
          double2* cp = p.C + (long)b * p.sC + (long)gm * p.ldc + gn;
          double2 out = cmul(p.alpha, v);
          if (p.beta.x != 0.0 || p.beta.y != 0.0) out = cadd(out, cmul(p.beta, *cp));
          *cp = out;
        }
      }
    }
  }
}

__global__ void splitk_reduce_kernel(const KArgs p) {
  if (p.skip != nullptr && *p.skip != 0) return;
  const long total = (long)p.batch * p.M * p.N;
  for (long idx = blockIdx.x * (long)blockDim.x + threadIdx.x; idx < total;
       idx += (long)gridDim.x * blockDim.x) {
    const long b = idx / ((long)p.M * p.N);
    const long mn = idx - b * (long)p.M * p.N;
    const int gm = (int)(mn / p.N), gn = (int)(mn % p.N);
    double2 s = make_double2(0.0, 0.0);
    for (int k = 0; k < p.splits; ++k) s = cadd(s, p.part[((b * p.splits + k) * p.M) * (long)p.N + mn]);
    double2* cp = p.C + b * p.sC + (long)gm * p.ldc + gn;
    double2 out = cmul(p.alpha, s);
    if (p.beta.x != 0.0 || p.beta.y != 0.0) out = cadd(out, cmul(p.beta, *cp));
    *cp = out;
  }
}

int op_code(char c) {
  switch (c) {
    case 'N': case 'n': return OP_N;
    case 'T': case 't': return OP_T;
    case 'C': case 'c': return OP_C;
    case 'H': case 'h': return OP_H;
    default: return -1;
  }
}

template <int OA>
void launch_b(int ob, dim3 grid, cudaStream_t st, const KArgs& k) {
  switch (ob) {
    case OP_N: zgemm_dmma_kernel<OA, OP_N><<<grid, THREADS, 0, st>>>(k); break;
    case OP_T: zgemm_dmma_kernel<OA, OP_T><<<grid, THREADS, 0, st>>>(k); break;
    case OP_C: zgemm_dmma_kernel<OA, OP_C><<<grid, THREADS, 0, st>>>(k); break;
    default:   zgemm_dmma_kernel<OA, OP_H><<<grid, THREADS, 0, st>>>(k); break;
  }
}

// K splits for skinny problems: up to PTN_TUNE_ZGEMM_SPLIT_WAVES waves of CTAs (at
// most 32 splits of at least 4 K slabs), choosing the count with the fewest
// waves x (K slabs per CTA + a fixed per-CTA cost of about SLAB_OVERHEAD slabs).
int choose_splits(int M, int N, int K, int batch) {
  constexpr int SLAB_OVERHEAD = 4;
  const long tiles = (long)((M + BM - 1) / BM) * ((N + BN - 1) / BN) * batch;
  const long sms = num_sms();
  const int waves = tune(PTN_TUNE_ZGEMM_SPLIT_WAVES);
  if (waves == 0 || tiles >= (long)waves * sms || K < 8 * BK) return 1;
  const long slabs = (K + BK - 1) / BK;
  long s_cap = ((long)waves * sms + tiles - 1) / tiles;
  s_cap = std::min<long>(s_cap, std::max(1, K / (4 * BK)));
  s_cap = std::min<long>(s_cap, 32);
  int best = 1;
  long best_cost = -1;
  for (long s = 1; s <= s_cap; ++s) {
    const long w = (tiles * s + sms - 1) / sms;
    const long cost = w * ((slabs + s - 1) / s + SLAB_OVERHEAD);
    if (best_cost < 0 || cost < best_cost) {
      best_cost = cost;
      best = (int)s;
    }
  }
  return best;
}

}  // namespace

void note_launches(int n);

size_t zgemm_workspace_bytes(int M, int N, int K, int batch) {
  const int s = choose_splits(M, N, K, batch);
  return s > 1 ? (size_t)s * batch * (size_t)M * N * sizeof(double2) : 0;
}

ptn_status zgemm(const GemmArgs& g, void* ws, size_t ws_bytes, cudaStream_t st) {
  const int oa = op_code(g.opA), ob = op_code(g.opB);
  PTN_CHECK_ARG(oa >= 0 && ob >= 0, "zgemm: bad op (%c, %c)", g.opA, g.opB);
  PTN_CHECK_ARG(g.M >= 0 && g.N >= 0 && g.K >= 0 && g.batch >= 1, "zgemm: bad sizes");
  if (g.M == 0 || g.N == 0) return PTN_OK;
  KArgs k;
  k.M = g.M; k.N = g.N; k.K = g.K; k.batch = g.batch;
  k.alpha = g.alpha; k.beta = g.beta;
  k.A = g.A; k.lda = g.lda; k.sA = g.sA;
  k.B = g.B; k.ldb = g.ldb; k.sB = g.sB;
  k.C = g.C; k.ldc = g.ldc; k.sC = g.sC;
  k.skip = g.skip;
  int splits = choose_splits(g.M, g.N, g.K, g.batch);
  while (splits > 1 && (size_t)splits * g.batch * (size_t)g.M * g.N * sizeof(double2) > ws_bytes)
    splits /= 2;
  if (splits < 1) splits = 1;
  k.splits = splits;
  k.kchunk = ((g.K + splits - 1) / splits + BK - 1) / BK * BK;
  if (k.kchunk == 0) k.kchunk = BK;
  k.part = splits > 1 ? static_cast<double2*>(ws) : nullptr;
  dim3 grid((g.N + BN - 1) / BN, (g.M + BM - 1) / BM, g.batch * splits);
  PTN_CHECK_ARG(grid.y <= 65535 && grid.z <= 65535, "zgemm: grid too large");
  const int prof = prof_begin(st, PROF_ZGEMM_F64, 8.0 * g.M * g.N * (double)g.K * g.batch,
                              16.0 * g.batch * ((double)g.M * g.K + (double)g.K * g.N + 2.0 * g.M * g.N));
  switch (oa) {
    case OP_N: launch_b<OP_N>(ob, grid, st, k); break;
    case OP_T: launch_b<OP_T>(ob, grid, st, k); break;
    case OP_C: launch_b<OP_C>(ob, grid, st, k); break;
    default:   launch_b<OP_H>(ob, grid, st, k); break;
  }
  PTN_LAUNCH_CHECK();
  note_launches(1);
  if (splits > 1) {
    const long total = (long)g.batch * g.M * g.N;
    const int blocks = (int)std::min<long>((total + 255) / 256, 4L * num_sms());
    splitk_reduce_kernel<<<blocks, 256, 0, st>>>(k);
    PTN_LAUNCH_CHECK();
    note_launches(1);
  }
  prof_end(st, prof);
  return PTN_OK;
}

}  // namespace ptn

extern "C" {

size_t ptn_zgemm_workspace_bytes(int M, int N, int K, int batch) {
  return ptn::zgemm_workspace_bytes(M, N, K, batch);
}

ptn_status ptn_zgemm(char opA, char opB, int M, int N, int K, ptn_c128 alpha, const ptn_c128* A,
                     long lda, long strideA, const ptn_c128* B, long ldb, long strideB,
                     ptn_c128 beta, ptn_c128* C, long ldc, long strideC, int batch, void* ws,
                     size_t ws_bytes, void* stream) {
  ptn::GemmArgs g;
  g.M = M; g.N = N; g.K = K; g.opA = opA; g.opB = opB;
  g.alpha = make_double2(alpha.re, alpha.im);
  g.beta = make_double2(beta.re, beta.im);
  g.A = reinterpret_cast<const double2*>(A); g.lda = lda; g.sA = strideA;
  g.B = reinterpret_cast<const double2*>(B); g.ldb = ldb; g.sB = strideB;
  g.C = reinterpret_cast<double2*>(C); g.ldc = ldc; g.sC = strideC;
  g.batch = batch; g.skip = nullptr;
  return ptn::zgemm(g, ws, ws_bytes, ptn::as_stream(stream));
}

}  // extern "C"
