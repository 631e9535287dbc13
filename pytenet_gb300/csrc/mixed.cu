// Mixed-precision form of the site / bond operators and of the environment steps
// (pytenet/chain_ops.py:16-99, 237-317): the two GEMMs of every contraction run
// on the tensor cores as split-BF16 products (tc_gemm.cu); the MPO stage, all
// intermediate sums of the split-K partials and everything outside the
// contractions stay in FP64.
//
// Data flow of H_eff . x (site tensors (Dl, d, Dr), MPO bonds cl / cr):
//   prepare (once per local step):  R -> Rt  (plain slices, rows (wr, r2), K = r0)
//                                   L -> Le  (embedded slices, n = l2, K = (l0, wl))
//   apply:  x -> Xe (embedded, n = (l0, t), K = r0)
//           GEMM 1: T1^T[(wr,r2)][(l0,t)] = Rt . Xe^T, written as T1[(l0,t)][(wr,r2)] (FP64)
//           MPO stage: T2[l0,(wl,s),r2] from T1 and W, written straight into the plain
//                      slices of GEMM 2's A operand, rows (s, r2), K = (l0, wl)
//           GEMM 2: out^T[(s,r2)][l2] = T2s . Le^T, written as out[l2][(s,r2)] (FP64)
// Every GEMM computes the transpose of the wanted product so that the epilogue
// thread of output row m writes consecutive addresses with its neighbours.
#include "ptn_common.cuh"
#include <cuda_bf16.h>
#include <algorithm>

namespace ptn {

void note_launches(int n);
ptn_status tc_gemm(const void* Aslices, long aplane, const void* Bslices, long bplane, int M,
                   int Nc, int Kc, long Kp, double2* out, long ldm, long ldn, bool accumulate,
                   void* ws, size_t ws_bytes, const int* skip, cudaStream_t st);
size_t tc_gemm_workspace_bytes(int M, int Ncomplex, int Kcomplex);

namespace {

typedef __nv_bfloat16 bf16;

__device__ __forceinline__ void split3(double x, bf16& a, bf16& b, bf16& c) {
  a = __double2bfloat16(x);
  double r = x - (double)__bfloat162float(a);
  b = __double2bfloat16(r);
  r -= (double)__bfloat162float(b);
  c = __double2bfloat16(r);
}

// write complex z into the plain slices at (row, complex column kc)
__device__ __forceinline__ void put_plain(bf16* dst, long Kp, long plane, long row, long kc,
                                          double2 z) {
  bf16 r0, r1, r2, i0, i1, i2;
  split3(z.x, r0, r1, r2);
  split3(z.y, i0, i1, i2);
  __nv_bfloat162* p = reinterpret_cast<__nv_bfloat162*>(dst + row * Kp + 2 * kc);
  p[0] = __halves2bfloat162(r0, i0);
  reinterpret_cast<__nv_bfloat162*>(dst + plane + row * Kp + 2 * kc)[0] = __halves2bfloat162(r1, i1);
  reinterpret_cast<__nv_bfloat162*>(dst + 2 * plane + row * Kp + 2 * kc)[0] =
      __halves2bfloat162(r2, i2);
}

// write complex z as the 2x2 block [[Re, -Im], [Im, Re]] at rows 2n, 2n+1, cols 2k, 2k+1
__device__ __forceinline__ void put_embed(bf16* dst, long Kp, long plane, long n, long k,
                                          double2 z) {
  bf16 r[3], i[3];
  split3(z.x, r[0], r[1], r[2]);
  split3(z.y, i[0], i[1], i[2]);
#pragma unroll
  for (int s = 0; s < 3; ++s) {
    bf16* base = dst + s * plane;
    reinterpret_cast<__nv_bfloat162*>(base + (2 * n) * Kp + 2 * k)[0] =
        __halves2bfloat162(r[s], __hneg(i[s]));
    reinterpret_cast<__nv_bfloat162*>(base + (2 * n + 1) * Kp + 2 * k)[0] =
        __halves2bfloat162(i[s], r[s]);
  }
}

__global__ void split_plain_kernel(const double2* __restrict__ src, long sm, long sk, int M, int K,
                                   int conj, bf16* __restrict__ dst, long Kp, long plane,
                                   const int* skip) {
  if (skip != nullptr && *skip != 0) return;
  const long total = (long)M * K;
  for (long idx = blockIdx.x * (long)blockDim.x + threadIdx.x; idx < total;
       idx += (long)gridDim.x * blockDim.x) {
    long m, k;
    if (sk == 1) { m = idx / K; k = idx % K; }      // read along k
    else         { k = idx / M; m = idx % M; }      // read along m (transposed source)
    double2 z = src[m * sm + k * sk];
    if (conj) z.y = -z.y;
    put_plain(dst, Kp, plane, m, k, z);
  }
}

__global__ void split_embed_kernel(const double2* __restrict__ src, long sn, long sk, int N, int K,
                                   int conj, bf16* __restrict__ dst, long Kp, long plane,
                                   const int* skip) {
  if (skip != nullptr && *skip != 0) return;
  const long total = (long)N * K;
  for (long idx = blockIdx.x * (long)blockDim.x + threadIdx.x; idx < total;
       idx += (long)gridDim.x * blockDim.x) {
    long n, k;
    if (sk == 1) { n = idx / K; k = idx % K; }
    else         { k = idx / N; n = idx % N; }
    double2 z = src[n * sn + k * sk];
    if (conj) z.y = -z.y;
    put_embed(dst, Kp, plane, n, k, z);
  }
}

// Output placement of the MPO stage: q = qa * Qb + qb,
// row  = x*Rx + qa*Rqa + qb*Rqb + y*Ry,  col = x*Cx + qa*Cqa + qb*Cqb + y*Cy
struct StageOut {
  bf16* dst;
  long Kp, plane;
  int embedded;
  int Qb;
  long Rx, Rqa, Rqb, Ry, Cx, Cqa, Cqb, Cy;
};

// out[x, q, y] = sum_p M[q, p] in[x, p, y] (M from w with strides ldq, ldp), written
// as BF16 slices. Same blocking as the FP64 stage: 128 consecutive y per CTA.
__global__ void mpo_stage_split_kernel(const double2* __restrict__ in,
                                       const double2* __restrict__ w, long ldq, long ldp, int X,
                                       int P, int Q, int Y, StageOut o, const int* skip) {
  if (skip != nullptr && *skip != 0) return;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  double2* sin = reinterpret_cast<double2*>(smem_raw);
  double2* sval = sin + (size_t)P * 128;
  int* sidx = reinterpret_cast<int*>(sval + (size_t)P * Q);
  __shared__ int qstart[65];
  const int x = blockIdx.y;
  const int ty = threadIdx.x;
  const int y = blockIdx.x * 128 + ty;
  if (threadIdx.x == 0) {
    int nz = 0;
    for (int q = 0; q < Q; ++q) {
      qstart[q] = nz;
      for (int p = 0; p < P; ++p) {
        const double2 v = w[q * ldq + p * ldp];
        if (v.x != 0.0 || v.y != 0.0) {
          sval[nz] = v;
          sidx[nz] = p;
          ++nz;
        }
      }
    }
    qstart[Q] = nz;
  }
  for (int p = 0; p < P; ++p)
    sin[p * 128 + ty] = (y < Y) ? in[((long)x * P + p) * Y + y] : make_double2(0.0, 0.0);
  __syncthreads();
  if (y >= Y) return;
  for (int q = 0; q < Q; ++q) {
    double2 acc = make_double2(0.0, 0.0);
    for (int e = qstart[q]; e < qstart[q + 1]; ++e) acc = cfma(sval[e], sin[sidx[e] * 128 + ty], acc);
    const int qa = q / o.Qb, qb = q % o.Qb;
    const long row = x * o.Rx + qa * o.Rqa + qb * o.Rqb + (long)y * o.Ry;
    const long col = x * o.Cx + qa * o.Cqa + qb * o.Cqb + (long)y * o.Cy;
    if (o.embedded) put_embed(o.dst, o.Kp, o.plane, row, col, acc);
    else put_plain(o.dst, o.Kp, o.plane, row, col, acc);
  }
}

int grid_for(long n) {
  long b = (n + 255) / 256;
  return (int)std::max(1L, std::min(b, 16L * num_sms()));
}

inline long kpad(long kc) { return (2 * kc + 63) / 64 * 64; }
inline size_t al(size_t b) { return (b + 255) & ~size_t(255); }

// bump allocator over the caller's workspace (null base: size query)
struct Carver {
  char* base;
  size_t off = 0;
  explicit Carver(void* b) : base(static_cast<char*>(b)) {}
  void* take(size_t bytes) {
    void* p = base ? base + off : nullptr;
    off += al(bytes);
    return p;
  }
};

// BF16 slice buffer: 3 planes of rows x Kp
struct Slices {
  bf16* p;
  long rows, kc, Kp;
  long plane() const { return rows * Kp; }
};

Slices take_slices(Carver& c, long rows, long kc) {
  Slices s;
  s.rows = rows;
  s.kc = kc;
  s.Kp = kpad(kc);
  s.p = static_cast<bf16*>(c.take((size_t)3 * rows * s.Kp * sizeof(bf16)));
  return s;
}

ptn_status plain(const double2* src, long sm, long sk, const Slices& d, bool conj, const int* skip,
                 cudaStream_t st) {
  split_plain_kernel<<<grid_for(d.rows * d.kc), 256, 0, st>>>(src, sm, sk, (int)d.rows, (int)d.kc,
                                                              conj ? 1 : 0, d.p, d.Kp, d.plane(),
                                                              skip);
  PTN_LAUNCH_CHECK();
  note_launches(1);
  return PTN_OK;
}

// embedded slices of an N x K complex matrix (2N rows)
ptn_status embed(const double2* src, long sn, long sk, long N, const Slices& d, bool conj,
                 const int* skip, cudaStream_t st) {
  split_embed_kernel<<<grid_for(N * d.kc), 256, 0, st>>>(src, sn, sk, (int)N, (int)d.kc,
                                                         conj ? 1 : 0, d.p, d.Kp, d.plane(), skip);
  PTN_LAUNCH_CHECK();
  note_launches(1);
  return PTN_OK;
}

ptn_status stage(const double2* in, const double2* w, long ldq, long ldp, int X, int P, int Q,
                 int Y, const StageOut& o, const int* skip, cudaStream_t st) {
  PTN_CHECK_ARG(P <= 64 && Q <= 64, "MPO stage: chi*d must be <= 64");
  const size_t smem = (size_t)P * 128 * sizeof(double2) + (size_t)P * Q * (sizeof(double2) + sizeof(int));
  static bool attr = false;
  if (!attr) {
    PTN_CUDA_TRY(cudaFuncSetAttribute(mpo_stage_split_kernel,
                                      cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      64 * 128 * 16 + 64 * 64 * 20));
    attr = true;
  }
  PTN_CHECK_ARG(X <= 65535, "MPO stage: X too large");
  mpo_stage_split_kernel<<<dim3((Y + 127) / 128, X), 128, smem, st>>>(in, w, ldq, ldp, X, P, Q, Y,
                                                                       o, skip);
  PTN_LAUNCH_CHECK();
  note_launches(1);
  return PTN_OK;
}

ptn_status gemm(const Slices& A, const Slices& Be, int M, int Nc, int Kc, double2* out, long ldm,
                long ldn, void* ws, size_t ws_bytes, const int* skip, cudaStream_t st) {
  return tc_gemm(A.p, A.plane(), Be.p, Be.plane(), M, Nc, Kc, A.Kp, out, ldm, ldn, false, ws,
                 ws_bytes, skip, st);
}

// ---------------------------------------------------------------- H_eff (site)
struct HeffWs {
  Slices Rt, Le, Xe, T2s;
  double2* T1;
  void* gws;
  size_t gbytes;
};

HeffWs heff_ws(Carver& c, int Dl, int d, int Dr, int cl, int cr) {
  HeffWs w;
  w.Rt = take_slices(c, (long)cr * Dr, Dr);
  w.Le = take_slices(c, 2L * Dl, (long)Dl * cl);
  w.Xe = take_slices(c, 2L * Dl * d, Dr);
  w.T2s = take_slices(c, (long)d * Dr, (long)Dl * cl);
  w.T1 = static_cast<double2*>(c.take((size_t)Dl * d * cr * Dr * sizeof(double2)));
  w.gbytes = std::max(tc_gemm_workspace_bytes(cr * Dr, Dl * d, Dr),
                      tc_gemm_workspace_bytes(d * Dr, Dl, Dl * cl));
  w.gws = c.take(w.gbytes);
  return w;
}

// ---------------------------------------------------------------- zero-site (bond)
struct BondWs {
  Slices Rt, Le, Xe, T1s;
  double2* T1;
  void* gws;
  size_t gbytes;
};

BondWs bond_ws(Carver& c, int Dl, int Dr, int chi) {
  BondWs w;
  w.Rt = take_slices(c, (long)chi * Dr, Dr);
  w.Le = take_slices(c, 2L * Dl, (long)Dl * chi);
  w.Xe = take_slices(c, 2L * Dl, Dr);
  w.T1s = take_slices(c, Dr, (long)Dl * chi);
  w.T1 = static_cast<double2*>(c.take((size_t)Dl * chi * Dr * sizeof(double2)));
  w.gbytes = std::max(tc_gemm_workspace_bytes(chi * Dr, Dl, Dr),
                      tc_gemm_workspace_bytes(Dr, Dl, Dl * chi));
  w.gws = c.take(w.gbytes);
  return w;
}

// ---------------------------------------------------------------- environments
struct EnvWs {
  Slices S1, E1, S2, E2;
  double2* T1;
  void* gws;
  size_t gbytes;
};

EnvWs env_left_ws(Carver& c, int Dl, int d, int Dr, int cl, int cr) {
  EnvWs w;
  w.S1 = take_slices(c, (long)d * Dr, Dl);              // conj(B)^T plain, rows (t, rb), K = l2
  w.E1 = take_slices(c, 2L * Dl * cl, Dl);              // L embedded, n = (l0, wl), K = l2
  w.S2 = take_slices(c, (long)cr * Dr, (long)Dl * d);   // T2^T plain, rows (wr, rb), K = (l0, s)
  w.E2 = take_slices(c, 2L * Dr, (long)Dl * d);         // A embedded, n = ra, K = (l0, s)
  w.T1 = static_cast<double2*>(c.take((size_t)Dl * cl * d * Dr * sizeof(double2)));
  w.gbytes = std::max(tc_gemm_workspace_bytes(d * Dr, Dl * cl, Dl),
                      tc_gemm_workspace_bytes(cr * Dr, Dr, Dl * d));
  w.gws = c.take(w.gbytes);
  return w;
}

EnvWs env_right_ws(Carver& c, int Dl, int d, int Dr, int cl, int cr) {
  EnvWs w;
  w.S1 = take_slices(c, (long)cr * Dr, Dr);             // R^T plain, rows (wr, r2), K = r0
  w.E1 = take_slices(c, 2L * Dl * d, Dr);               // A embedded, n = (l0, s), K = r0
  w.S2 = take_slices(c, Dl, (long)d * Dr);              // conj(B) plain, rows lb, K = (t, r2)
  w.E2 = take_slices(c, 2L * Dl * cl, (long)d * Dr);    // T2 embedded, n = (l0, wl), K = (t, r2)
  w.T1 = static_cast<double2*>(c.take((size_t)Dl * d * cr * Dr * sizeof(double2)));
  w.gbytes = std::max(tc_gemm_workspace_bytes(cr * Dr, Dl * d, Dr),
                      tc_gemm_workspace_bytes(Dl, Dl * cl, d * Dr));
  w.gws = c.take(w.gbytes);
  return w;
}

}  // namespace

// ================================================================ site operator
size_t heff_workspace_bytes_mixed(int Dl, int d, int Dr, int chil, int chir) {
  Carver c(nullptr);
  heff_ws(c, Dl, d, Dr, chil, chir);
  return c.off;
}

ptn_status heff_prepare_mixed(const double2* w, const double2* l, const double2* r, int Dl, int d,
                              int Dr, int chil, int chir, void* ws, size_t ws_bytes,
                              cudaStream_t st) {
  (void)w;
  PTN_CHECK_ARG(ws_bytes >= heff_workspace_bytes_mixed(Dl, d, Dr, chil, chir),
                "mixed heff: workspace too small");
  Carver c(ws);
  HeffWs h = heff_ws(c, Dl, d, Dr, chil, chir);
  // Rt[(wr, r2)][r0] = R[r0][(wr, r2)]
  PTN_TRY(plain(r, 1, (long)chir * Dr, h.Rt, false, nullptr, st));
  // Le: element (n = l2, k = (l0, wl)) = L[(l0, wl)][l2]
  PTN_TRY(embed(l, 1, Dl, Dl, h.Le, false, nullptr, st));
  return PTN_OK;
}

ptn_status heff_apply_mixed(const double2* x, double2* y, const double2* w, int Dl, int d, int Dr,
                            int chil, int chir, void* ws, size_t ws_bytes, const int* skip,
                            cudaStream_t st) {
  (void)ws_bytes;
  Carver c(ws);
  HeffWs h = heff_ws(c, Dl, d, Dr, chil, chir);
  // Xe: element (n = (l0, t), k = r0) = x[(l0, t)][r0]
  PTN_TRY(embed(x, Dr, 1, (long)Dl * d, h.Xe, false, skip, st));
  // T1[(l0,t)][(wr,r2)] via T1^T = Rt . Xe^T   (M = chir*Dr, N = Dl*d, K = Dr)
  PTN_TRY(gemm(h.Rt, h.Xe, chir * Dr, Dl * d, Dr, h.T1, 1, (long)chir * Dr, h.gws, h.gbytes, skip,
               st));
  // T2[l0, (wl, s), r2] -> plain slices rows (s, r2), K = (l0, wl)
  StageOut o;
  o.dst = h.T2s.p; o.Kp = h.T2s.Kp; o.plane = h.T2s.plane(); o.embedded = 0; o.Qb = d;
  o.Rx = 0; o.Rqa = 0; o.Rqb = Dr; o.Ry = 1;
  o.Cx = chil; o.Cqa = 1; o.Cqb = 0; o.Cy = 0;
  PTN_TRY(stage(h.T1, w, (long)d * chir, 1, Dl, d * chir, chil * d, Dr, o, skip, st));
  // out^T[(s, r2)][l2] = T2s . Le^T  (M = d*Dr, N = Dl, K = Dl*chil) -> out[l2][(s, r2)]
  PTN_TRY(gemm(h.T2s, h.Le, d * Dr, Dl, Dl * chil, y, 1, (long)d * Dr, h.gws, h.gbytes, skip, st));
  return PTN_OK;
}

ptn_status heff_apply_mixed_entry(const double2* a, const double2* w, const double2* l,
                                  const double2* r, double2* out, int Dl, int d, int Dr, int chil,
                                  int chir, void* ws, size_t ws_bytes, cudaStream_t st) {
  PTN_TRY(heff_prepare_mixed(w, l, r, Dl, d, Dr, chil, chir, ws, ws_bytes, st));
  return heff_apply_mixed(a, out, w, Dl, d, Dr, chil, chir, ws, ws_bytes, nullptr, st);
}

// ================================================================ bond operator
size_t bond_workspace_bytes_mixed(int Dl, int Dr, int chi) {
  Carver c(nullptr);
  bond_ws(c, Dl, Dr, chi);
  return c.off;
}

ptn_status bond_prepare_mixed(const double2* l, const double2* r, int Dl, int Dr, int chi, void* ws,
                              size_t ws_bytes, cudaStream_t st) {
  PTN_CHECK_ARG(ws_bytes >= bond_workspace_bytes_mixed(Dl, Dr, chi), "mixed bond: workspace too small");
  Carver c(ws);
  BondWs b = bond_ws(c, Dl, Dr, chi);
  PTN_TRY(plain(r, 1, (long)chi * Dr, b.Rt, false, nullptr, st));
  PTN_TRY(embed(l, 1, Dl, Dl, b.Le, false, nullptr, st));
  return PTN_OK;
}

ptn_status bond_apply_mixed(const double2* x, double2* y, int Dl, int Dr, int chi, void* ws,
                            size_t ws_bytes, const int* skip, cudaStream_t st) {
  (void)ws_bytes;
  Carver c(ws);
  BondWs b = bond_ws(c, Dl, Dr, chi);
  // Xe: element (n = l0, k = r0) = C[l0][r0]
  PTN_TRY(embed(x, Dr, 1, Dl, b.Xe, false, skip, st));
  // T1[l0][(w, r2)] via T1^T = Rt . Xe^T  (M = chi*Dr, N = Dl, K = Dr)
  PTN_TRY(gemm(b.Rt, b.Xe, chi * Dr, Dl, Dr, b.T1, 1, (long)chi * Dr, b.gws, b.gbytes, skip, st));
  // T1s: element (m = r2, k = (l0, w)) = T1[(l0, w)][r2]
  PTN_TRY(plain(b.T1, 1, Dr, b.T1s, false, skip, st));
  // out^T[r2][l2] = T1s . Le^T  (M = Dr, N = Dl, K = Dl*chi) -> out[l2][r2]
  PTN_TRY(gemm(b.T1s, b.Le, Dr, Dl, Dl * chi, y, 1, Dr, b.gws, b.gbytes, skip, st));
  return PTN_OK;
}

ptn_status bond_apply_mixed_entry(const double2* cm, const double2* l, const double2* r,
                                  double2* out, int Dl, int Dr, int chi, void* ws, size_t ws_bytes,
                                  cudaStream_t st) {
  PTN_TRY(bond_prepare_mixed(l, r, Dl, Dr, chi, ws, ws_bytes, st));
  return bond_apply_mixed(cm, out, Dl, Dr, chi, ws, ws_bytes, nullptr, st);
}

// ================================================================ environments
size_t env_workspace_bytes_mixed(int Dl, int d, int Dr, int cl, int cr) {
  Carver a(nullptr), b(nullptr);
  env_left_ws(a, Dl, d, Dr, cl, cr);
  env_right_ws(b, Dl, d, Dr, cl, cr);
  return std::max(a.off, b.off);
}

// l_next[ra, wr, rb] = sum A[l0,s,ra] W[wl,t,s,wr] L[l0,wl,l2] conj(B[l2,t,rb])
ptn_status env_left_mixed(const double2* a, const double2* b, const double2* w, const double2* l,
                          double2* lnext, int Dl, int d, int Dr, int cl, int cr, void* ws,
                          size_t ws_bytes, cudaStream_t st) {
  PTN_CHECK_ARG(ws_bytes >= env_workspace_bytes_mixed(Dl, d, Dr, cl, cr), "mixed env: workspace too small");
  Carver c(ws);
  EnvWs e = env_left_ws(c, Dl, d, Dr, cl, cr);
  // S1: element (m = (t, rb), k = l2) = conj(B[l2][(t, rb)])
  PTN_TRY(plain(b, 1, (long)d * Dr, e.S1, true, nullptr, st));
  // E1: element (n = (l0, wl), k = l2) = L[(l0, wl)][l2]
  PTN_TRY(embed(l, Dl, 1, (long)Dl * cl, e.E1, false, nullptr, st));
  // T1^T[(t, rb)][(l0, wl)] -> T1[(l0, wl)][(t, rb)]  (M = d*Dr, N = Dl*cl, K = Dl)
  PTN_TRY(gemm(e.S1, e.E1, d * Dr, Dl * cl, Dl, e.T1, 1, (long)d * Dr, e.gws, e.gbytes, nullptr, st));
  // T2[l0, (s, wr), rb] -> plain slices rows (wr, rb), K = (l0, s)
  StageOut o;
  o.dst = e.S2.p; o.Kp = e.S2.Kp; o.plane = e.S2.plane(); o.embedded = 0; o.Qb = cr;
  o.Rx = 0; o.Rqa = 0; o.Rqb = Dr; o.Ry = 1;
  o.Cx = d; o.Cqa = 1; o.Cqb = 0; o.Cy = 0;
  PTN_TRY(stage(e.T1, w, 1, (long)d * cr, Dl, cl * d, d * cr, Dr, o, nullptr, st));
  // E2: element (n = ra, k = (l0, s)) = A[(l0, s)][ra]
  PTN_TRY(embed(a, 1, Dr, Dr, e.E2, false, nullptr, st));
  // l_next^T[(wr, rb)][ra] = S2 . E2^T  (M = cr*Dr, N = Dr, K = Dl*d) -> l_next[ra][(wr, rb)]
  PTN_TRY(gemm(e.S2, e.E2, cr * Dr, Dr, Dl * d, lnext, 1, (long)cr * Dr, e.gws, e.gbytes, nullptr, st));
  return PTN_OK;
}

// r_next[la, wl, lb] = sum A[la,s,r0] W[wl,t,s,wr] R[r0,wr,r2] conj(B[lb,t,r2])
ptn_status env_right_mixed(const double2* a, const double2* b, const double2* w, const double2* r,
                           double2* rnext, int Dl, int d, int Dr, int cl, int cr, void* ws,
                           size_t ws_bytes, cudaStream_t st) {
  PTN_CHECK_ARG(ws_bytes >= env_workspace_bytes_mixed(Dl, d, Dr, cl, cr), "mixed env: workspace too small");
  Carver c(ws);
  EnvWs e = env_right_ws(c, Dl, d, Dr, cl, cr);
  PTN_TRY(plain(r, 1, (long)cr * Dr, e.S1, false, nullptr, st));
  PTN_TRY(embed(a, Dr, 1, (long)Dl * d, e.E1, false, nullptr, st));
  // T1^T[(wr, r2)][(l0, s)] -> T1[(l0, s)][(wr, r2)]  (M = cr*Dr, N = Dl*d, K = Dr)
  PTN_TRY(gemm(e.S1, e.E1, cr * Dr, Dl * d, Dr, e.T1, 1, (long)cr * Dr, e.gws, e.gbytes, nullptr, st));
  // T2[l0, (wl, t), r2] -> embedded slices n = (l0, wl), K = (t, r2)
  StageOut o;
  o.dst = e.E2.p; o.Kp = e.E2.Kp; o.plane = e.E2.plane(); o.embedded = 1; o.Qb = d;
  o.Rx = cl; o.Rqa = 1; o.Rqb = 0; o.Ry = 0;
  o.Cx = 0; o.Cqa = 0; o.Cqb = Dr; o.Cy = 1;
  PTN_TRY(stage(e.T1, w, (long)d * cr, 1, Dl, d * cr, cl * d, Dr, o, nullptr, st));
  // S2: element (m = lb, k = (t, r2)) = conj(B[lb][(t, r2)])
  PTN_TRY(plain(b, (long)d * Dr, 1, e.S2, true, nullptr, st));
  // r_next^T[lb][(l0, wl)] = S2 . E2^T  (M = Dl, N = Dl*cl, K = d*Dr) -> r_next[(l0, wl)][lb]
  PTN_TRY(gemm(e.S2, e.E2, Dl, Dl * cl, d * Dr, rnext, 1, Dl, e.gws, e.gbytes, nullptr, st));
  return PTN_OK;
}

// ================================================================ plain GEMM entry
size_t zgemm_split_workspace_bytes(int M, int N, int K) {
  Carver c(nullptr);
  take_slices(c, M, K);
  take_slices(c, 2L * N, K);
  c.take(tc_gemm_workspace_bytes(M, N, K));
  return c.off;
}

// C = A B (row-major complex, M x K times K x N) through split-BF16 tensor-core products
ptn_status zgemm_split(const double2* A, long lda, const double2* B, long ldb, double2* C, long ldc,
                       int M, int N, int K, void* ws, size_t ws_bytes, cudaStream_t st) {
  PTN_CHECK_ARG(M > 0 && N > 0 && K > 0, "zgemm_split: bad sizes");
  PTN_CHECK_ARG(ws_bytes >= zgemm_split_workspace_bytes(M, N, K), "zgemm_split: workspace too small");
  Carver c(ws);
  Slices As = take_slices(c, M, K);
  Slices Bs = take_slices(c, 2L * N, K);
  const size_t gb = tc_gemm_workspace_bytes(M, N, K);
  void* g = c.take(gb);
  PTN_TRY(plain(A, lda, 1, As, false, nullptr, st));
  PTN_TRY(embed(B, 1, ldb, N, Bs, false, nullptr, st));
  return gemm(As, Bs, M, N, K, C, ldc, 1, g, gb, nullptr, st);
}

}  // namespace ptn

extern "C" {

size_t ptn_zgemm_split_bf16_workspace_bytes(int M, int N, int K) {
  return ptn::zgemm_split_workspace_bytes(M, N, K);
}

ptn_status ptn_zgemm_split_bf16(const ptn_c128* A, long lda, const ptn_c128* B, long ldb,
                                ptn_c128* C, long ldc, int M, int N, int K, void* ws,
                                size_t ws_bytes, void* stream) {
  return ptn::zgemm_split(reinterpret_cast<const double2*>(A), lda,
                          reinterpret_cast<const double2*>(B), ldb, reinterpret_cast<double2*>(C),
                          ldc, M, N, K, ws, ws_bytes, ptn::as_stream(stream));
}

int ptn_tc_error(void) {
  extern int tc_gemm_error_and_reset_c(void);
  return tc_gemm_error_and_reset_c();
}

}  // extern "C"
