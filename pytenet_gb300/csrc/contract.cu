// Chain contractions of the single-site sweep (pytenet/chain_ops.py), plain FP64 form.
//
// Each contraction is two complex GEMMs around a small "MPO stage" that mixes the
// (physical, MPO-bond) index pairs with W:
//
//   H_eff.A   (chain_ops.py:237-279)
//     T1[(l0,t),(wr,r2)] = A[(l0,t),r0] R[r0,(wr,r2)]            GEMM  M=Dl*d  N=chir*Dr K=Dr
//     T2[l0,(wl,s),r2]   = sum_(t,wr) W[(wl,s),(t,wr)] T1[l0,(t,wr),r2]   MPO stage
//     out[l2,(s,r2)]     = sum_(l0,wl) L[(l0,wl),l2] T2[(l0,wl),(s,r2)]   GEMM  op(A)=L^T
//   zero-site  (chain_ops.py:282-317): T1 = C R, out = L^T T1
//   env left   (chain_ops.py:60-99):   T1 = L conj(B), MPO stage with W^T, l_next = A^T T2
//   env right  (chain_ops.py:16-57):   T1 = A R, MPO stage with W, r_next = T2 B^H
//
// The MPO stage is HBM-bound (it reads and writes the d*chi-times larger
// intermediate once) and skips the zero entries of W, which for the XXZ MPO are
// ~90% of the (chi d)^2 matrix.
#include "ptn_common.cuh"
#include <algorithm>

namespace ptn {

void note_launches(int n);

namespace {

// out[x, q, y] = sum_p M[q, p] in[x, p, y]; M given by (ldq, ldp) strides into w.
// One CTA per (x, 128-wide y chunk); the nonzeros of M are compacted into shared
// memory first, the P input rows of the chunk are staged in shared memory.
__global__ void mpo_stage_kernel(const double2* __restrict__ in, double2* __restrict__ out,
                                 const double2* __restrict__ w, long ldq, long ldp, int X, int P,
                                 int Q, int Y, const int* skip) {
  if (skip != nullptr && *skip != 0) return;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  double2* sin = reinterpret_cast<double2*>(smem_raw);             // [P][128]
  double2* sval = sin + (size_t)P * 128;                            // [P*Q] nonzero values
  int* sidx = reinterpret_cast<int*>(sval + (size_t)P * Q);         // [P*Q] their p index
  __shared__ int snnz;
  __shared__ int qstart[65];

  const int x = blockIdx.y;
  const int y0 = blockIdx.x * 128;
  const int ty = threadIdx.x;   // 128 threads

  // compact the nonzeros of M in row-major (q, p) order (deterministic: one thread)
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
    snnz = nz;
  }
  const int y = y0 + ty;
  for (int p = 0; p < P; ++p)
    sin[p * 128 + ty] = (y < Y) ? in[((long)x * P + p) * Y + y] : make_double2(0.0, 0.0);
  __syncthreads();
  if (y >= Y) return;
  for (int q = 0; q < Q; ++q) {
    double2 acc = make_double2(0.0, 0.0);
    for (int e = qstart[q]; e < qstart[q + 1]; ++e) acc = cfma(sval[e], sin[sidx[e] * 128 + ty], acc);
    out[((long)x * Q + q) * Y + y] = acc;
  }
}

ptn_status mpo_stage(const double2* in, double2* out, const double2* w, long ldq, long ldp, int X,
                     int P, int Q, int Y, const int* skip, cudaStream_t st) {
  PTN_CHECK_ARG(P <= 64 && Q <= 64, "MPO stage: chi*d must be <= 64 (got %d, %d)", P, Q);
  if (X == 0 || Y == 0) return PTN_OK;
  const size_t smem = (size_t)P * 128 * sizeof(double2) + (size_t)P * Q * (sizeof(double2) + sizeof(int));
  static bool attr_done = false;
  if (!attr_done) {
    PTN_CUDA_TRY(cudaFuncSetAttribute(mpo_stage_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      64 * 128 * 16 + 64 * 64 * 20));
    attr_done = true;
  }
  dim3 grid((Y + 127) / 128, X);
  PTN_CHECK_ARG(X <= 65535, "MPO stage: X too large");
  mpo_stage_kernel<<<grid, 128, smem, st>>>(in, out, w, ldq, ldp, X, P, Q, Y, skip);
  PTN_LAUNCH_CHECK();
  note_launches(1);
  return PTN_OK;
}

}  // namespace

ptn_status mpo_stage_f64(const double2* in, double2* out, const double2* w, long ldq, long ldp, int X,
                         int P, int Q, int Y, const int* skip, cudaStream_t st) {
  return mpo_stage(in, out, w, ldq, ldp, X, P, Q, Y, skip, st);
}

namespace {

inline size_t align256(size_t b) { return (b + 255) & ~size_t(255); }

GemmArgs gemm_args(char oa, char ob, int M, int N, int K, const double2* A, long lda,
                   const double2* B, long ldb, double2* C, long ldc, const int* skip) {
  GemmArgs g;
  g.M = M; g.N = N; g.K = K; g.opA = oa; g.opB = ob;
  g.alpha = make_double2(1.0, 0.0); g.beta = make_double2(0.0, 0.0);
  g.A = A; g.lda = lda; g.sA = 0;
  g.B = B; g.ldb = ldb; g.sB = 0;
  g.C = C; g.ldc = ldc; g.sC = 0;
  g.batch = 1; g.skip = skip;
  return g;
}

}  // namespace

// ------------------------------------------------------------------ workspace layout
// [T1 | T2 | split-K partials]
struct ContractWs {
  double2* t1;
  double2* t2;
  void* gemm_ws;
  size_t gemm_bytes;
};

static size_t heff_t_elems(int Dl, int d, int Dr, int chil, int chir) {
  return (size_t)Dl * std::max(d * chir, chil * d) * Dr;
}

static size_t heff_gemm_ws(int Dl, int d, int Dr, int chil, int chir) {
  return std::max(zgemm_workspace_bytes(Dl * d, chir * Dr, Dr, 1),
                  zgemm_workspace_bytes(Dl, d * Dr, Dl * chil, 1));
}

size_t heff_workspace_bytes_f64(int Dl, int d, int Dr, int chil, int chir) {
  const size_t t = align256(heff_t_elems(Dl, d, Dr, chil, chir) * sizeof(double2));
  return 2 * t + align256(heff_gemm_ws(Dl, d, Dr, chil, chir));
}

static ContractWs carve(void* ws, size_t t_elems, size_t ws_bytes) {
  ContractWs c;
  char* p = static_cast<char*>(ws);
  const size_t t = align256(t_elems * sizeof(double2));
  c.t1 = reinterpret_cast<double2*>(p);
  c.t2 = reinterpret_cast<double2*>(p + t);
  c.gemm_ws = p + 2 * t;
  c.gemm_bytes = ws_bytes > 2 * t ? ws_bytes - 2 * t : 0;
  return c;
}

ptn_status heff_apply_f64(const double2* a, const double2* w, const double2* l, const double2* r,
                          double2* out, int Dl, int d, int Dr, int chil, int chir, void* ws,
                          size_t ws_bytes, const int* skip, cudaStream_t st) {
  PTN_CHECK_ARG(ws_bytes >= 2 * align256(heff_t_elems(Dl, d, Dr, chil, chir) * sizeof(double2)),
                "heff: workspace too small");
  ContractWs c = carve(ws, heff_t_elems(Dl, d, Dr, chil, chir), ws_bytes);
  // T1[(l0,t),(wr,r2)] = A[(l0,t), r0] R[r0, (wr,r2)]
  PTN_TRY(zgemm(gemm_args('N', 'N', Dl * d, chir * Dr, Dr, a, Dr, r, (long)chir * Dr, c.t1,
                          (long)chir * Dr, skip), c.gemm_ws, c.gemm_bytes, st));
  // T2[l0,(wl,s),r2] = sum_(t,wr) W[(wl,s),(t,wr)] T1[l0,(t,wr),r2]
  PTN_TRY(mpo_stage(c.t1, c.t2, w, (long)d * chir, 1, Dl, d * chir, chil * d, Dr, skip, st));
  // out[l2,(s,r2)] = sum_(l0,wl) L[(l0,wl), l2] T2[(l0,wl),(s,r2)]
  PTN_TRY(zgemm(gemm_args('T', 'N', Dl, d * Dr, Dl * chil, l, Dl, c.t2, (long)d * Dr, out,
                          (long)d * Dr, skip), c.gemm_ws, c.gemm_bytes, st));
  return PTN_OK;
}

size_t bond_workspace_bytes_f64(int Dl, int Dr, int chi) {
  const size_t t = align256((size_t)Dl * chi * Dr * sizeof(double2));
  const size_t g = std::max(zgemm_workspace_bytes(Dl, chi * Dr, Dr, 1),
                            zgemm_workspace_bytes(Dl, Dr, Dl * chi, 1));
  return 2 * t + align256(g);
}

ptn_status bond_apply_f64(const double2* cm, const double2* l, const double2* r, double2* out,
                          int Dl, int Dr, int chi, void* ws, size_t ws_bytes, const int* skip,
                          cudaStream_t st) {
  PTN_CHECK_ARG(ws_bytes >= 2 * align256((size_t)Dl * chi * Dr * sizeof(double2)),
                "bond: workspace too small");
  ContractWs c = carve(ws, (size_t)Dl * chi * Dr, ws_bytes);
  // T1[l0,(w,r2)] = C[l0,r0] R[r0,(w,r2)]
  PTN_TRY(zgemm(gemm_args('N', 'N', Dl, chi * Dr, Dr, cm, Dr, r, (long)chi * Dr, c.t1,
                          (long)chi * Dr, skip), c.gemm_ws, c.gemm_bytes, st));
  // out[l2,r2] = sum_(l0,w) L[(l0,w),l2] T1[(l0,w),r2]
  PTN_TRY(zgemm(gemm_args('T', 'N', Dl, Dr, Dl * chi, l, Dl, c.t1, Dr, out, Dr, skip), c.gemm_ws,
                c.gemm_bytes, st));
  return PTN_OK;
}

size_t env_workspace_bytes_f64(int Dl, int d, int Dr, int chil, int chir) {
  const size_t te = (size_t)std::max(Dl * chil * d * Dr, Dl * d * chir * Dr);
  const size_t t = align256(te * sizeof(double2));
  size_t g = zgemm_workspace_bytes(Dl * chil, d * Dr, Dl, 1);
  g = std::max(g, zgemm_workspace_bytes(Dr, chir * Dr, Dl * d, 1));
  g = std::max(g, zgemm_workspace_bytes(Dl * d, chir * Dr, Dr, 1));
  g = std::max(g, zgemm_workspace_bytes(Dl * chil, Dl, d * Dr, 1));
  return 2 * t + align256(g);
}

ptn_status env_left_f64(const double2* a, const double2* b, const double2* w, const double2* l,
                        double2* lnext, int Dl, int d, int Dr, int chil, int chir, void* ws,
                        size_t ws_bytes, cudaStream_t st) {
  const size_t te = (size_t)std::max(Dl * chil * d * Dr, Dl * d * chir * Dr);
  PTN_CHECK_ARG(ws_bytes >= 2 * align256(te * sizeof(double2)), "env_left: workspace too small");
  ContractWs c = carve(ws, te, ws_bytes);
  // T1[(l0,wl),(t,rb)] = sum_l2 L[(l0,wl), l2] conj(B)[l2,(t,rb)]
  PTN_TRY(zgemm(gemm_args('N', 'C', Dl * chil, d * Dr, Dl, l, Dl, b, (long)d * Dr, c.t1,
                          (long)d * Dr, nullptr), c.gemm_ws, c.gemm_bytes, st));
  // T2[l0,(s,wr),rb] = sum_(wl,t) W[wl,t,s,wr] T1[l0,(wl,t),rb]   (stage matrix = W^T)
  PTN_TRY(mpo_stage(c.t1, c.t2, w, 1, (long)d * chir, Dl, chil * d, d * chir, Dr, nullptr, st));
  // l_next[ra,(wr,rb)] = sum_(l0,s) A[(l0,s),ra] T2[(l0,s),(wr,rb)]
  PTN_TRY(zgemm(gemm_args('T', 'N', Dr, chir * Dr, Dl * d, a, Dr, c.t2, (long)chir * Dr, lnext,
                          (long)chir * Dr, nullptr), c.gemm_ws, c.gemm_bytes, st));
  return PTN_OK;
}

ptn_status env_right_f64(const double2* a, const double2* b, const double2* w, const double2* r,
                         double2* rnext, int Dl, int d, int Dr, int chil, int chir, void* ws,
                         size_t ws_bytes, cudaStream_t st) {
  const size_t te = (size_t)std::max(Dl * chil * d * Dr, Dl * d * chir * Dr);
  PTN_CHECK_ARG(ws_bytes >= 2 * align256(te * sizeof(double2)), "env_right: workspace too small");
  ContractWs c = carve(ws, te, ws_bytes);
  // T1[(l0,s),(wr,r2)] = A[(l0,s),r0] R[r0,(wr,r2)]
  PTN_TRY(zgemm(gemm_args('N', 'N', Dl * d, chir * Dr, Dr, a, Dr, r, (long)chir * Dr, c.t1,
                          (long)chir * Dr, nullptr), c.gemm_ws, c.gemm_bytes, st));
  // T2[l0,(wl,t),r2] = sum_(s,wr) W[(wl,t),(s,wr)] T1[l0,(s,wr),r2]
  PTN_TRY(mpo_stage(c.t1, c.t2, w, (long)d * chir, 1, Dl, d * chir, chil * d, Dr, nullptr, st));
  // r_next[(l0,wl),lb] = sum_(t,r2) T2[(l0,wl),(t,r2)] conj(B[lb,(t,r2)])
  PTN_TRY(zgemm(gemm_args('N', 'H', Dl * chil, Dl, d * Dr, c.t2, (long)d * Dr, b, (long)d * Dr,
                          rnext, Dl, nullptr), c.gemm_ws, c.gemm_bytes, st));
  return PTN_OK;
}

}  // namespace ptn

// ---------------------------------------------------------------------- C ABI
using namespace ptn;

static inline const double2* D2(const ptn_c128* p) { return reinterpret_cast<const double2*>(p); }
static inline double2* D2(ptn_c128* p) { return reinterpret_cast<double2*>(p); }

namespace ptn {
size_t heff_workspace_bytes_mixed(int Dl, int d, int Dr, int chil, int chir);
size_t bond_workspace_bytes_mixed(int Dl, int Dr, int chi);
ptn_status heff_apply_mixed_entry(const double2*, const double2*, const double2*, const double2*,
                                  double2*, int, int, int, int, int, void*, size_t, cudaStream_t);
ptn_status bond_apply_mixed_entry(const double2*, const double2*, const double2*, double2*, int,
                                  int, int, void*, size_t, cudaStream_t);
size_t env_workspace_bytes_mixed(int Dl, int d, int Dr, int cl, int cr);
ptn_status env_left_mixed(const double2*, const double2*, const double2*, const double2*, double2*,
                          int, int, int, int, int, void*, size_t, cudaStream_t);
ptn_status env_right_mixed(const double2*, const double2*, const double2*, const double2*, double2*,
                           int, int, int, int, int, void*, size_t, cudaStream_t);
}  // namespace ptn

extern "C" {

size_t ptn_heff_workspace_bytes(int Dl, int d, int Dr, int chil, int chir, int prec) {
  return prec == PTN_PREC_FP64 ? heff_workspace_bytes_f64(Dl, d, Dr, chil, chir)
                               : heff_workspace_bytes_mixed(Dl, d, Dr, chil, chir);
}

size_t ptn_bond_workspace_bytes(int Dl, int Dr, int chi, int prec) {
  return prec == PTN_PREC_FP64 ? bond_workspace_bytes_f64(Dl, Dr, chi)
                               : bond_workspace_bytes_mixed(Dl, Dr, chi);
}

size_t ptn_env_workspace_bytes(int Dl, int d, int Dr, int chil, int chir, int prec) {
  return prec == PTN_PREC_FP64 ? env_workspace_bytes_f64(Dl, d, Dr, chil, chir)
                               : env_workspace_bytes_mixed(Dl, d, Dr, chil, chir);
}

ptn_status ptn_heff_apply(const ptn_c128* a, const ptn_c128* w, const ptn_c128* l,
                          const ptn_c128* r, ptn_c128* out, int Dl, int d, int Dr, int chil,
                          int chir, int prec, void* ws, size_t ws_bytes, void* stream) {
  PTN_CHECK_ARG(Dl > 0 && d > 0 && Dr > 0 && chil > 0 && chir > 0, "heff: bad dims");
  if (prec == PTN_PREC_FP64)
    return heff_apply_f64(D2(a), D2(w), D2(l), D2(r), D2(out), Dl, d, Dr, chil, chir, ws, ws_bytes,
                          nullptr, as_stream(stream));
  return heff_apply_mixed_entry(D2(a), D2(w), D2(l), D2(r), D2(out), Dl, d, Dr, chil, chir, ws,
                                ws_bytes, as_stream(stream));
}

ptn_status ptn_bond_apply(const ptn_c128* c, const ptn_c128* l, const ptn_c128* r, ptn_c128* out,
                          int Dl, int Dr, int chi, int prec, void* ws, size_t ws_bytes,
                          void* stream) {
  PTN_CHECK_ARG(Dl > 0 && Dr > 0 && chi > 0, "bond: bad dims");
  if (prec == PTN_PREC_FP64)
    return bond_apply_f64(D2(c), D2(l), D2(r), D2(out), Dl, Dr, chi, ws, ws_bytes, nullptr,
                          as_stream(stream));
  return bond_apply_mixed_entry(D2(c), D2(l), D2(r), D2(out), Dl, Dr, chi, ws, ws_bytes,
                                as_stream(stream));
}

ptn_status ptn_env_step_left(const ptn_c128* a, const ptn_c128* b, const ptn_c128* w,
                             const ptn_c128* l, ptn_c128* l_next, int Dl, int d, int Dr, int chil,
                             int chir, int prec, void* ws, size_t ws_bytes, void* stream) {
  PTN_CHECK_ARG(Dl > 0 && d > 0 && Dr > 0 && chil > 0 && chir > 0, "env_left: bad dims");
  if (prec != PTN_PREC_FP64)
    return env_left_mixed(D2(a), D2(b), D2(w), D2(l), D2(l_next), Dl, d, Dr, chil, chir, ws,
                          ws_bytes, as_stream(stream));
  return env_left_f64(D2(a), D2(b), D2(w), D2(l), D2(l_next), Dl, d, Dr, chil, chir, ws, ws_bytes,
                      as_stream(stream));
}

ptn_status ptn_env_step_right(const ptn_c128* a, const ptn_c128* b, const ptn_c128* w,
                              const ptn_c128* r, ptn_c128* r_next, int Dl, int d, int Dr, int chil,
                              int chir, int prec, void* ws, size_t ws_bytes, void* stream) {
  PTN_CHECK_ARG(Dl > 0 && d > 0 && Dr > 0 && chil > 0 && chir > 0, "env_right: bad dims");
  if (prec != PTN_PREC_FP64)
    return env_right_mixed(D2(a), D2(b), D2(w), D2(r), D2(r_next), Dl, d, Dr, chil, chir, ws,
                           ws_bytes, as_stream(stream));
  return env_right_f64(D2(a), D2(b), D2(w), D2(r), D2(r_next), Dl, d, Dr, chil, chir, ws, ws_bytes,
                       as_stream(stream));
}

}  // extern "C"
