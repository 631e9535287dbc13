// Mixed-precision form of the site / bond operators and of the environment steps
// (pytenet/chain_ops.py:16-99, 237-317): the two GEMMs of every contraction run on
// the tensor cores as exact fixed-point BF16 digit products (tc_gemm.cu); the MPO
// stage, the digit levels, the split-K sums and everything outside the
// contractions are FP64.
//
// Operand conversion ("digits"): a complex matrix view (element (r, k) at
// src[r * sr + k * sk]) becomes five BF16 digit planes plus one power-of-two
// exponent per row r. Two tiled passes: the first finds each row's largest
// |component| (atomicMax of the IEEE exponent field), the second forms the
// fixed-point integer round(x 2^(39 - e)) from the IEEE fields and cuts it into
// five balanced base-256 digits with integer arithmetic only, stored k-contiguously. "Plain" operands keep
// re/im interleaved along K; "embedded" operands store z as [[Re, -Im], [Im, Re]].
//
// Data flow of H_eff . x (site tensors (Dl, d, Dr), MPO bonds cl / cr):
//   prepare (once per local step):  R -> Rt  (plain, rows (wr, r2), K = r0)
//                                   L -> Le  (embedded, n = l2, K = (l0, wl))
//   apply:  x -> Xe (embedded, n = (l0, t), K = r0)
//           GEMM 1: T1^T[(wr,r2)][(l0,t)] = Rt . Xe^T, written as T1[(l0,t)][(wr,r2)]
//           MPO stage (FP64): T2[l0,(wl,s),r2]
//           T2 -> T2s (plain, rows (s, r2), K = (l0, wl))
//           GEMM 2: out^T[(s,r2)][l2] = T2s . Le^T, written as out[l2][(s,r2)]
// Every GEMM computes the transpose of the wanted product so that the epilogue
// thread of output row m writes consecutive addresses with its neighbours.
#include "ptn_common.cuh"
#include <cuda_bf16.h>
#include <algorithm>

namespace ptn {

void note_launches(int n);
ptn_status tc_gemm(const void* Aslices, long aplane, const int* ea, const void* Bslices, long bplane,
                   const int* eb, int M, int Nc, int Kc, long Kp, double2* out, long ldm, long ldn,
                   bool accumulate, void* ws, size_t ws_bytes, const int* skip, cudaStream_t st,
                   const unsigned char* fa, const unsigned char* fb, int fk);
size_t tc_gemm_workspace_bytes(int M, int Ncomplex, int Kcomplex);
ptn_status mpo_stage_f64(const double2* in, double2* out, const double2* w, long ldq, long ldp, int X,
                         int P, int Q, int Y, const int* skip, cudaStream_t st);

namespace {

typedef __nv_bfloat16 bf16;
constexpr int NDIGIT = 5;
constexpr int EXP_ZERO = -2000;   // rows with no non-zero entry (memset 0x80 gives less)

// 32 x 32 complex tile of the view, rows r0.., cols k0..; threads (32, 8)
__device__ __forceinline__ void load_tile(double2 (*tile)[33], const double2* __restrict__ src,
                                          long sr, long sk, int R, int K, int r0, int k0, int conj) {
  const int tx = threadIdx.x, ty = threadIdx.y;
  if (sk == 1) {
    for (int rr = ty; rr < 32; rr += 8) {
      const int r = r0 + rr, k = k0 + tx;
      double2 v = (r < R && k < K) ? src[(long)r * sr + k] : make_double2(0.0, 0.0);
      if (conj) v.y = -v.y;
      tile[rr][tx] = v;
    }
  } else {
    for (int kk = ty; kk < 32; kk += 8) {
      const int r = r0 + tx, k = k0 + kk;
      double2 v = (r < R && k < K) ? src[(long)r * sr + (long)k * sk] : make_double2(0.0, 0.0);
      if (conj) v.y = -v.y;
      tile[tx][kk] = v;
    }
  }
}

__device__ __forceinline__ int biased_exp(double x) {
  return (int)((__double_as_longlong(x) >> 52) & 0x7FF);
}

__global__ void rowexp_kernel(const double2* __restrict__ src, long sr, long sk, int R, int K,
                              int* __restrict__ e, const int* skip) {
  if (skip != nullptr && *skip != 0) return;
  __shared__ double2 tile[32][33];
  const int r0 = blockIdx.y * 32, k0 = blockIdx.x * 32;
  load_tile(tile, src, sr, sk, R, K, r0, k0, 0);
  __syncthreads();
  for (int rr = threadIdx.y; rr < 32; rr += 8) {
    const double2 v = tile[rr][threadIdx.x];
    // biased exponent fields (integer work only; zero and subnormal entries give 0)
    int m = max(biased_exp(v.x), biased_exp(v.y));
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) m = max(m, __shfl_xor_sync(0xffffffffu, m, o));
    if (threadIdx.x == 0 && r0 + rr < R && m > 0) {
      // a normal |x| with biased exponent E lies in [2^(E-1023), 2^(E-1022)): every
      // entry of the row is below 2^ex (frexp's exponent of the largest one)
      atomicMax(&e[r0 + rr], m - 1022);
    }
  }
}

// Balanced base-256 digits of x 2^(7 - ex) (|x| < 2^ex): the fixed-point integer
// T = round(x 2^(39 - ex)) (|T| <= 2^39) is cut into
// T = d0 2^32 + d1 2^24 + d2 2^16 + d3 2^8 + d4 with d1..d4 in [-128, 127] and
// |d0| <= 128, each exact in BF16. Integer
// arithmetic on the IEEE fields only: the CUDA-core FP64 rate of this part is low.
// Zero and subnormal entries (below 2^-1022) give zero digits.
__device__ __forceinline__ void digits_of(double x, int ex, bf16 (&d)[NDIGIT]) {
  const long long b = __double_as_longlong(x);
  const int E = (int)((b >> 52) & 0x7FF);
  long long T = 0;
  if (E != 0) {
    const long long mant = (b & ((1LL << 52) - 1)) | (1LL << 52);
    // x = mant 2^(E - 1075): T = round(mant 2^(E - 1075 + 39 - ex)), shift always right
    const int rs = 1075 - (8 * NDIGIT - 1) + ex - E;
    if (rs < 63) T = (rs <= 0) ? (mant << (-rs)) : ((mant + (1LL << (rs - 1))) >> rs);
    if (b < 0) T = -T;
  }
#pragma unroll
  for (int i = NDIGIT - 1; i > 0; --i) {
    const int di = (int)((T + 128) & 255) - 128;
    d[i] = __int2bfloat16_rn(di);
    T = (T - di) >> 8;   // exact
  }
  d[0] = __int2bfloat16_rn((int)T);
}

// With zero-tile flags on (flags_on), also marks flags[1 + (r / fg) * fk + k / 16]
// for every non-zero entry (r, k): the tiles of the digit GEMM (128 rows of a plain
// operand, 48 complex columns of an embedded one) by K block of 16 complex entries,
// so that the GEMM can skip all-zero tiles (quantum-number block sparsity); one
// store per warp, row and K block (the buffer is zeroed before). flags[0] tells the
// GEMM whether the flags of this conversion are valid.
__global__ void digits_kernel(const double2* __restrict__ src, long sr, long sk, int R, int K,
                              int conj, const int* __restrict__ e, bf16* __restrict__ dst, long Kp,
                              long plane, int embedded, unsigned char* __restrict__ flags,
                              int flags_on, int fg, long fk, const int* skip) {
  if (skip != nullptr && *skip != 0) return;
  if (blockIdx.x == 0 && blockIdx.y == 0 && threadIdx.x == 0 && threadIdx.y == 0)
    flags[0] = (unsigned char)flags_on;
  __shared__ double2 tile[32][33];
  const int r0 = blockIdx.y * 32, k0 = blockIdx.x * 32;
  load_tile(tile, src, sr, sk, R, K, r0, k0, conj);
  __syncthreads();
  if (flags_on) {
    // lanes 0..15 and 16..31 of a row cover one K block each
    for (int rr = threadIdx.y; rr < 32; rr += 8) {
      const int r = r0 + rr, k = k0 + threadIdx.x;
      const double2 z = tile[rr][threadIdx.x];
      const unsigned nz = __ballot_sync(0xffffffffu, r < R && k < K && (z.x != 0.0 || z.y != 0.0));
      const unsigned half = (threadIdx.x < 16) ? (nz & 0xFFFFu) : (nz >> 16);
      if ((threadIdx.x & 15) == 0 && half != 0) flags[1 + (long)(r / fg) * fk + (k >> 4)] = 1;
    }
  }
  const int k = k0 + threadIdx.x;
  if (k >= K) return;
  for (int rr = threadIdx.y; rr < 32; rr += 8) {
    const int r = r0 + rr;
    if (r >= R) break;
    const int ex = e[r];
    const double2 z = tile[rr][threadIdx.x];
    bf16 dr[NDIGIT], di[NDIGIT];
    if (ex > EXP_ZERO) {
      digits_of(z.x, ex, dr);
      digits_of(z.y, ex, di);
    } else {
#pragma unroll
      for (int i = 0; i < NDIGIT; ++i) dr[i] = di[i] = __double2bfloat16(0.0);
    }
#pragma unroll
    for (int i = 0; i < NDIGIT; ++i) {
      bf16* base = dst + (long)i * plane;
      if (!embedded) {
        reinterpret_cast<__nv_bfloat162*>(base + (long)r * Kp + 2L * k)[0] =
            __halves2bfloat162(dr[i], di[i]);
      } else {
        reinterpret_cast<__nv_bfloat162*>(base + (2L * r) * Kp + 2L * k)[0] =
            __halves2bfloat162(dr[i], __hneg(di[i]));
        reinterpret_cast<__nv_bfloat162*>(base + (2L * r + 1) * Kp + 2L * k)[0] =
            __halves2bfloat162(di[i], dr[i]);
      }
    }
  }
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

// The split-K scratch of the digit GEMMs is the last piece of every workspace
// layout: give the GEMMs all that the caller's workspace has left (the GEMM picks
// its K splits to fit, never below what exact accumulation needs), so a workspace
// sized under other tuning-knob values still works.
template <class W>
void use_rest(W& w, void* ws, size_t ws_bytes) {
  const size_t off = (size_t)(static_cast<char*>(w.gws) - static_cast<char*>(ws));
  w.gbytes = ws_bytes > off ? ws_bytes - off : 0;
}

// bytes a layout needs before its GEMM scratch
template <class W>
size_t before_gemm(const Carver& c, const W& w) {
  return c.off - al(w.gbytes);
}

// BF16 digit planes of a complex matrix with `rows` rows (2 * rows real rows when
// embedded) and kc complex columns, plus the per-row exponents
struct Digits {
  bf16* p;
  int* e;
  unsigned char* f;   // non-zero flags per (GEMM tile of rows, K block of 16 complex)
  long rows, kc, Kp;
  bool embedded;
  int fgroup() const { return embedded ? 48 : 128; }
  long fk() const { return (kc + 15) / 16; }
  long frows() const { return (rows + fgroup() - 1) / fgroup(); }
  long real_rows() const { return embedded ? 2 * rows : rows; }
  long plane() const { return real_rows() * Kp; }
};

Digits take_digits(Carver& c, long rows, long kc, bool embedded) {
  Digits d;
  d.rows = rows;
  d.kc = kc;
  d.Kp = kpad(kc);
  d.embedded = embedded;
  d.p = static_cast<bf16*>(c.take((size_t)NDIGIT * d.real_rows() * d.Kp * sizeof(bf16)));
  d.e = static_cast<int*>(c.take((size_t)rows * sizeof(int)));
  d.f = static_cast<unsigned char*>(c.take(1 + (size_t)d.frows() * d.fk()));
  return d;
}

// view (r, k) -> src[r * sr + k * sk], r < d.rows, k < d.kc
ptn_status to_digits(const double2* src, long sr, long sk, const Digits& d, bool conj,
                     const int* skip, cudaStream_t st) {
  PTN_CUDA_TRY(cudaMemsetAsync(d.e, 0x80, (size_t)d.rows * sizeof(int), st));
  const int flags_on = tune(PTN_TUNE_TC_SKIP_ZERO) != 0 ? 1 : 0;
  if (flags_on) PTN_CUDA_TRY(cudaMemsetAsync(d.f, 0, 1 + (size_t)d.frows() * d.fk(), st));
  dim3 grid((unsigned)((d.kc + 31) / 32), (unsigned)((d.rows + 31) / 32));
  PTN_CHECK_ARG(grid.y <= 65535, "digits: too many rows");
  rowexp_kernel<<<grid, dim3(32, 8), 0, st>>>(src, sr, sk, (int)d.rows, (int)d.kc, d.e, skip);
  digits_kernel<<<grid, dim3(32, 8), 0, st>>>(src, sr, sk, (int)d.rows, (int)d.kc, conj ? 1 : 0,
                                              d.e, d.p, d.Kp, d.plane(), d.embedded ? 1 : 0, d.f,
                                              flags_on, d.fgroup(), d.fk(), skip);
  PTN_LAUNCH_CHECK();
  note_launches(2);
  return PTN_OK;
}

// C = A . B^T over the digit planes: A plain (M x Kc), B embedded (Nc x Kc)
ptn_status gemm(const Digits& A, const Digits& Be, double2* out, long ldm, long ldn, void* ws,
                size_t ws_bytes, const int* skip, cudaStream_t st) {
  const bool flags = tune(PTN_TUNE_TC_SKIP_ZERO) != 0;
  return tc_gemm(A.p, A.plane(), A.e, Be.p, Be.plane(), Be.e, (int)A.rows, (int)Be.rows,
                 (int)A.kc, A.Kp, out, ldm, ldn, false, ws, ws_bytes, skip, st,
                 flags ? A.f : nullptr, flags ? Be.f : nullptr, (int)A.fk());
}

// ---------------------------------------------------------------- H_eff (site)
struct HeffWs {
  Digits Rt, Le, Xe, T2s;
  double2 *T1, *T2;
  void* gws;
  size_t gbytes;
};

HeffWs heff_ws(Carver& c, int Dl, int d, int Dr, int cl, int cr) {
  HeffWs w;
  w.Rt = take_digits(c, (long)cr * Dr, Dr, false);
  w.Le = take_digits(c, Dl, (long)Dl * cl, true);
  w.Xe = take_digits(c, (long)Dl * d, Dr, true);
  w.T2s = take_digits(c, (long)d * Dr, (long)Dl * cl, false);
  w.T1 = static_cast<double2*>(c.take((size_t)Dl * d * cr * Dr * sizeof(double2)));
  w.T2 = static_cast<double2*>(c.take((size_t)Dl * cl * d * Dr * sizeof(double2)));
  w.gbytes = std::max(tc_gemm_workspace_bytes(cr * Dr, Dl * d, Dr),
                      tc_gemm_workspace_bytes(d * Dr, Dl, Dl * cl));
  w.gws = c.take(w.gbytes);
  return w;
}

// ---------------------------------------------------------------- zero-site (bond)
struct BondWs {
  Digits Rt, Le, Xe, T1s;
  double2* T1;
  void* gws;
  size_t gbytes;
};

BondWs bond_ws(Carver& c, int Dl, int Dr, int chi) {
  BondWs w;
  w.Rt = take_digits(c, (long)chi * Dr, Dr, false);
  w.Le = take_digits(c, Dl, (long)Dl * chi, true);
  w.Xe = take_digits(c, Dl, Dr, true);
  w.T1s = take_digits(c, Dr, (long)Dl * chi, false);
  w.T1 = static_cast<double2*>(c.take((size_t)Dl * chi * Dr * sizeof(double2)));
  w.gbytes = std::max(tc_gemm_workspace_bytes(chi * Dr, Dl, Dr),
                      tc_gemm_workspace_bytes(Dr, Dl, Dl * chi));
  w.gws = c.take(w.gbytes);
  return w;
}

// ---------------------------------------------------------------- environments
struct EnvWs {
  Digits S1, E1, S2, E2;
  double2 *T1, *T2;
  void* gws;
  size_t gbytes;
};

EnvWs env_left_ws(Carver& c, int Dl, int d, int Dr, int cl, int cr) {
  EnvWs w;
  w.S1 = take_digits(c, (long)d * Dr, Dl, false);           // conj(B)^T, rows (t, rb), K = l2
  w.E1 = take_digits(c, (long)Dl * cl, Dl, true);           // L, n = (l0, wl), K = l2
  w.S2 = take_digits(c, (long)cr * Dr, (long)Dl * d, false); // T2^T, rows (wr, rb), K = (l0, s)
  w.E2 = take_digits(c, Dr, (long)Dl * d, true);            // A, n = ra, K = (l0, s)
  w.T1 = static_cast<double2*>(c.take((size_t)Dl * cl * d * Dr * sizeof(double2)));
  w.T2 = static_cast<double2*>(c.take((size_t)Dl * d * cr * Dr * sizeof(double2)));
  w.gbytes = std::max(tc_gemm_workspace_bytes(d * Dr, Dl * cl, Dl),
                      tc_gemm_workspace_bytes(cr * Dr, Dr, Dl * d));
  w.gws = c.take(w.gbytes);
  return w;
}

EnvWs env_right_ws(Carver& c, int Dl, int d, int Dr, int cl, int cr) {
  EnvWs w;
  w.S1 = take_digits(c, (long)cr * Dr, Dr, false);          // R^T, rows (wr, r2), K = r0
  w.E1 = take_digits(c, (long)Dl * d, Dr, true);            // A, n = (l0, s), K = r0
  w.S2 = take_digits(c, Dl, (long)d * Dr, false);           // conj(B), rows lb, K = (t, r2)
  w.E2 = take_digits(c, (long)Dl * cl, (long)d * Dr, true); // T2, n = (l0, wl), K = (t, r2)
  w.T1 = static_cast<double2*>(c.take((size_t)Dl * d * cr * Dr * sizeof(double2)));
  w.T2 = static_cast<double2*>(c.take((size_t)Dl * cl * d * Dr * sizeof(double2)));
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
  {
    Carver q(nullptr);
    const HeffWs hq = heff_ws(q, Dl, d, Dr, chil, chir);
    PTN_CHECK_ARG(ws_bytes >= before_gemm(q, hq), "mixed heff: workspace too small");
  }
  Carver c(ws);
  HeffWs h = heff_ws(c, Dl, d, Dr, chil, chir);
  // Rt: (m = (wr, r2), k = r0) = R[r0][(wr, r2)]
  PTN_TRY(to_digits(r, 1, (long)chir * Dr, h.Rt, false, nullptr, st));
  // Le: (n = l2, k = (l0, wl)) = L[(l0, wl)][l2]
  PTN_TRY(to_digits(l, 1, Dl, h.Le, false, nullptr, st));
  return PTN_OK;
}

ptn_status heff_apply_mixed(const double2* x, double2* y, const double2* w, int Dl, int d, int Dr,
                            int chil, int chir, void* ws, size_t ws_bytes, const int* skip,
                            cudaStream_t st) {
  Carver c(ws);
  HeffWs h = heff_ws(c, Dl, d, Dr, chil, chir);
  use_rest(h, ws, ws_bytes);
  // Xe: (n = (l0, t), k = r0) = x[(l0, t)][r0]
  PTN_TRY(to_digits(x, Dr, 1, h.Xe, false, skip, st));
  // T1[(l0,t)][(wr,r2)] via T1^T = Rt . Xe^T
  PTN_TRY(gemm(h.Rt, h.Xe, h.T1, 1, (long)chir * Dr, h.gws, h.gbytes, skip, st));
  // T2[l0][(wl, s)][r2] = sum_(t, wr) W[(wl, s), (t, wr)] T1[l0][(t, wr)][r2]
  PTN_TRY(mpo_stage_f64(h.T1, h.T2, w, (long)d * chir, 1, Dl, d * chir, chil * d, Dr, skip, st));
  // T2s: (m = (s, r2), k = (l0, wl)) = T2[(l0, wl)][(s, r2)]
  PTN_TRY(to_digits(h.T2, 1, (long)d * Dr, h.T2s, false, skip, st));
  // out^T[(s, r2)][l2] = T2s . Le^T -> out[l2][(s, r2)]
  PTN_TRY(gemm(h.T2s, h.Le, y, 1, (long)d * Dr, h.gws, h.gbytes, skip, st));
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
  {
    Carver q(nullptr);
    const BondWs bq = bond_ws(q, Dl, Dr, chi);
    PTN_CHECK_ARG(ws_bytes >= before_gemm(q, bq), "mixed bond: workspace too small");
  }
  Carver c(ws);
  BondWs b = bond_ws(c, Dl, Dr, chi);
  PTN_TRY(to_digits(r, 1, (long)chi * Dr, b.Rt, false, nullptr, st));
  PTN_TRY(to_digits(l, 1, Dl, b.Le, false, nullptr, st));
  return PTN_OK;
}

ptn_status bond_apply_mixed(const double2* x, double2* y, int Dl, int Dr, int chi, void* ws,
                            size_t ws_bytes, const int* skip, cudaStream_t st) {
  Carver c(ws);
  BondWs b = bond_ws(c, Dl, Dr, chi);
  use_rest(b, ws, ws_bytes);
  // Xe: (n = l0, k = r0) = C[l0][r0]
  PTN_TRY(to_digits(x, Dr, 1, b.Xe, false, skip, st));
  // T1[l0][(w, r2)] via T1^T = Rt . Xe^T
  PTN_TRY(gemm(b.Rt, b.Xe, b.T1, 1, (long)chi * Dr, b.gws, b.gbytes, skip, st));
  // T1s: (m = r2, k = (l0, w)) = T1[(l0, w)][r2]
  PTN_TRY(to_digits(b.T1, 1, Dr, b.T1s, false, skip, st));
  // out^T[r2][l2] = T1s . Le^T -> out[l2][r2]
  PTN_TRY(gemm(b.T1s, b.Le, y, 1, Dr, b.gws, b.gbytes, skip, st));
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
  Carver c(ws);
  EnvWs e = env_left_ws(c, Dl, d, Dr, cl, cr);
  PTN_CHECK_ARG(ws_bytes >= before_gemm(c, e), "mixed env: workspace too small");
  use_rest(e, ws, ws_bytes);
  // S1: (m = (t, rb), k = l2) = conj(B[l2][(t, rb)])
  PTN_TRY(to_digits(b, 1, (long)d * Dr, e.S1, true, nullptr, st));
  // E1: (n = (l0, wl), k = l2) = L[(l0, wl)][l2]
  PTN_TRY(to_digits(l, Dl, 1, e.E1, false, nullptr, st));
  // T1^T[(t, rb)][(l0, wl)] -> T1[(l0, wl)][(t, rb)]
  PTN_TRY(gemm(e.S1, e.E1, e.T1, 1, (long)d * Dr, e.gws, e.gbytes, nullptr, st));
  // T2[l0][(s, wr)][rb] = sum_(wl, t) W[wl,t,s,wr] T1[l0][(wl, t)][rb]   (stage matrix W^T)
  PTN_TRY(mpo_stage_f64(e.T1, e.T2, w, 1, (long)d * cr, Dl, cl * d, d * cr, Dr, nullptr, st));
  // S2: (m = (wr, rb), k = (l0, s)) = T2[(l0, s)][(wr, rb)]
  PTN_TRY(to_digits(e.T2, 1, (long)cr * Dr, e.S2, false, nullptr, st));
  // E2: (n = ra, k = (l0, s)) = A[(l0, s)][ra]
  PTN_TRY(to_digits(a, 1, Dr, e.E2, false, nullptr, st));
  // l_next^T[(wr, rb)][ra] = S2 . E2^T -> l_next[ra][(wr, rb)]
  PTN_TRY(gemm(e.S2, e.E2, lnext, 1, (long)cr * Dr, e.gws, e.gbytes, nullptr, st));
  return PTN_OK;
}

// r_next[la, wl, lb] = sum A[la,s,r0] W[wl,t,s,wr] R[r0,wr,r2] conj(B[lb,t,r2])
ptn_status env_right_mixed(const double2* a, const double2* b, const double2* w, const double2* r,
                           double2* rnext, int Dl, int d, int Dr, int cl, int cr, void* ws,
                           size_t ws_bytes, cudaStream_t st) {
  Carver c(ws);
  EnvWs e = env_right_ws(c, Dl, d, Dr, cl, cr);
  PTN_CHECK_ARG(ws_bytes >= before_gemm(c, e), "mixed env: workspace too small");
  use_rest(e, ws, ws_bytes);
  // S1: (m = (wr, r2), k = r0) = R[r0][(wr, r2)]
  PTN_TRY(to_digits(r, 1, (long)cr * Dr, e.S1, false, nullptr, st));
  // E1: (n = (l0, s), k = r0) = A[(l0, s)][r0]
  PTN_TRY(to_digits(a, Dr, 1, e.E1, false, nullptr, st));
  // T1^T[(wr, r2)][(l0, s)] -> T1[(l0, s)][(wr, r2)]
  PTN_TRY(gemm(e.S1, e.E1, e.T1, 1, (long)cr * Dr, e.gws, e.gbytes, nullptr, st));
  // T2[l0][(wl, t)][r2] = sum_(s, wr) W[(wl, t), (s, wr)] T1[l0][(s, wr)][r2]
  PTN_TRY(mpo_stage_f64(e.T1, e.T2, w, (long)d * cr, 1, Dl, d * cr, cl * d, Dr, nullptr, st));
  // E2: (n = (l0, wl), k = (t, r2)) = T2[(l0, wl)][(t, r2)]
  PTN_TRY(to_digits(e.T2, (long)d * Dr, 1, e.E2, false, nullptr, st));
  // S2: (m = lb, k = (t, r2)) = conj(B[lb][(t, r2)])
  PTN_TRY(to_digits(b, (long)d * Dr, 1, e.S2, true, nullptr, st));
  // r_next^T[lb][(l0, wl)] = S2 . E2^T -> r_next[(l0, wl)][lb]
  PTN_TRY(gemm(e.S2, e.E2, rnext, 1, Dl, e.gws, e.gbytes, nullptr, st));
  return PTN_OK;
}

// ================================================================ plain GEMM entry
size_t zgemm_split_workspace_bytes(int M, int N, int K) {
  Carver c(nullptr);
  take_digits(c, M, K, false);
  take_digits(c, N, K, true);
  c.take(tc_gemm_workspace_bytes(M, N, K));
  return c.off;
}

// C = A B (row-major complex, M x K times K x N) through the digit products
ptn_status zgemm_split(const double2* A, long lda, const double2* B, long ldb, double2* C, long ldc,
                       int M, int N, int K, void* ws, size_t ws_bytes, cudaStream_t st) {
  PTN_CHECK_ARG(M > 0 && N > 0 && K > 0, "zgemm_split: bad sizes");
  Carver c(ws);
  Digits As = take_digits(c, M, K, false);
  Digits Bs = take_digits(c, N, K, true);
  PTN_CHECK_ARG(ws_bytes >= c.off, "zgemm_split: workspace too small");
  void* g = c.take(0);
  const size_t gb = ws_bytes - c.off;
  PTN_TRY(to_digits(A, lda, 1, As, false, nullptr, st));
  // B as the view (n, k) = B[k][n]
  PTN_TRY(to_digits(B, 1, ldb, Bs, false, nullptr, st));
  return gemm(As, Bs, C, ldc, 1, g, gb, nullptr, st);
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
