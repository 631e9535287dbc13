/*
 * pytenet_gb300 -- C ABI of the GB300 engine for single-site TDVP / DMRG sweeps.
 *
 * This is the drop-in boundary below the Python API that mirrors PyTeNet
 * (cmendl/pytenet). Each entry point names the reference function it replaces
 * (paths relative to the reference project root). The reference is pure Python:
 * its "FFI" is the Python call itself, so the host-side binding is the ctypes
 * module pytenet_gb300/_lib.py.
 *
 * Conventions
 *  - All tensors are row-major (C-contiguous) device buffers owned by the caller.
 *    Complex128 values are {re, im} pairs of doubles (numpy.complex128 layout).
 *  - Index layouts follow the reference exactly:
 *      MPS site tensor A  (Dl, d, Dr)         pytenet/mps.py:14-26
 *      MPO site tensor W  (chil, d, d, chir)  pytenet/mpo.py:15-29 (stored complex here)
 *      left env  L        (Dl, chil, Dl)      pytenet/tdvp.py:55-58
 *      right env R        (Dr, chir, Dr)      pytenet/chain_ops.py:102-113
 *  - `stream` is a cudaStream_t (NULL = legacy default stream). No entry point
 *    synchronises the device, allocates device memory or reads device memory on
 *    the host: every launch is asynchronous and can be captured in a CUDA graph.
 *    Scratch memory is passed in as `ws` / `ws_bytes`; the *_workspace_bytes
 *    functions give the size needed.
 *  - Errors are returned as ptn_status; ptn_last_error() gives the message.
 *    The reference raises AssertionError for the same conditions.
 */
#ifndef PYTENET_GB300_H
#define PYTENET_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum {
  PTN_OK = 0,
  PTN_BAD_SHAPE = 1,   /* shape / argument check failed (reference: AssertionError) */
  PTN_BREAKDOWN = 2,   /* informational: Lanczos stopped early (reference: RuntimeWarning) */
  PTN_NAN = 3,         /* zero or non-finite norm of a Krylov start vector */
  PTN_TIMEOUT = 4,     /* a bounded device-side wait gave up */
  PTN_CUDA_ERROR = 5,  /* CUDA runtime error (launch failure etc.) */
  PTN_UNSUPPORTED = 6  /* configuration not built into this library */
} ptn_status;

typedef enum {
  PTN_PREC_FP64 = 0,        /* plain complex128 (FP64 DMMA tensor cores) */
  PTN_PREC_SPLIT_BF16 = 1   /* fixed-point BF16 digit products on tcgen05 (5 digits per
                               row-scaled value, exact FP32 integer accumulation per digit
                               level, FP64 recombination): ~2e-11 relative per contraction */
} ptn_precision;

typedef struct { double re, im; } ptn_c128;

#define PTN_ABI_VERSION 3
#define PTN_KRYLOV_MAXITER 64

/* Device-resident state of one Krylov (Lanczos) run. Laid out for direct reads
 * from the host after the stream is synchronised. */
typedef struct {
  int32_t m_used;      /* Lanczos vectors in use (numiter, or fewer after a breakdown) */
  int32_t stopped;     /* 1 once beta_j < 100 * n * eps stopped the iteration */
  int32_t maxiter;     /* requested number of iterations */
  int32_t status;      /* PTN_OK, or PTN_NAN if the start vector norm was zero / not finite */
  int32_t breakdowns;  /* cumulative count of early stops since the buffer was zeroed */
  int32_t m_target;    /* learned depth at which the residual is tested (0: fixed depth) */
  double nrm;          /* norm of the start vector */
  double beta_next;    /* norm of the residual left after the final iteration */
  double eval0;        /* lowest Ritz value (eigh mode) */
  double resid;        /* relative a-posteriori error estimate beta_m |e_m^T f(T) e_1|
                          (the estimate of the step's error divided by nrm), in every mode */
  int32_t early_exits; /* cumulative count of accepted learned depths */
  int32_t iters_total; /* cumulative count of Lanczos vectors used (operator applies) */
  float feat[12];      /* features of the current local step (learned depth) */
  double alpha[PTN_KRYLOV_MAXITER];
  double beta[PTN_KRYLOV_MAXITER];
  ptn_c128 coef[PTN_KRYLOV_MAXITER];  /* combination coefficients of the Lanczos vectors */
} ptn_krylov_state;

/* ---------------------------------------------------------------- library */
int ptn_abi_version(void);
const char* ptn_version(void);
const char* ptn_last_error(void);
/* number of kernel launches issued by this library since load (diagnostics) */
uint64_t ptn_launch_count(void);

/* Tuning knobs (process-wide). They are read when an entry point chooses its
 * launch shape on the host, so a CUDA graph keeps the values it was captured
 * with; workspace queries read them too (query and call under the same values).
 *   PTN_TUNE_TC_SPLIT_WAVES    split-K of the tensor-core GEMM aims at this many
 *                              waves of CTAs (0..16, default 1; never fewer
 *                              splits than exact integer accumulation needs)
 *   PTN_TUNE_ZGEMM_SPLIT_WAVES split-K target of the FP64 GEMM (0..16, default 2;
 *                              0 = no split-K)
 *   PTN_TUNE_LARFB_TILE        QR block update: 0 register-tiled FMA-only kernels
 *                              (default); 1..5 the earlier three-pass kernels with
 *                              tile 1 16x16, 2 32x16, 3 32x32, 4 64x32 (rows x
 *                              columns) or 5 chosen per call
 *   PTN_TUNE_QR_CLUSTER        largest thread-block cluster of the QR panel: 0 the
 *                              device's (default; at least 32 rows per CTA), or 1..16
 *   PTN_TUNE_KRYLOV_FUSED      1 (default): each Lanczos step on vectors of at least 2^18
 *                              entries is one cooperative launch (dot, update, norm, scale
 *                              with two grid barriers, half the memory traffic); 0: three
 *                              launches. Runs that share the GPU with concurrent work on
 *                              other streams set 0.
 *   PTN_TUNE_QR_PANEL          QR panel kernel: 0 (default) two warps per 32-row group
 *                              (even / odd columns, one per SM sub-partition for 64-row
 *                              CTAs), select-free products summed through shared memory,
 *                              next pivot's norm published before the other updates;
 *                              3 the same layout with a shuffle reduce-scatter; 1 the
 *                              earlier one-warp-per-row-group panel; 2 that panel with
 *                              the reflector scalars and the cluster gather in one warp.
 *   PTN_TUNE_TC_PERSISTENT     0 (default): the tensor-core GEMM runs one CTA per (tile,
 *                              K split) unit; 1: one CTA per SM over all units, the next
 *                              unit's loads and MMAs overlapping the current one's
 *                              epilogue (same results bit for bit; measured slower on
 *                              dense data).
 *   PTN_TUNE_TC_SKIP_ZERO      1: the digit conversion flags the all-zero (tile, K block)
 *                              cells of each operand and the GEMM (persistent form) skips
 *                              them (quantum-number block sparsity, exact); 0 (default):
 *                              every block is multiplied (the 128 x 96 tiles are coarser
 *                              than the sectors at bonds up to 256: no measured gain).
 * Used by the batched driver's autotuner (no reference counterpart). */
enum {
  PTN_TUNE_TC_SPLIT_WAVES = 0,
  PTN_TUNE_ZGEMM_SPLIT_WAVES = 1,
  PTN_TUNE_LARFB_TILE = 2,
  PTN_TUNE_QR_CLUSTER = 3,
  PTN_TUNE_KRYLOV_FUSED = 4,
  PTN_TUNE_QR_PANEL = 5,
  PTN_TUNE_TC_PERSISTENT = 6,
  PTN_TUNE_TC_SKIP_ZERO = 7,
  PTN_TUNE_COUNT = 8
};
ptn_status ptn_tune_set(int key, int value);
int ptn_tune_get(int key);
/* Live kernel timing. ptn_prof_start(mask) clears the record and, for every
 * kind k with bit k set (0 FP64 GEMM, 1 tensor-core GEMM, 2 MPO stage, 3 QR,
 * 4 Krylov passes), brackets each launch with CUDA events on its stream (not
 * while a stream is being captured). After synchronising, ptn_prof_read sums
 * the event intervals, the algorithmic flops and bytes and the launch count. */
void ptn_prof_start(unsigned kind_mask);
void ptn_prof_stop(void);
ptn_status ptn_prof_read(int kind, double* total_ms, double* flops, double* bytes,
                         long* launches);

/* ----------------------------------------------------------- contractions */

/* a1: out = H_eff . a, out[l2, s, r2] = sum L[l0,wl,l2] W[wl,s,t,wr] a[l0,t,r0] R[r0,wr,r2].
 * Replaces apply_local_hamiltonian, pytenet/chain_ops.py:237-279. */
size_t ptn_heff_workspace_bytes(int Dl, int d, int Dr, int chil, int chir, int prec);
ptn_status ptn_heff_apply(const ptn_c128* a, const ptn_c128* w, const ptn_c128* l,
                          const ptn_c128* r, ptn_c128* out, int Dl, int d, int Dr,
                          int chil, int chir, int prec, void* ws, size_t ws_bytes,
                          void* stream);

/* H_eff . a exactly as ptn_heff_apply with prec = PTN_PREC_FP64, but without a
 * workspace argument, for callers that cannot allocate device memory (an FFI host
 * without a CUDA allocator, a process whose device memory belongs to another
 * framework's pool, code running where allocation is forbidden). No counterpart
 * in the reference: it is an addition of this library.
 * The intermediates live in one file-scope device array of PTN_HEFF_NOALLOC_BYTES
 * that every GPU loading the library holds until the process exits; sizes with
 * 2 * Dl * max(d*chir, chil*d) * Dr * 16 bytes above it are rejected with
 * PTN_BAD_SHAPE. All calls share the array: calls that overlap on the GPU race.
 * The first call on a device looks the array up (cudaGetSymbolAddress with that
 * device current) and caches the address with the device's current context; make
 * it before any stream capture. A later call under another context (after
 * cudaDeviceReset) looks it up again. It allocates nothing. */
#define PTN_HEFF_NOALLOC_BYTES (32u << 20)
size_t ptn_heff_noalloc_capacity_bytes(void);
ptn_status ptn_heff_apply_noalloc(const ptn_c128* a, const ptn_c128* w, const ptn_c128* l,
                                  const ptn_c128* r, ptn_c128* out, int Dl, int d, int Dr,
                                  int chil, int chir, void* stream);

/* a2: out = zero-site H_eff . c, out[l2, r2] = sum L[l0,w,l2] c[l0,r0] R[r0,w,r2].
 * Replaces apply_local_bond_contraction, pytenet/chain_ops.py:282-317. */
size_t ptn_bond_workspace_bytes(int Dl, int Dr, int chi, int prec);
ptn_status ptn_bond_apply(const ptn_c128* c, const ptn_c128* l, const ptn_c128* r,
                          ptn_c128* out, int Dl, int Dr, int chi, int prec, void* ws,
                          size_t ws_bytes, void* stream);

/* a3: l_next[ra, wr, rb] = sum a[l0,s,ra] W[wl,t,s,wr] l[l0,wl,l2] conj(b[l2,t,rb]).
 * Replaces contraction_operator_step_left, pytenet/chain_ops.py:60-99. */
size_t ptn_env_workspace_bytes(int Dl, int d, int Dr, int chil, int chir, int prec);
ptn_status ptn_env_step_left(const ptn_c128* a, const ptn_c128* b, const ptn_c128* w,
                             const ptn_c128* l, ptn_c128* l_next, int Dl, int d, int Dr,
                             int chil, int chir, int prec, void* ws, size_t ws_bytes,
                             void* stream);

/* a4: r_next[la, wl, lb] = sum a[la,s,r0] W[wl,t,s,wr] r[r0,wr,r2] conj(b[lb,t,r2]).
 * Replaces contraction_operator_step_right, pytenet/chain_ops.py:16-57. */
ptn_status ptn_env_step_right(const ptn_c128* a, const ptn_c128* b, const ptn_c128* w,
                              const ptn_c128* r, ptn_c128* r_next, int Dl, int d, int Dr,
                              int chil, int chir, int prec, void* ws, size_t ws_bytes,
                              void* stream);

/* General complex128 GEMM, C = alpha op(A) op(B) + beta C, row-major, op in
 * 'N','T','C','H'. Used for the tensordot steps of the sweep (absorbing the bond
 * matrix into the neighbouring site, pytenet/tdvp.py:84,112). */
size_t ptn_zgemm_workspace_bytes(int M, int N, int K, int batch);
ptn_status ptn_zgemm(char opA, char opB, int M, int N, int K, ptn_c128 alpha,
                     const ptn_c128* A, long lda, long strideA, const ptn_c128* B, long ldb,
                     long strideB, ptn_c128 beta, ptn_c128* C, long ldc, long strideC,
                     int batch, void* ws, size_t ws_bytes, void* stream);

/* C = A B for row-major complex A (M x K, leading dim lda) and B (K x N, ldb) on the
 * tensor cores: fixed-point BF16 digit products (the arithmetic of
 * PTN_PREC_SPLIT_BF16), FP64 output. */
size_t ptn_zgemm_split_bf16_workspace_bytes(int M, int N, int K);
ptn_status ptn_zgemm_split_bf16(const ptn_c128* A, long lda, const ptn_c128* B, long ldb,
                                ptn_c128* C, long ldc, int M, int N, int K, void* ws,
                                size_t ws_bytes, void* stream);
/* Sticky error code of the tensor-core kernels (1-3: a bounded wait expired in
 * the producer / MMA / epilogue role), then reset to 0. Synchronises the device. */
int ptn_tc_error(void);

/* ------------------------------------------------------------ Krylov core
 * lanczos_iteration / expm_krylov / eigh_krylov, pytenet/krylov.py:12-150.
 * The caller owns `V`, a (maxiter, n) complex buffer of Lanczos vectors, and a
 * state buffer of ptn_krylov_state_bytes() bytes (ptn_krylov_state followed by
 * reduction scratch). A generic Lanczos run with any operator is:
 *   ptn_krylov_start(vstart -> V[0]);
 *   for j in 0..numiter-2: { V[j+1] = A V[j];  ptn_krylov_step(j); }
 *   V[numiter] (or any n-vector buffer w) = A V[numiter-1]; ptn_krylov_last(w);
 *   ptn_krylov_expm_coef(dt) or ptn_krylov_eigh_coef(); ptn_krylov_combine -> out.
 * After a breakdown every later step is a device-side no-op; the operator
 * launches can test `stopped` through ptn_krylov_stop_flag(). */
size_t ptn_krylov_state_bytes(void);
const int32_t* ptn_krylov_stop_flag(const void* state);
ptn_status ptn_krylov_start(void* state, const ptn_c128* vstart, ptn_c128* V, long n,
                            int maxiter, void* stream);
ptn_status ptn_krylov_step(void* state, ptn_c128* V, long n, int j, void* stream);
ptn_status ptn_krylov_last(void* state, const ptn_c128* V, const ptn_c128* w, long n, int j,
                           void* stream);
ptn_status ptn_krylov_expm_coef(void* state, double dt_re, double dt_im, void* stream);
ptn_status ptn_krylov_eigh_coef(void* state, void* stream);
ptn_status ptn_krylov_combine(const void* state, const ptn_c128* V, long n, ptn_c128* out,
                              void* stream);
/* eigh_tridiag (pytenet/krylov.py:142-150) of the current run: eigenvalues
 * ascending into evals[m_used], eigenvectors into evecs[m_used * m_used] with
 * evecs[k * m_used + j] = U[k][j]. */
ptn_status ptn_krylov_tridiag_eig(const void* state, double* evals, double* evecs, void* stream);

/* a7 + a10 fused: a <- expm(dt H_eff) a with `numiter` Lanczos steps, H_eff the
 * site operator of ptn_heff_apply; dt already carries the sign (the reference
 * passes -dt, pytenet/tdvp.py:223-229). V holds (numiter + 1) vectors of n =
 * Dl*d*Dr. The whole step runs on the stream without host synchronisation. */
size_t ptn_site_step_workspace_bytes(int Dl, int d, int Dr, int chil, int chir, int prec);
ptn_status ptn_expm_site(ptn_c128* a, const ptn_c128* w, const ptn_c128* l, const ptn_c128* r,
                         int Dl, int d, int Dr, int chil, int chir, double dt_re, double dt_im,
                         int numiter, int prec, ptn_c128* V, void* state, void* ws,
                         size_t ws_bytes, void* stream);
/* zero-site version (pytenet/tdvp.py:232-238); c is (Dl, Dr). */
size_t ptn_bond_step_workspace_bytes(int Dl, int Dr, int chi, int prec);
ptn_status ptn_expm_bond(ptn_c128* c, const ptn_c128* l, const ptn_c128* r, int Dl, int Dr,
                         int chi, double dt_re, double dt_im, int numiter, int prec,
                         ptn_c128* V, void* state, void* ws, size_t ws_bytes, void* stream);
/* Learned Lanczos depth for the fused steps (ptn_expm_site_ex / ptn_expm_bond_ex).
 * After the first Lanczos iteration a 12-64-64-1 MLP (ptn_mlp_*) predicts the
 * depth m_target from: site position, log2 bond dimensions, step kind, the
 * scale |dt| |H v0|, and |dt| alpha_0..3 / beta_0..2 of the previous run at the
 * same site. At depth m_target the a-posteriori estimate
 * beta_m |e_m^T exp(dt T_m) e_1| / |v| is evaluated on the device; if it is
 * <= tol the run ends there, otherwise it continues to the full numiter (the
 * fixed-depth method). No entry point of the reference corresponds to this. */
typedef struct {
  const float* params;   /* MLP parameters on the device, or NULL (fixed depth, features only) */
  float* history;        /* device [nslots][8]: previous alpha_0..3, beta_0..2, valid flag */
  int slot;              /* history slot of this local step, e.g. 2*site + kind */
  int site, nsites, kind;/* kind 0: site step, 1: bond step */
  double tol;            /* relative residual tolerance of the early exit */
  double* log;           /* device training-record buffer [capacity][PTN_DEPTH_RECORD], or NULL */
  int* log_count;        /* device record counter */
  int log_capacity;
  int check_from;        /* with params == NULL: > 0 tests the estimate after every iteration
                            from this depth on (at least 2) with no network, the residual-only
                            criterion; 0 keeps the fixed depth */
} ptn_depth_ctx;
#define PTN_DEPTH_RECORD 64   /* doubles per record: 12 features, alpha[24], beta[24], nrm, dt re/im, m_used */
ptn_status ptn_expm_site_ex(ptn_c128* a, const ptn_c128* w, const ptn_c128* l, const ptn_c128* r,
                            int Dl, int d, int Dr, int chil, int chir, double dt_re, double dt_im,
                            int numiter, int prec, const ptn_depth_ctx* depth, ptn_c128* V,
                            void* state, void* ws, size_t ws_bytes, void* stream);
ptn_status ptn_expm_bond_ex(ptn_c128* c, const ptn_c128* l, const ptn_c128* r, int Dl, int Dr,
                            int chi, double dt_re, double dt_im, int numiter, int prec,
                            const ptn_depth_ctx* depth, ptn_c128* V, void* state, void* ws,
                            size_t ws_bytes, void* stream);
/* Labels of recorded runs: the smallest depth m <= m_max whose estimate
 * beta_{m-1} |e_m^T exp(dt T_m) e_1| is <= tol (m_max if none). */
ptn_status ptn_depth_labels(const double* log, int count, int m_max, double tol, int* labels,
                            void* stream);

/* MLP (12 -> 64 -> 64 -> 1, FP32, GELU) for the learned depth: forward pass,
 * mean-squared-loss gradient (deterministic batch reduction) and Adam update. */
int ptn_mlp_param_count(void);
size_t ptn_mlp_workspace_bytes(int batch);
ptn_status ptn_mlp_forward(const float* params, const float* X, int batch, float* Y, void* stream);
ptn_status ptn_mlp_grad(const float* params, const float* X, const float* T, int batch,
                        float* grad, float* loss, void* ws, size_t ws_bytes, void* stream);
ptn_status ptn_mlp_adam(float* params, const float* grad, float* m, float* v, float lr,
                        float beta1, float beta2, float eps, int step, void* stream);

/* a9 + a11: a <- lowest Ritz vector of H_eff (pytenet/dmrg.py:181-189); the Ritz
 * value is left in state->eval0. */
ptn_status ptn_eigh_site(ptn_c128* a, const ptn_c128* w, const ptn_c128* l, const ptn_c128* r,
                         int Dl, int d, int Dr, int chil, int chir, int numiter, int prec,
                         ptn_c128* V, void* state, void* ws, size_t ws_bytes, void* stream);

/* -------------------------------------------------------------------- QR
 * a12: Householder QR with LAPACK's reflector convention (real diagonal of R,
 * beta = -sign(Re alpha) |x|), as numpy.linalg.qr(mode="reduced") computes it;
 * the per-block kernel of block_sparse_qr, pytenet/block_sparse_util.py:106-180.
 * `a` (m x n, row-major, lda = n) is overwritten. Q is m x k, R is k x n,
 * k = min(m, n), written with leading dimensions ldq / ldr. */
size_t ptn_qr_workspace_bytes(int m, int n);
ptn_status ptn_qr(ptn_c128* a, int m, int n, ptn_c128* q, long ldq, ptn_c128* r, long ldr,
                  void* ws, size_t ws_bytes, void* stream);
/* dst[p*nc + c] = src[row_off[p] + col_off[c]] (gather one quantum-number block,
 * with any transposition folded into the offsets) */
ptn_status ptn_gather(const ptn_c128* src, const int64_t* row_off, const int64_t* col_off,
                      int nr, int nc, ptn_c128* dst, void* stream);
/* dst[row_off[p] + col_off[c]] = src[p*ld + c] */
ptn_status ptn_scatter(const ptn_c128* src, long ld, const int64_t* row_off,
                       const int64_t* col_off, int nr, int nc, ptn_c128* dst, void* stream);
/* Norm convention of MPS.orthonormalize (pytenet/mps.py:170-176): nrm = Re r00;
 * if nrm < 0 the n entries of `a` are negated and nrm = -nrm; *nrm_out = nrm. */
ptn_status ptn_sign_fix(ptn_c128* a, long n, const ptn_c128* r00, double* nrm_out, void* stream);
/* out[i] = alpha * in[i] (complex), n elements; in == out allowed */
ptn_status ptn_scale(const ptn_c128* in, ptn_c128* out, long n, ptn_c128 alpha, void* stream);
/* out[c, b, a] = in[a, b, c] for `in` of shape (n0, n1, n2): the transpose((2, 1, 0))
 * of the right-to-left sweep, pytenet/tdvp.py:95,104 */
ptn_status ptn_transpose_210(const ptn_c128* in, ptn_c128* out, int n0, int n1, int n2,
                             void* stream);

/* -------------------------------------------------------------------- SVD
 * Thin SVD a = u diag(s) vh of a complex128 matrix (m x n, row-major, leading
 * dimension lda), k = min(m, n): u is m x k (ldu), s has k entries in decreasing
 * order, vh is k x n (ldvh). One-sided Jacobi in FP64 on one CTA. Replaces the
 * numpy.linalg.svd(full_matrices=False) call per quantum-number block of
 * block_sparse_svd, pytenet/block_sparse_util.py:244-330 (used by the two-site
 * splits, pytenet/bond_ops.py:41-53 and pytenet/mps.py:538-568). Singular vectors
 * are fixed up to a phase per singular value, not necessarily LAPACK's phase.
 * `sweeps` (device int, or NULL) receives the number of Jacobi sweeps used. */
size_t ptn_svd_workspace_bytes(int m, int n);
ptn_status ptn_svd(const ptn_c128* a, int m, int n, long lda, ptn_c128* u, long ldu, double* s,
                   ptn_c128* vh, long ldvh, int* sweeps, void* ws, size_t ws_bytes,
                   void* stream);
/* a[i][j] *= s[j] (side 0) or s[i] (side 1) for a rows x cols row-major matrix
 * with leading dimension ld: distributing singular values onto a split factor
 * (the svd_distr argument of pytenet/mps.py:538-568). */
ptn_status ptn_diag_scale(ptn_c128* a, long rows, long cols, long ld, const double* s, int side,
                          void* stream);

#ifdef __cplusplus
}
#endif

#endif /* PYTENET_GB300_H */
