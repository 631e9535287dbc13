// Complex GEMM from fixed-point BF16 digits on the 5th-generation tensor cores (tcgen05, sm_103a),
// with FP64-class accuracy from exact fixed-point digit products.
//
// A complex product C = op(A) op(B) is computed as one real GEMM:
//   - the "plain" operand A is the row-major complex matrix read as real
//     (M x 2K: re/im interleaved along K), the "embedded" operand B holds each
//     complex entry z as the 2x2 real block [[Re z, -Im z], [Im z, Re z]]
//     (2N x 2K, K-major), so that the real product (M x 2N) is the complex
//     product with re/im interleaved -- i.e. the complex128 output layout;
//   - every operand row r is scaled by its own power of two 2^-e[r] (|x| < 2^e[r]
//     over the row) and cut into five signed 8-bit integer digits held exactly in
//     BF16: x = 2^(e[r]-7) * sum_i 2^(-8 i) d_i, |d_i| <= 128 (Ozaki, Ogita, Oishi
//     and Rump's error-free splitting, in fixed point per row);
//   - a digit product is an integer of at most 14 bits; the products of one level
//     s = i + j (pairs with s <= 4, fifteen in all) go to that level's FP32
//     accumulator in tensor memory (5 levels x 96 columns of the 512).
// Exactness, whatever the signs of the data:
//   - levels 0..2 (weights 1, 2^-8, 2^-16 of the leading one) restart every
//     FLUSH_KB K blocks (320 reals): at most 3 pairs x 2^14 x 320 < 2^24, so
//     every partial sum is an exactly represented integer. The epilogue warps
//     drain each period into int64 registers (exact) while the tensor cores go on
//     with the level 3..4 products of the next K block;
//   - levels 3..4 (weights 2^-24, 2^-32) accumulate over the whole split of at
//     most MAX_K_SPLIT = 4096 reals in FP32. Their rounding, even with every
//     product of one sign and a rounding after every 4 products, stays below
//     2^-45 K (3e-11 at K = 4096 per split after the split-K sum) relative to
//     max|row| max|col| K; for data of mixed signs it is far smaller.
//   - the epilogue combines the int64 sum of levels 0..2 with levels 3..4 in
//     int64 and applies the row and column scales 2^(eA[m] + eB[n] - 46) with one
//     rounding to FP64. Split-K partials are FP64.
// What remains is the truncation after the fifth digit and the dropped level-5
// products, ~2^-39 of the row maxima: FP64-class for the sweep's purposes.
//
// Kernel: one 128 x 96 output tile per CTA (UMMA M=128, N=96, K=16), BK=32
// (one 64-byte swizzle atom of BF16). A pipeline stage is one K block with all
// five digit planes of both operands (3-D TMA boxes of 32 x 128 x 5 and
// 32 x 96 x 5, 70 KB), so every plane is fetched once and feeds the 15 digit
// pairs x 2 MMAs of that K block; 3 stages with full/empty mbarriers. Warp 0 lane 0
// issues TMA, warp 1 lane 0 issues tcgen05.mma and tcgen05.commit, warps 2..9 drain
// the accumulators with tcgen05.ld (warp w owns TMEM lanes 32*(w%4).. and half of the
// 96 columns) and write FP64 complex results (or FP64 split-K partials). Every
// mbarrier wait is bounded: on expiry the kernel records an error code, stops
// issuing work, lets its copies in flight land and still frees its TMEM.
#include "ptn_common.cuh"
#include <cuda.h>
#include <cuda_bf16.h>
#include <algorithm>
#include <climits>
#include <mutex>
#include <vector>

namespace ptn {

void note_launches(int n);

namespace {

constexpr int BM = 128, BN = 96, BK = 32;
constexpr int STAGES = 3;
constexpr int NDIGIT = 5;                 // digits per operand value
constexpr int NPAIR = 15;                 // digit pairs (i, j) with i + j <= 4
constexpr int NLEVEL = 5;
constexpr int EXACT_PAIRS = 6;            // pairs of levels 0..2 (first in the pair tables)
constexpr int FLUSH_KB = 10;              // K blocks per exact period of levels 0..2
// operand rows without a non-zero entry carry an exponent below this (the digit
// converter fills the exponent arrays with 0x80 bytes before its max pass)
constexpr int EXP_NONE = -2000;
constexpr int A_TILE = BM * BK * 2;           // one digit plane of A: 8 KB
constexpr int B_TILE = BN * BK * 2;
constexpr int A_STAGE = NDIGIT * A_TILE;       // all five planes
constexpr int B_STAGE = NDIGIT * B_TILE;
constexpr int STAGE_BYTES = A_STAGE + B_STAGE; // 70 KB
// real K entries per split: bounds the FP32 rounding of levels 3..4 and keeps the
// int64 sums of levels 0..2 below 2^63 (at most 13 periods of < 2^40.01 each,
// times 2^16 at the end: < 2^60)
constexpr int MAX_K_SPLIT = 4096;
constexpr int EPI_WARPS = 8;
constexpr int EPI_COLS = BN / 2;              // columns per epilogue warp (two per lane quadrant)
constexpr int THREADS = 64 + 32 * EPI_WARPS;
constexpr int TMEM_USED = NLEVEL * BN;   // 480: one accumulator per level
constexpr int TMEM_COLS = 512;           // allocation (a power of two)
constexpr int SMEM_BYTES = STAGES * STAGE_BYTES + 1024 + 512;   // + barriers, column exponents
constexpr long WAIT_LIMIT = 1L << 22;
// kind::f16 instruction descriptor: FP32 accumulate (bit 4), A and B BF16
// (bits 7, 10), both K-major, N >> 3 at bit 17, M >> 4 at bit 24.
constexpr uint32_t IDESC = (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(BN >> 3) << 17) |
                           ((uint32_t)(BM >> 4) << 24);
static_assert(TMEM_USED <= TMEM_COLS, "tensor memory holds 512 columns");
static_assert(SMEM_BYTES <= 227 * 1024, "shared memory per CTA");
// every partial sum of levels 0..2 in a period is an integer below 2^24
static_assert(3L * (1L << 14) * FLUSH_KB * BK < (1L << 24), "exact period of levels 0..2");
static_assert(MAX_K_SPLIT % BK == 0 && EPI_COLS % 16 == 0, "tiling");

struct TcArgs {
  int M, N;            // output rows, real output columns (2 x complex columns)
  int nkb;             // K blocks (of BK)
  int kb_per_split, splits;
  const int* ea;       // row exponents of A (M), below EXP_NONE for an all-zero row
  const int* eb;       // exponents of B per complex column (N / 2)
  double2* out;        // complex output element (m, c) at out[m * ldm + c * ldn]
  long ldm, ldn;
  int accumulate;      // out += result instead of out = result
  double* part;        // split-K partials [splits][M][N], or null
  int* err;
  const int* skip;
  // non-zero flags of (128-row tile of A, K block) and (96-row tile of B, K block),
  // fk K blocks per row of flags after a validity byte, or null: the persistent
  // kernel skips every K block where either operand tile is zero (exact: those
  // products are zero); flags whose validity byte is 0 are ignored
  const unsigned char* fa;
  const unsigned char* fb;
  int fk;
};

// digit pairs, grouped by level; the first pair of each level starts its accumulator
__constant__ int c_pair_a[NPAIR] = {0, 0, 1, 0, 1, 2, 0, 1, 2, 3, 0, 1, 2, 3, 4};
__constant__ int c_pair_b[NPAIR] = {0, 1, 0, 2, 1, 0, 3, 2, 1, 0, 4, 3, 2, 1, 0};
__constant__ int c_pair_l[NPAIR] = {0, 1, 1, 2, 2, 2, 3, 3, 3, 3, 4, 4, 4, 4, 4};

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)),
               "r"(bytes)
               : "memory");
}

__device__ __forceinline__ void mbar_arrive(uint64_t* bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}

// bounded wait on the phase with parity `parity`; false on expiry
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity) {
  const uint32_t a = smem_u32(bar);
  for (long it = 0; it < WAIT_LIMIT; ++it) {
    uint32_t done;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
        " selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(done)
        : "r"(a), "r"(parity)
        : "memory");
    if (done) return true;
  }
  return false;
}

// bounded wait that also gives up once another role raised the CTA's abort flag
__device__ __forceinline__ bool mbar_wait_or_abort(uint64_t* bar, uint32_t parity,
                                                   const int* abort_flag) {
  const uint32_t a = smem_u32(bar);
  for (long it = 0; it < WAIT_LIMIT; ++it) {
    uint32_t done;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
        " selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(done)
        : "r"(a), "r"(parity)
        : "memory");
    if (done) return true;
    if (*(volatile const int*)abort_flag) return false;
  }
  return false;
}

__device__ __forceinline__ void tma_load_3d(void* dst, const CUtensorMap* tm, int x, int y, int z,
                                            uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.tensor.3d.shared::cluster.global.mbarrier::complete_tx::bytes"
      " [%0], [%1, {%2, %3, %4}], [%5];" ::"r"(smem_u32(dst)),
      "l"(reinterpret_cast<uint64_t>(tm)), "r"(x), "r"(y), "r"(z), "r"(smem_u32(bar))
      : "memory");
}

// shared-memory matrix descriptor: K-major, 64-byte swizzle (layout type 4), rows of
// 64 B, 8-row groups 512 B apart
__device__ __forceinline__ uint64_t sdesc(uint32_t saddr) {
  uint64_t d = (uint64_t)((saddr >> 4) & 0x3FFFu);
  d |= (uint64_t)1 << 16;
  d |= (uint64_t)((8 * BK * 2) >> 4) << 32;
  d |= (uint64_t)1 << 46;
  d |= (uint64_t)4 << 61;
  return d;
}

__device__ __forceinline__ void umma(uint32_t tmem, uint64_t ad, uint64_t bd, uint32_t acc) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
      " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(tmem),
      "l"(ad), "l"(bd), "r"(IDESC), "r"(acc)
      : "memory");
}

__device__ __forceinline__ void umma_commit(uint64_t* bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                   smem_u32(bar))
               : "memory");
}

// issue one 32-lane x 16-column load from tensor memory (complete at tmem_wait_ld)
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, uint32_t (&v)[16]) {
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15},"
      " [%16];"
      : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]),
        "=r"(v[7]), "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]),
        "=r"(v[14]), "=r"(v[15])
      : "r"(taddr));
}

// issue one 32-lane x 8-column load from tensor memory (complete at tmem_wait_ld)
__device__ __forceinline__ void tmem_ld8(uint32_t taddr, uint32_t (&v)[8]) {
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
      : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]),
        "=r"(v[7])
      : "r"(taddr));
}

__device__ __forceinline__ void tmem_wait_ld() {
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
}

// keeps every use of v after the preceding tcgen05.wait::ld: the empty volatile
// statements stay in order behind it and redefine the registers
template <int N>
__device__ __forceinline__ void after_wait(uint32_t (&v)[N]) {
#pragma unroll
  for (int i = 0; i < N; ++i) asm volatile("" : "+r"(v[i]));
}

// one period of levels 0..2 as an exact integer: 2^16 L0 + 2^8 L1 + L2, the L
// integer-valued FP32 sums below 2^24 (|result| < 2^40.01)
__device__ __forceinline__ long long exact_levels(uint32_t a0, uint32_t a1, uint32_t a2) {
  const long long i0 = __float2int_rn(__uint_as_float(a0));
  const long long i1 = __float2int_rn(__uint_as_float(a1));
  const long long i2 = __float2int_rn(__uint_as_float(a2));
  return i0 * 65536LL + i1 * 256LL + i2;
}

// (2^16 x + 2^8 L3 + L4) 2^sh as FP64: x the int64 sum of the exact periods of
// levels 0..2, L3 / L4 integer-valued FP32 sums. Integer arithmetic throughout
// (the CUDA-core FP64 rate of this part is low): the only FP64 operation is the
// int64 -> double conversion (the one rounding); the power of two goes into the
// exponent field directly (ldexp only where that would leave the normal range).
__device__ __forceinline__ double finish_value(long long x, uint32_t a3, uint32_t a4, int sh) {
  const long long v = x * 65536LL + __float2ll_rn(__uint_as_float(a3)) * 256LL +
                      __float2ll_rn(__uint_as_float(a4));   // |v| < 2^61
  if (v == 0) return 0.0;
  const double r = (double)v;
  const long long b = __double_as_longlong(r);
  const int e = (int)((b >> 52) & 0x7FF) + sh;
  if (e > 0 && e < 2047) return __longlong_as_double(b + ((long long)sh << 52));
  return ldexp(r, sh);
}

// K blocks [k0, k1) of a unit (at most MAX_K_SPLIT / BK = 128) that have both
// operand tiles non-zero, as four 32-bit masks; all lanes of the warp take part
__device__ __forceinline__ int unit_mask(const TcArgs& p, int m0, int n0, int k0, int k1, int lane,
                                         uint32_t (&mk)[4]) {
  if (p.fa == nullptr) {   // dense: every block of the unit (uniform over the launch)
    mk[0] = mk[1] = mk[2] = mk[3] = 0xffffffffu;
    return k1 - k0;
  }
  int n = 0;
#pragma unroll
  for (int w = 0; w < 4; ++w) {
    const int k = k0 + w * 32 + lane;
    bool act = k < k1;
    if (act && p.fa != nullptr && p.fa[0] != 0 && p.fb[0] != 0)
      act = p.fa[1 + (long)(m0 / BM) * p.fk + k] != 0 && p.fb[1 + (long)(n0 / BN) * p.fk + k] != 0;
    mk[w] = __ballot_sync(0xffffffffu, act);
    n += __popc(mk[w]);
  }
  return n;
}

// bit j of the unit mask (selects, no dynamically indexed register array); always
// set when the GEMM has no zero-tile flags
__device__ __forceinline__ bool mask_bit(const uint32_t (&mk)[4], int j) {
  const uint32_t w = (j < 64) ? ((j < 32) ? mk[0] : mk[1]) : ((j < 96) ? mk[2] : mk[3]);
  return (w >> (j & 31)) & 1u;
}

// the MMAs of digit pairs [P0, P1) of one K block (stage addresses a0 / b0); the
// first pair of a level starts its accumulator when `restart`
template <int P0, int P1>
__device__ __forceinline__ void issue_pairs(uint32_t tmem, uint32_t a0, uint32_t b0, bool restart) {
#pragma unroll
  for (int pr = P0; pr < P1; ++pr) {
    const uint32_t acc_col = (uint32_t)(c_pair_l[pr] * BN);
    const bool first_of_level = restart && (pr == 0 || c_pair_l[pr] != c_pair_l[pr - 1]);
    const uint32_t ap = a0 + (uint32_t)(c_pair_a[pr] * A_TILE);
    const uint32_t bp = b0 + (uint32_t)(c_pair_b[pr] * B_TILE);
#pragma unroll
    for (int k = 0; k < BK / 16; ++k)
      umma(tmem + acc_col, sdesc(ap + k * 32), sdesc(bp + k * 32),
           (first_of_level && k == 0) ? 0u : 1u);
  }
}

// 10 warps: two of the SM's four sub-partitions hold three of them, which caps a
// thread at 168 registers (16K registers per sub-partition)
__global__ void __launch_bounds__(THREADS, 1)
    tc_gemm_kernel(const __grid_constant__ CUtensorMap tmA, const __grid_constant__ CUtensorMap tmB,
                   const TcArgs p) {
  if (p.skip != nullptr && *p.skip != 0) return;  // uniform: before any barrier or allocation
  extern __shared__ uint8_t smem_raw[];
  uint8_t* smem = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) &
                                             ~uintptr_t(1023));
  uint8_t* sA = smem;
  uint8_t* sB = smem + STAGES * A_STAGE;
  uint64_t* full = reinterpret_cast<uint64_t*>(smem + STAGES * STAGE_BYTES);
  uint64_t* empty = full + STAGES;
  uint64_t* tfull = empty + STAGES;   // levels 0..2 of a period are complete
  uint64_t* tempty = tfull + 1;       // the epilogue has drained levels 0..2
  uint64_t* tdone = tempty + 1;       // every MMA of the split is complete
  uint32_t* tslot = reinterpret_cast<uint32_t*>(tdone + 1);
  int* abort_flag = reinterpret_cast<int*>(tslot + 1);
  int* s_eb = abort_flag + 1;   // column exponents of this tile (BN / 2 complex columns)

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int m0 = blockIdx.y * BM, n0 = blockIdx.x * BN;
  const int split = blockIdx.z;
  const int kb0 = split * p.kb_per_split;
  const int kb1 = min(p.nkb, kb0 + p.kb_per_split);
  // one pipeline step per K block; exact periods of FLUSH_KB steps
  const int it0 = kb0, it1 = kb1;
  const int nper = (it1 > it0) ? (it1 - it0 + FLUSH_KB - 1) / FLUSH_KB : 0;

  if (threadIdx.x == 0) {
    for (int s = 0; s < STAGES; ++s) {
      mbar_init(&full[s], 1);
      mbar_init(&empty[s], 1);
    }
    mbar_init(tfull, 1);
    mbar_init(tempty, EPI_WARPS);
    mbar_init(tdone, 1);
    *abort_flag = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  }
  if (warp == 1) {
    __syncwarp();
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                     smem_u32(tslot)),
                 "r"(TMEM_COLS)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = *tslot;

  if (warp == 0 && lane == 0) {
    // ---------------- TMA producer
    int issued = 0;
    for (int it = it0, i = 0; it < it1; ++it, ++i) {
      const int s = i % STAGES;
      const uint32_t ph = (uint32_t)(i / STAGES) & 1u;
      if (i >= STAGES && !mbar_wait_or_abort(&empty[s], ph ^ 1u, abort_flag)) {
        atomicExch(p.err, 1);
        *(volatile int*)abort_flag = 1;
        break;
      }
      if (*(volatile int*)abort_flag) break;
      mbar_expect_tx(&full[s], STAGE_BYTES);
      tma_load_3d(sA + s * A_STAGE, &tmA, it * BK, m0, 0, &full[s]);
      tma_load_3d(sB + s * B_STAGE, &tmB, it * BK, n0, 0, &full[s]);
      ++issued;
    }
    if (*(volatile int*)abort_flag) {
      // drain: let the copies still in flight land before the CTA retires (bounded)
      for (int i = max(0, issued - STAGES); i < issued; ++i)
        mbar_wait(&full[i % STAGES], (uint32_t)(i / STAGES) & 1u);
    }
  } else if (warp == 1 && lane == 0) {
    // ---------------- MMA issuer
    // Per K block: the level 0..2 pairs, then the level 3..4 pairs. At the end of
    // an exact period (or of the split) the level 0..2 MMAs are committed to tfull
    // before the level 3..4 MMAs are issued; the first K block of the next period
    // issues its level 3..4 pairs before it waits for the epilogue to release the
    // level 0..2 columns, so the tensor cores stay busy while they are drained.
    int issued = 0;
    for (int it = it0, i = 0; it < it1; ++it, ++i) {
      const int s = i % STAGES;
      const uint32_t ph = (uint32_t)(i / STAGES) & 1u;
      if (!mbar_wait_or_abort(&full[s], ph, abort_flag)) {
        atomicExch(p.err, 2);
        *(volatile int*)abort_flag = 1;
        break;
      }
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      const uint32_t a0 = smem_u32(sA + s * A_STAGE), b0 = smem_u32(sB + s * B_STAGE);
      const int q = i / FLUSH_KB;
      const bool period_start = (i % FLUSH_KB) == 0;
      const bool period_end = ((i + 1) % FLUSH_KB) == 0 || it + 1 == it1;
      if (period_start && q > 0) {
        issue_pairs<EXACT_PAIRS, NPAIR>(tmem, a0, b0, false);
        if (!mbar_wait_or_abort(tempty, (uint32_t)(q - 1) & 1u, abort_flag)) {
          atomicExch(p.err, 2);
          *(volatile int*)abort_flag = 1;
          umma_commit(&empty[s]);
          break;
        }
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        issue_pairs<0, EXACT_PAIRS>(tmem, a0, b0, true);
        if (period_end) umma_commit(tfull);
      } else {
        issue_pairs<0, EXACT_PAIRS>(tmem, a0, b0, period_start);
        if (period_end) umma_commit(tfull);
        issue_pairs<EXACT_PAIRS, NPAIR>(tmem, a0, b0, i == 0);
      }
      umma_commit(&empty[s]);
      ++issued;
    }
    if (issued > 0) umma_commit(tdone);
    else mbar_arrive(tdone);
  } else if (warp >= 2) {
    // ---------------- epilogue: exact periods of levels 0..2 -> int64, then
    // levels 3..4 -> FP64 -> global. Warp w reads TMEM lanes 32 (w % 4).. and
    // the columns [h * 48, h * 48 + 48) of every level, h = (w - 2) / 4.
    // Exponents first, while the main loop runs: the row's in a register, the
    // tile's column exponents in shared memory (epilogue warps' named barrier).
    const int g = warp & 3;
    const int h = (warp - 2) >> 2;
    const int row = m0 + 32 * g + lane;
    const int ea = (row < p.M) ? p.ea[row] : EXP_NONE - 1;
    if (warp == 2)
      for (int c = lane; c < BN / 2; c += 32) {
        const int col = (n0 >> 1) + c;
        s_eb[c] = (2 * col < p.N) ? p.eb[col] : EXP_NONE - 1;
      }
    asm volatile("bar.sync 1, 256;" ::: "memory");
    const uint32_t tl = tmem + ((uint32_t)(32 * g) << 16) + (uint32_t)(h * EPI_COLS);
    long long acc[EPI_COLS];
#pragma unroll
    for (int j = 0; j < EPI_COLS; ++j) acc[j] = 0;
    bool ok = true;
    for (int q = 0; q < nper && ok; ++q) {
      if (!mbar_wait_or_abort(tfull, (uint32_t)q & 1u, abort_flag)) {
        ok = false;
        break;
      }
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
#pragma unroll
      for (int c0 = 0; c0 < EPI_COLS; c0 += 8) {
        uint32_t v0[8], v1[8], v2[8];
        __syncwarp();
        tmem_ld8(tl + (uint32_t)c0, v0);
        tmem_ld8(tl + (uint32_t)(BN + c0), v1);
        tmem_ld8(tl + (uint32_t)(2 * BN + c0), v2);
        tmem_wait_ld();
        after_wait(v0);
        after_wait(v1);
        after_wait(v2);
        if (c0 + 8 == EPI_COLS) {
          // every level 0..2 column of this warp is in registers: release them
          asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
          __syncwarp();
          if (lane == 0) mbar_arrive(tempty);
        }
#pragma unroll
        for (int j = 0; j < 8; ++j) acc[c0 + j] += exact_levels(v0[j], v1[j], v2[j]);
      }
    }
    if (ok && nper > 0 && !mbar_wait_or_abort(tdone, 0, abort_flag)) ok = false;
    if (!ok && !*(volatile int*)abort_flag) atomicExch(p.err, 3);
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const bool have = ok && nper > 0 && !*(volatile int*)abort_flag;
#pragma unroll
    for (int c0 = 0; c0 < EPI_COLS; c0 += 16) {
      uint32_t v3[16], v4[16];
      __syncwarp();
      tmem_ld16(tl + (uint32_t)(3 * BN + c0), v3);
      tmem_ld16(tl + (uint32_t)(4 * BN + c0), v4);
      tmem_wait_ld();
      after_wait(v3);
      after_wait(v4);
      if (row < p.M) {
#pragma unroll
        for (int j = 0; j < 16; j += 2) {
          const int cl = h * EPI_COLS + c0 + j;   // column within the tile
          const int col = n0 + cl;
          if (col >= p.N) break;
          double re = 0.0, im = 0.0;
          const int eb = s_eb[cl >> 1];
          if (have && ea > EXP_NONE && eb > EXP_NONE) {
            // value = (sum_s 2^(8 (4 - s)) level_s) 2^(ea + eb - 46), one rounding
            const int sh = ea + eb - 46;
            re = finish_value(acc[c0 + j], v3[j], v4[j], sh);
            im = finish_value(acc[c0 + j + 1], v3[j + 1], v4[j + 1], sh);
          }
          if (p.part != nullptr) {
            double2* dst = reinterpret_cast<double2*>(p.part + ((long)split * p.M + row) * p.N + col);
            *dst = make_double2(re, im);
          } else {
            double2* o = p.out + (long)row * p.ldm + (long)(col >> 1) * p.ldn;
            double2 x = make_double2(re, im);
            if (p.accumulate) {
              const double2 y = *o;
              x.x += y.x;
              x.y += y.y;
            }
            *o = x;
          }
        }
      }
    }
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (warp == 1) {
    __syncwarp();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem),
                 "r"(TMEM_COLS)
                 : "memory");
  }
}

// Persistent form of tc_gemm_kernel: one CTA per SM walks the work units
// u = blockIdx.x, blockIdx.x + gridDim.x, ... (u -> N tile fastest, then M tile,
// then K split), with the same warp roles, the same digit pairs and the same exact
// periods per unit. The stage ring, the period count of tfull / tempty and the
// unit count of tdone / tfree continue from unit to unit, so the TMA producer
// fetches the next unit's first K blocks while the current one is finished, and
// the MMA warp starts the next unit as soon as the epilogue has read the last
// accumulator columns out of tensor memory (tfree); the epilogue converts into its
// registers first and writes the outputs while the next unit's MMAs run. TMEM is
// allocated and the barriers initialised once per CTA.
__global__ void __launch_bounds__(THREADS, 1)
    tc_gemm_persistent_kernel(const __grid_constant__ CUtensorMap tmA,
                              const __grid_constant__ CUtensorMap tmB, const TcArgs p, int gx,
                              int gy, int units) {
  if (p.skip != nullptr && *p.skip != 0) return;  // uniform: before any barrier or allocation
  extern __shared__ uint8_t smem_raw[];
  uint8_t* smem = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) &
                                             ~uintptr_t(1023));
  uint8_t* sA = smem;
  uint8_t* sB = smem + STAGES * A_STAGE;
  uint64_t* full = reinterpret_cast<uint64_t*>(smem + STAGES * STAGE_BYTES);
  uint64_t* empty = full + STAGES;
  uint64_t* tfull = empty + STAGES;   // levels 0..2 of a period are complete
  uint64_t* tempty = tfull + 1;       // the epilogue has drained levels 0..2
  uint64_t* tdone = tempty + 1;       // every MMA of the unit is complete
  uint64_t* tfree = tdone + 1;        // the epilogue has read the unit's levels 3..4
  uint32_t* tslot = reinterpret_cast<uint32_t*>(tfree + 1);
  int* abort_flag = reinterpret_cast<int*>(tslot + 1);

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int G = gridDim.x;
  auto coords = [&](int u, int& m0, int& n0, int& split, int& k0, int& k1) {
    n0 = (u % gx) * BN;
    m0 = ((u / gx) % gy) * BM;
    split = u / (gx * gy);
    k0 = split * p.kb_per_split;
    k1 = min(p.nkb, k0 + p.kb_per_split);
  };

  if (threadIdx.x == 0) {
    for (int s = 0; s < STAGES; ++s) {
      mbar_init(&full[s], 1);
      mbar_init(&empty[s], 1);
    }
    mbar_init(tfull, 1);
    mbar_init(tempty, EPI_WARPS);
    mbar_init(tdone, 1);
    mbar_init(tfree, EPI_WARPS);
    *abort_flag = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  }
  if (warp == 1) {
    __syncwarp();
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                     smem_u32(tslot)),
                 "r"(TMEM_COLS)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = *tslot;

  if (warp == 0) {
    // ---------------- TMA producer (lane 0): one ring over the active K blocks of all
    // units; the whole warp forms each unit's mask
    int i = 0, issued = 0;
    bool stop = false;
    for (int u = blockIdx.x; u < units && !stop; u += G) {
      int m0, n0, split, k0, k1;
      coords(u, m0, n0, split, k0, k1);
      uint32_t mk[4];
      unit_mask(p, m0, n0, k0, k1, lane, mk);
      if (lane == 0) {
        for (int it = k0; it < k1; ++it) {
          if (!mask_bit(mk, it - k0)) continue;
          const int s = i % STAGES;
          const uint32_t ph = (uint32_t)(i / STAGES) & 1u;
          if (i >= STAGES && !mbar_wait_or_abort(&empty[s], ph ^ 1u, abort_flag)) {
            atomicExch(p.err, 1);
            *(volatile int*)abort_flag = 1;
            stop = true;
            break;
          }
          if (*(volatile int*)abort_flag) {
            stop = true;
            break;
          }
          mbar_expect_tx(&full[s], STAGE_BYTES);
          tma_load_3d(sA + s * A_STAGE, &tmA, it * BK, m0, 0, &full[s]);
          tma_load_3d(sB + s * B_STAGE, &tmB, it * BK, n0, 0, &full[s]);
          ++issued;
          ++i;
        }
      }
      stop = __shfl_sync(0xffffffffu, stop ? 1 : 0, 0) != 0;
    }
    if (lane == 0 && *(volatile int*)abort_flag) {
      // drain: let the copies still in flight land before the CTA retires (bounded)
      for (int j = issued > STAGES ? issued - STAGES : 0; j < issued; ++j)
        mbar_wait(&full[j % STAGES], (uint32_t)(j / STAGES) & 1u);
    }
  } else if (warp == 1) {
    // ---------------- MMA issuer (lane 0; same per-K-block schedule as tc_gemm_kernel
    // over the unit's active K blocks; the period index runs on across units, the
    // first unit after another waits for tfree)
    int i = 0, Q = 0, t = 0;
    bool stop = false;
    for (int u = blockIdx.x; u < units && !stop; u += G, ++t) {
      int m0, n0, split, k0, k1;
      coords(u, m0, n0, split, k0, k1);
      uint32_t mk[4];
      const int nk = unit_mask(p, m0, n0, k0, k1, lane, mk);
      if (lane == 0) {
        bool ok = true;
        if (t > 0) {
          if (!mbar_wait_or_abort(tfree, (uint32_t)(t - 1) & 1u, abort_flag)) {
            atomicExch(p.err, 2);
            *(volatile int*)abort_flag = 1;
            ok = false;
          } else {
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
          }
        }
        for (int it = k0, k = 0; ok && it < k1; ++it) {
          if (!mask_bit(mk, it - k0)) continue;
          const int s = i % STAGES;
          const uint32_t ph = (uint32_t)(i / STAGES) & 1u;
          if (!mbar_wait_or_abort(&full[s], ph, abort_flag)) {
            atomicExch(p.err, 2);
            *(volatile int*)abort_flag = 1;
            ok = false;
            break;
          }
          asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
          const uint32_t a0 = smem_u32(sA + s * A_STAGE), b0 = smem_u32(sB + s * B_STAGE);
          const int q = k / FLUSH_KB;
          const bool period_start = (k % FLUSH_KB) == 0;
          const bool period_end = ((k + 1) % FLUSH_KB) == 0 || k + 1 == nk;
          if (period_start && q > 0) {
            issue_pairs<EXACT_PAIRS, NPAIR>(tmem, a0, b0, false);
            if (!mbar_wait_or_abort(tempty, (uint32_t)(Q + q - 1) & 1u, abort_flag)) {
              atomicExch(p.err, 2);
              *(volatile int*)abort_flag = 1;
              umma_commit(&empty[s]);
              ok = false;
              break;
            }
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
            issue_pairs<0, EXACT_PAIRS>(tmem, a0, b0, true);
            if (period_end) umma_commit(tfull);
          } else {
            // a unit's first period: tfree (all of the previous unit's columns read)
            // covers the drain of that unit's last period
            issue_pairs<0, EXACT_PAIRS>(tmem, a0, b0, period_start);
            if (period_end) umma_commit(tfull);
            issue_pairs<EXACT_PAIRS, NPAIR>(tmem, a0, b0, k == 0);
          }
          umma_commit(&empty[s]);
          ++k;
          ++i;
        }
        if (ok) {
          Q += (nk + FLUSH_KB - 1) / FLUSH_KB;
          if (nk > 0) umma_commit(tdone);
          else mbar_arrive(tdone);
        }
        stop = !ok;
      }
      stop = __shfl_sync(0xffffffffu, stop ? 1 : 0, 0) != 0;
    }
  } else if (warp >= 2) {
    // ---------------- epilogue, per unit: exact periods of levels 0..2 -> int64,
    // levels 3..4 -> FP64 values in registers (then tfree), outputs -> global
    const int g = warp & 3;
    const int h = (warp - 2) >> 2;
    const uint32_t tl = tmem + ((uint32_t)(32 * g) << 16) + (uint32_t)(h * EPI_COLS);
    int Q = 0;
    int t = 0;
    for (int u = blockIdx.x; u < units; u += G, ++t) {
      int m0, n0, split, k0, k1;
      coords(u, m0, n0, split, k0, k1);
      uint32_t mk[4];
      const int nper = (unit_mask(p, m0, n0, k0, k1, lane, mk) + FLUSH_KB - 1) / FLUSH_KB;
      const int row = m0 + 32 * g + lane;
      const int ea = (row < p.M) ? p.ea[row] : EXP_NONE - 1;
      // exponents of this warp's EPI_COLS / 2 complex columns, lane c holding column c
      // (no barrier among the epilogue warps: each reads its own)
      const int ccol = (n0 >> 1) + h * (EPI_COLS / 2) + lane;
      const int ebr = (lane < EPI_COLS / 2 && 2 * ccol < p.N) ? p.eb[ccol] : EXP_NONE - 1;
      long long acc[EPI_COLS];
#pragma unroll
      for (int j = 0; j < EPI_COLS; ++j) acc[j] = 0;
      bool ok = !*(volatile int*)abort_flag;
      for (int q = 0; q < nper && ok; ++q) {
        if (!mbar_wait_or_abort(tfull, (uint32_t)(Q + q) & 1u, abort_flag)) {
          ok = false;
          break;
        }
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
#pragma unroll
        for (int c0 = 0; c0 < EPI_COLS; c0 += 8) {
          uint32_t v0[8], v1[8], v2[8];
          __syncwarp();
          tmem_ld8(tl + (uint32_t)c0, v0);
          tmem_ld8(tl + (uint32_t)(BN + c0), v1);
          tmem_ld8(tl + (uint32_t)(2 * BN + c0), v2);
          tmem_wait_ld();
          after_wait(v0);
          after_wait(v1);
          after_wait(v2);
          if (c0 + 8 == EPI_COLS) {
            asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
            __syncwarp();
            if (lane == 0) mbar_arrive(tempty);
          }
#pragma unroll
          for (int j = 0; j < 8; ++j) acc[c0 + j] += exact_levels(v0[j], v1[j], v2[j]);
        }
      }
      // every unit's tdone phase is consumed, so the parities stay in step
      if (ok && !mbar_wait_or_abort(tdone, (uint32_t)t & 1u, abort_flag)) ok = false;
      if (!ok) {
        if (!*(volatile int*)abort_flag) atomicExch(p.err, 3);
        break;
      }
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      const bool have = nper > 0;
      // levels 3..4 -> FP64 values (kept in acc as bit patterns), then release TMEM
#pragma unroll
      for (int c0 = 0; c0 < EPI_COLS; c0 += 16) {
        uint32_t v3[16], v4[16];
        __syncwarp();
        tmem_ld16(tl + (uint32_t)(3 * BN + c0), v3);
        tmem_ld16(tl + (uint32_t)(4 * BN + c0), v4);
        tmem_wait_ld();
        after_wait(v3);
        after_wait(v4);
#pragma unroll
        for (int j = 0; j < 16; ++j) {
          const int eb = __shfl_sync(0xffffffffu, ebr, (c0 + j) >> 1);
          double v = 0.0;
          if (have && ea > EXP_NONE && eb > EXP_NONE)
            v = finish_value(acc[c0 + j], v3[j], v4[j], ea + eb - 46);
          acc[c0 + j] = __double_as_longlong(v);
        }
      }
      asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
      __syncwarp();
      if (lane == 0) mbar_arrive(tfree);
      if (row < p.M) {
#pragma unroll
        for (int j = 0; j < EPI_COLS; j += 2) {
          const int cl = h * EPI_COLS + j;
          const int col = n0 + cl;
          if (col >= p.N) break;
          const double re = __longlong_as_double(acc[j]), im = __longlong_as_double(acc[j + 1]);
          if (p.part != nullptr) {
            double2* dst = reinterpret_cast<double2*>(p.part + ((long)split * p.M + row) * p.N + col);
            *dst = make_double2(re, im);
          } else {
            double2* o = p.out + (long)row * p.ldm + (long)(col >> 1) * p.ldn;
            double2 x = make_double2(re, im);
            if (p.accumulate) {
              const double2 y = *o;
              x.x += y.x;
              x.y += y.y;
            }
            *o = x;
          }
        }
      }
      Q += nper;
    }
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (warp == 1) {
    __syncwarp();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem),
                 "r"(TMEM_COLS)
                 : "memory");
  }
}

__global__ void splitk_sum_kernel(const double* __restrict__ part, int splits, int M, int N,
                                  double2* __restrict__ out, long ldm, long ldn, int accumulate,
                                  const int* skip) {
  if (skip != nullptr && *skip != 0) return;
  const int nc = N >> 1;
  const long total = (long)M * nc;
  for (long idx = blockIdx.x * (long)blockDim.x + threadIdx.x; idx < total;
       idx += (long)gridDim.x * blockDim.x) {
    // consecutive threads take consecutive rows: the complex outputs of the
    // transposed-output GEMMs are then written contiguously
    const int m = (int)(idx % M), c = (int)(idx / M);
    double re = 0.0, im = 0.0;
    for (int s = 0; s < splits; ++s) {
      const double2 v = *reinterpret_cast<const double2*>(part + ((long)s * M + m) * N + 2 * c);
      re += v.x;
      im += v.y;
    }
    double2* o = out + (long)m * ldm + (long)c * ldn;
    if (accumulate) {
      const double2 y = *o;
      re += y.x;
      im += y.y;
    }
    *o = make_double2(re, im);
  }
}

// ------------------------------------------------------------------ tensor maps
typedef CUresult (*EncodeTiledFn)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*,
                                  const cuuint64_t*, const cuuint64_t*, const cuuint32_t*,
                                  const cuuint32_t*, CUtensorMapInterleave, CUtensorMapSwizzle,
                                  CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

EncodeTiledFn encode_fn() {
  static EncodeTiledFn fn = nullptr;
  static std::once_flag once;
  std::call_once(once, [] {
    void* f = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &f, 12000, cudaEnableDefault,
                                         &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<EncodeTiledFn>(f);
  });
  return fn;
}

struct MapKey {
  const void* ptr;
  long rows, K, Kp, plane;
  int box_rows;
  bool operator==(const MapKey& o) const {
    return ptr == o.ptr && rows == o.rows && K == o.K && Kp == o.Kp && plane == o.plane &&
           box_rows == o.box_rows;
  }
};

struct MapCache {
  std::vector<std::pair<MapKey, CUtensorMap>> entries;
  std::mutex mu;
};

MapCache& map_cache() {
  static MapCache c;
  return c;
}

// 3-D map over the NDIGIT digit planes [5][rows][Kp] of BF16, logical extent
// (K, rows, 5), box (BK, box_rows, 5): one load brings a K block of all five planes
bool make_map(CUtensorMap* out, const void* ptr, long rows, long K, long Kp, long plane,
              int box_rows) {
  MapKey key{ptr, rows, K, Kp, plane, box_rows};
  MapCache& c = map_cache();
  {
    std::lock_guard<std::mutex> lk(c.mu);
    for (auto& e : c.entries)
      if (e.first == key) {
        *out = e.second;
        return true;
      }
  }
  EncodeTiledFn fn = encode_fn();
  if (fn == nullptr) return false;
  cuuint64_t dims[3] = {(cuuint64_t)K, (cuuint64_t)rows, (cuuint64_t)NDIGIT};
  cuuint64_t strides[2] = {(cuuint64_t)Kp * 2, (cuuint64_t)plane * 2};
  cuuint32_t box[3] = {(cuuint32_t)BK, (cuuint32_t)box_rows, (cuuint32_t)NDIGIT};
  cuuint32_t estr[3] = {1, 1, 1};
  CUtensorMap m;
  CUresult r = fn(&m, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 3, const_cast<void*>(ptr), dims, strides,
                  box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_64B,
                  CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) return false;
  std::lock_guard<std::mutex> lk(c.mu);
  if (c.entries.size() > 512) c.entries.clear();
  c.entries.push_back({key, m});
  *out = m;
  return true;
}

// sticky error code of the tensor-core kernels (bounded waits that expired)
__device__ int g_tc_err;

int* err_flag() {
  static int* flag = nullptr;
  static std::once_flag once;
  std::call_once(once, [] {
    void* a = nullptr;
    if (cudaGetSymbolAddress(&a, g_tc_err) == cudaSuccess) flag = static_cast<int*>(a);
  });
  return flag;
}

}  // namespace

// K splits: at least what the accuracy bound needs (MAX_K_SPLIT reals per split), at most enough CTAs for twice PTN_TUNE_TC_SPLIT_WAVES waves (one CTA per SM);
// in between, the split count with the fewest waves x (K blocks per CTA + a fixed
// per-CTA cost of prologue and epilogue, about KB_OVERHEAD K blocks) -- a grid that
// spills a few CTAs into another wave costs that whole wave.
static int choose_splits(int M, int N, int nkb) {
  constexpr int KB_OVERHEAD = 6;
  const long tiles = (long)((N + BN - 1) / BN) * ((M + BM - 1) / BM);
  const long sms = num_sms();
  const int kb_max = MAX_K_SPLIT / BK;
  const int s_min = std::max(1, (nkb + kb_max - 1) / kb_max);
  const int waves = tune(PTN_TUNE_TC_SPLIT_WAVES);
  if (waves == 0) return std::min(s_min, std::max(1, nkb));
  const long s_cap =
      std::max<long>(s_min, std::min<long>(nkb, (2L * waves * sms + tiles - 1) / tiles));
  int best = s_min;
  long best_cost = -1;
  for (long s = s_min; s <= s_cap; ++s) {
    const long w = (tiles * s + sms - 1) / sms;
    const long cost = w * ((nkb + s - 1) / s + KB_OVERHEAD);
    if (best_cost < 0 || cost < best_cost) {
      best_cost = cost;
      best = (int)s;
    }
  }
  return std::min(best, std::max(1, nkb));
}

size_t tc_gemm_workspace_bytes(int M, int Ncomplex, int Kcomplex) {
  const int N = 2 * Ncomplex, K = 2 * Kcomplex;
  const int nkb = (K + BK - 1) / BK;
  const int splits = choose_splits(M, N, nkb);
  return splits > 1 ? (size_t)splits * M * N * sizeof(double) : 0;
}

// C (M x Nc complex) = A (M x Kc) * B (Kc x Nc) from digit planes:
//   Aslices: [5][M][Kp] BF16 (plain) with row exponents ea[M],
//   Bslices: [5][2 Nc][Kp] BF16 (embedded) with exponents eb[Nc]; Kp >= 2 Kc, Kp % 8 == 0.
//   fa / fb (or null): a validity byte, then non-zero flags per (128-row tile of A,
//   K block of 16 complex) and (48-column tile of B, K block), fk K blocks per flag
//   row; K blocks where either tile is zero are skipped by the persistent kernel.
ptn_status tc_gemm(const void* Aslices, long aplane, const int* ea, const void* Bslices, long bplane,
                   const int* eb, int M, int Nc, int Kc, long Kp, double2* out, long ldm, long ldn,
                   bool accumulate, void* ws, size_t ws_bytes, const int* skip, cudaStream_t st,
                   const unsigned char* fa, const unsigned char* fb, int fk) {
  const int N = 2 * Nc, K = 2 * Kc;
  PTN_CHECK_ARG(M > 0 && Nc > 0 && Kc > 0 && Kp >= K && Kp % 8 == 0, "tc_gemm: bad sizes");
  PTN_CHECK_ARG(reinterpret_cast<uintptr_t>(Aslices) % 16 == 0 &&
                    reinterpret_cast<uintptr_t>(Bslices) % 16 == 0,
                "tc_gemm: digit buffers must be 16-byte aligned");
  CUtensorMap ma, mb;
  if (!make_map(&ma, Aslices, M, K, Kp, aplane, BM) || !make_map(&mb, Bslices, N, K, Kp, bplane, BN)) {
    set_error("tc_gemm: cuTensorMapEncodeTiled failed");
    return PTN_CUDA_ERROR;
  }
  static bool attr = false;
  if (!attr) {
    PTN_CUDA_TRY(cudaFuncSetAttribute(tc_gemm_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      SMEM_BYTES));
    PTN_CUDA_TRY(cudaFuncSetAttribute(tc_gemm_persistent_kernel,
                                      cudaFuncAttributeMaxDynamicSharedMemorySize, SMEM_BYTES));
    attr = true;
  }
  TcArgs a;
  a.M = M;
  a.N = N;
  a.nkb = (K + BK - 1) / BK;
  const int gx = (N + BN - 1) / BN, gy = (M + BM - 1) / BM;
  int splits = choose_splits(M, N, a.nkb);
  // a workspace sized under other knob values: fall back to fewer splits, but
  // never below what the accuracy bound needs
  const int min_splits = (a.nkb + MAX_K_SPLIT / BK - 1) / (MAX_K_SPLIT / BK);
  while (splits > min_splits && (size_t)splits * M * N * sizeof(double) > ws_bytes) --splits;
  if (splits > 1 && (size_t)splits * M * N * sizeof(double) > ws_bytes) {
    set_error("tc_gemm: workspace too small for %d K splits", splits);
    return PTN_BAD_SHAPE;
  }
  a.kb_per_split = (a.nkb + splits - 1) / splits;
  splits = (a.nkb + a.kb_per_split - 1) / a.kb_per_split;   // no empty split
  a.splits = splits;
  a.ea = ea;
  a.eb = eb;
  a.out = out;
  a.ldm = ldm;
  a.ldn = ldn;
  a.accumulate = accumulate ? 1 : 0;
  a.part = splits > 1 ? static_cast<double*>(ws) : nullptr;
  a.err = err_flag();
  a.skip = skip;
  const bool flags = fa != nullptr && fb != nullptr;
  PTN_CHECK_ARG(!flags || fk == a.nkb, "tc_gemm: flag rows of %d K blocks for %d", fk, a.nkb);
  a.fa = flags ? fa : nullptr;
  a.fb = flags ? fb : nullptr;
  a.fk = fk;
  PTN_CHECK_ARG(a.err != nullptr, "tc_gemm: error flag lookup failed");
  PTN_CHECK_ARG(gy <= 65535 && splits <= 65535, "tc_gemm: grid too large");
  const int prof = prof_begin(st, PROF_TC_GEMM, 8.0 * M * (double)Nc * Kc,
                              2.0 * NDIGIT * ((double)M * Kp + (double)N * Kp) + 16.0 * M * Nc);
  const long units = (long)gx * gy * splits;
  // the persistent form when asked for, and always for zero-tile skipping (only it
  // reads the flags); one CTA per unit otherwise (measured faster on dense data)
  if ((tune(PTN_TUNE_TC_PERSISTENT) != 0 || flags) && units <= INT_MAX) {
    const int grid = (int)std::min<long>(units, num_sms());
    tc_gemm_persistent_kernel<<<grid, THREADS, SMEM_BYTES, st>>>(ma, mb, a, gx, gy, (int)units);
  } else {
    tc_gemm_kernel<<<dim3(gx, gy, splits), THREADS, SMEM_BYTES, st>>>(ma, mb, a);
  }
  PTN_LAUNCH_CHECK();
  note_launches(1);
  if (splits > 1) {
    const long tot = (long)M * Nc;
    const int blocks = (int)std::min<long>((tot + 255) / 256, 8L * num_sms());
    splitk_sum_kernel<<<blocks, 256, 0, st>>>(a.part, splits, M, N, out, ldm, ldn, a.accumulate,
                                              skip);
    PTN_LAUNCH_CHECK();
    note_launches(1);
  }
  prof_end(st, prof);
  return PTN_OK;
}

// host read of the sticky error flag (0 = fine); resets it
int tc_gemm_error_and_reset() {
  int v = 0;
  if (cudaMemcpyFromSymbol(&v, g_tc_err, sizeof(int)) != cudaSuccess) return -1;
  if (v != 0) {
    const int zero = 0;
    cudaMemcpyToSymbol(g_tc_err, &zero, sizeof(int));
  }
  return v;
}

}  // namespace ptn

extern "C" int tc_gemm_error_and_reset_c(void) { return ptn::tc_gemm_error_and_reset(); }
