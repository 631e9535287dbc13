// Krylov core of the sweep (pytenet/krylov.py:12-150), fully on the device.
//
// lanczos_iteration (krylov.py:12-57) is split into memory-bound passes over the
// n-vectors; every reduction is two-phase (per-CTA partials, then each consumer
// CTA re-reduces the partials in a fixed order), so results are deterministic and
// no pass needs a host round trip:
//   start : nrm = |v|, V[0] = v / nrm
//   step j: (w = A V[j] already in V[j+1])
//           alpha_j = Re <w, V[j]>                            dot pass
//           w -= alpha_j V[j] + beta_{j-1} V[j-1]; |w|^2        update pass
//           beta_j = |w|; breakdown if beta_j < 100 n eps, else V[j+1] = w / beta_j
//   last  : alpha_{m-1} = Re <A V[m-1], V[m-1]> and the residual norm beta_next
// A breakdown sets state->stopped: all later passes (and the operator launches,
// which test the same flag) return immediately, m_used keeps the truncated size,
// exactly the early return of krylov.py:44-50.
// The tridiagonal eigenproblem (eigh_tridiag, krylov.py:142-150) is solved by one
// warp with the implicit QL algorithm with Wilkinson shifts (Bowdler, Martin,
// Reinsch, Wilkinson 1968); lane k carries row k of the eigenvector matrix, every
// lane runs the same scalar recurrence, so no synchronisation is needed.
// expm_krylov (krylov.py:122-136) and eigh_krylov (krylov.py:110-119) then reduce
// to coefficients c_k and one combination pass out = sum_k c_k V[k].
#include "ptn_common.cuh"
#include "mlp_common.cuh"
#include <cfloat>
#include <algorithm>

namespace ptn {

void note_launches(int n);

namespace {

constexpr int RED_MAX = 1024;   // max CTAs of a vector pass (partials per reduction)
constexpr int VT = 256;         // threads per CTA of a vector pass

struct KState {
  ptn_krylov_state s;
  double part_a[RED_MAX];
  double part_b[RED_MAX];
  int nblocks;                  // CTAs used by the vector passes of this run
  int coef_ready;               // an accepted learned depth already stored coef[]
  unsigned int bar;             // grid-barrier tickets of the fused Lanczos step
};

__device__ __forceinline__ double reduce_partials(const double* part, int nb, double* sh) {
  double v = 0.0;
  for (int i = threadIdx.x; i < nb; i += blockDim.x) v += part[i];
  return block_sum(v, sh);
}

__global__ void __launch_bounds__(VT) k_norm_partial(KState* st, const double2* __restrict__ x,
                                                     long n) {
  __shared__ double sh[33];
  double acc = 0.0;
  for (long i = blockIdx.x * (long)VT + threadIdx.x; i < n; i += (long)gridDim.x * VT) {
    const double2 v = x[i];
    acc = fma(v.x, v.x, acc);
    acc = fma(v.y, v.y, acc);
  }
  acc = block_sum(acc, sh);
  if (threadIdx.x == 0) st->part_a[blockIdx.x] = acc;
}

__global__ void __launch_bounds__(VT) k_start_finish(KState* st, const double2* __restrict__ x,
                                                     double2* __restrict__ v0, long n, int maxiter) {
  __shared__ double sh[33];
  const int nb = gridDim.x;
  const double nrm = sqrt(reduce_partials(st->part_a, nb, sh));
  const bool ok = (nrm > 0.0) && isfinite(nrm);
  if (ok) {
    const double inv = 1.0 / nrm;
    for (long i = blockIdx.x * (long)VT + threadIdx.x; i < n; i += (long)gridDim.x * VT) {
      const double2 v = x[i];
      v0[i] = make_double2(v.x * inv, v.y * inv);
    }
  }
  if (blockIdx.x == 0) {
    for (int i = threadIdx.x; i < PTN_KRYLOV_MAXITER; i += blockDim.x) {
      st->s.alpha[i] = 0.0;
      st->s.beta[i] = 0.0;
      st->s.coef[i].re = 0.0;
      st->s.coef[i].im = 0.0;
    }
    if (threadIdx.x == 0) {
      st->s.nrm = nrm;
      st->s.m_used = 1;
      st->s.stopped = ok ? 0 : 1;
      st->s.maxiter = maxiter;
      st->s.status = ok ? PTN_OK : PTN_NAN;
      st->s.beta_next = 0.0;
      st->s.eval0 = 0.0;
      st->s.resid = 0.0;
      st->s.m_target = 0;
      st->coef_ready = 0;
      st->bar = 0;
      st->nblocks = nb;
    }
  }
}

// partial Re <w, v> = sum w.x v.x + w.y v.y
__global__ void __launch_bounds__(VT) k_dot_partial(KState* st, const double2* __restrict__ w,
                                                    const double2* __restrict__ v, long n) {
  if (st->s.stopped) return;
  __shared__ double sh[33];
  double acc = 0.0;
  for (long i = blockIdx.x * (long)VT + threadIdx.x; i < n; i += (long)gridDim.x * VT) {
    const double2 a = w[i], b = v[i];
    acc = fma(a.x, b.x, acc);
    acc = fma(a.y, b.y, acc);
  }
  acc = block_sum(acc, sh);
  if (threadIdx.x == 0) st->part_a[blockIdx.x] = acc;
}

// w -= alpha_j v_j + beta_{j-1} v_{j-1}; partial |w|^2. With `inplace` false the
// residual norm is accumulated without writing w (final iteration).
__global__ void __launch_bounds__(VT) k_update(KState* st, double2* __restrict__ w,
                                               const double2* __restrict__ vj,
                                               const double2* __restrict__ vjm1, long n, int j,
                                               int inplace) {
  if (st->s.stopped) return;
  __shared__ double sh[33];
  const double alpha = reduce_partials(st->part_a, gridDim.x, sh);
  const double beta = (j > 0) ? st->s.beta[j - 1] : 0.0;
  double acc = 0.0;
  for (long i = blockIdx.x * (long)VT + threadIdx.x; i < n; i += (long)gridDim.x * VT) {
    const double2 a = vj[i];
    double2 t = make_double2(alpha * a.x, alpha * a.y);
    if (j > 0) {
      const double2 b = vjm1[i];
      t.x += beta * b.x;
      t.y += beta * b.y;
    }
    double2 x = w[i];
    x.x -= t.x;
    x.y -= t.y;
    if (inplace) w[i] = x;
    acc = fma(x.x, x.x, acc);
    acc = fma(x.y, x.y, acc);
  }
  acc = block_sum(acc, sh);
  if (threadIdx.x == 0) {
    st->part_b[blockIdx.x] = acc;
    if (blockIdx.x == 0) st->s.alpha[j] = alpha;
  }
}

__global__ void __launch_bounds__(VT) k_scale(KState* st, double2* __restrict__ w, long n, int j,
                                              double thresh) {
  if (st->s.stopped) return;
  __shared__ double sh[33];
  const double beta = sqrt(reduce_partials(st->part_b, gridDim.x, sh));
  if (beta < thresh) {
    if (blockIdx.x == 0 && threadIdx.x == 0) {
      st->s.beta_next = beta;
      st->s.m_used = j + 1;
      st->s.stopped = 1;
      st->s.breakdowns += 1;
    }
    return;
  }
  const double inv = 1.0 / beta;
  for (long i = blockIdx.x * (long)VT + threadIdx.x; i < n; i += (long)gridDim.x * VT) {
    double2 x = w[i];
    w[i] = make_double2(x.x * inv, x.y * inv);
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    st->s.beta[j] = beta;
    st->s.m_used = j + 2;
  }
}

// ------------------------------------------------------------------ fused step
// One Lanczos step (krylov.py:40-51) as one cooperative launch: phase 1 reads w and
// v_j once into registers (FR entries per thread) and forms the partials of
// alpha_j = Re <w, v_j>; phase 2, after a grid barrier, forms w - alpha_j v_j -
// beta_{j-1} v_{j-1} in registers with the partials of |w|^2; phase 3, after a
// second barrier, tests beta_j against the breakdown threshold and writes
// v_{j+1} = w / beta_j. Every block reduces the same partials in the same order,
// so all blocks take identical decisions. Traffic: three vector reads and one
// write instead of the eight passes of the three-launch step.
constexpr int FT = 512;           // threads per CTA of the fused step
constexpr int FR = 4;             // vector entries per thread held in registers
constexpr long BAR_SPIN_LIMIT = 1L << 24;

// partials written by other CTAs of this grid: read past L1
__device__ __forceinline__ double reduce_partials_cg(const double* part, int nb, double* sh) {
  double v = 0.0;
  for (int i = threadIdx.x; i < nb; i += blockDim.x) v += __ldcg(part + i);
  return block_sum(v, sh);
}

// grid-wide barrier over co-resident CTAs (cooperative launch); bounded: on expiry
// it reports false (the step then stops with PTN_TIMEOUT instead of waiting on)
__device__ bool grid_barrier(KState* st) {
  __shared__ int s_ok;
  __syncthreads();
  if (threadIdx.x == 0) {
    __threadfence();
    const unsigned nb = gridDim.x;
    const unsigned t = atomicAdd(&st->bar, 1u);
    const unsigned target = (t / nb + 1u) * nb;
    int ok = 1;
    for (long it = 0;; ++it) {
      unsigned v;
      asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(&st->bar) : "memory");
      if ((int)(v - target) >= 0) break;
      if (it > BAR_SPIN_LIMIT) {
        ok = 0;
        break;
      }
      __nanosleep(20);
    }
    __threadfence();
    s_ok = ok;
  }
  __syncthreads();
  return s_ok != 0;
}

__global__ void __launch_bounds__(FT, 2) k_lanczos_fused(KState* st, double2* __restrict__ w,
                                                         const double2* __restrict__ vj,
                                                         const double2* __restrict__ vjm1,
                                                         long n, int j, double thresh) {
  if (st->s.stopped) return;   // set by earlier launches only: uniform over the grid
  __shared__ double sh[33];
  const long T = (long)gridDim.x * FT;
  const long base = blockIdx.x * (long)FT + threadIdx.x;
  double2 x[FR], a[FR];
  double acc = 0.0;
#pragma unroll
  for (int r = 0; r < FR; ++r) {
    const long i = base + r * T;
    x[r] = make_double2(0.0, 0.0);
    a[r] = make_double2(0.0, 0.0);
    if (i < n) {
      x[r] = w[i];
      a[r] = vj[i];
      acc = fma(x[r].x, a[r].x, acc);
      acc = fma(x[r].y, a[r].y, acc);
    }
  }
  acc = block_sum(acc, sh);
  if (threadIdx.x == 0) st->part_a[blockIdx.x] = acc;
  if (!grid_barrier(st)) {
    if (threadIdx.x == 0) {
      st->s.status = PTN_TIMEOUT;
      st->s.stopped = 1;
    }
    return;
  }
  const double alpha = reduce_partials_cg(st->part_a, gridDim.x, sh);
  const double beta = (j > 0) ? st->s.beta[j - 1] : 0.0;
  acc = 0.0;
#pragma unroll
  for (int r = 0; r < FR; ++r) {
    const long i = base + r * T;
    if (i < n) {
      double2 t = make_double2(alpha * a[r].x, alpha * a[r].y);
      if (j > 0) {
        const double2 b = vjm1[i];
        t.x += beta * b.x;
        t.y += beta * b.y;
      }
      x[r].x -= t.x;
      x[r].y -= t.y;
      acc = fma(x[r].x, x[r].x, acc);
      acc = fma(x[r].y, x[r].y, acc);
    }
  }
  acc = block_sum(acc, sh);
  if (threadIdx.x == 0) st->part_b[blockIdx.x] = acc;
  if (!grid_barrier(st)) {
    if (threadIdx.x == 0) {
      st->s.status = PTN_TIMEOUT;
      st->s.stopped = 1;
    }
    return;
  }
  const double bnext = sqrt(reduce_partials_cg(st->part_b, gridDim.x, sh));
  if (bnext < thresh) {
    if (blockIdx.x == 0 && threadIdx.x == 0) {
      st->s.alpha[j] = alpha;
      st->s.beta_next = bnext;
      st->s.m_used = j + 1;
      st->s.stopped = 1;
      st->s.breakdowns += 1;
    }
    return;
  }
  const double inv = 1.0 / bnext;
#pragma unroll
  for (int r = 0; r < FR; ++r) {
    const long i = base + r * T;
    if (i < n) w[i] = make_double2(x[r].x * inv, x[r].y * inv);
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    st->s.alpha[j] = alpha;
    st->s.beta[j] = bnext;
    st->s.m_used = j + 2;
  }
}

// final alpha; beta_next comes from the partials of a non-writing update pass
__global__ void k_last_alpha(KState* st, int j) {
  if (st->s.stopped) return;
  __shared__ double sh[33];
  const double alpha = reduce_partials(st->part_a, st->nblocks, sh);
  if (threadIdx.x == 0) st->s.alpha[j] = alpha;
}

__global__ void k_last_resid(KState* st) {
  if (st->s.stopped) return;
  __shared__ double sh[33];
  const double b = sqrt(reduce_partials(st->part_b, st->nblocks, sh));
  if (threadIdx.x == 0) st->s.beta_next = b;
}

// Symmetric tridiagonal eigenproblem by implicit QL with Wilkinson shifts.
// d[0..n-1] diagonal, e[0..n-2] off-diagonal (e[n-1] ignored); on return d holds
// the eigenvalues and z (this lane's row of the eigenvector matrix) the rotations.
__device__ void tridiag_ql(double* d, double* e, int n, double* z) {
  if (n > 0) e[n - 1] = 0.0;
  for (int l = 0; l < n; ++l) {
    for (int iter = 0; iter < 80; ++iter) {
      int mm = l;
      for (; mm < n - 1; ++mm) {
        const double dd = fabs(d[mm]) + fabs(d[mm + 1]);
        if (fabs(e[mm]) <= DBL_EPSILON * dd) break;
      }
      if (mm == l) break;
      double g = (d[l + 1] - d[l]) / (2.0 * e[l]);
      double r = hypot(g, 1.0);
      g = d[mm] - d[l] + e[l] / (g + copysign(r, g));
      double s = 1.0, c = 1.0, p = 0.0;
      bool deflated = false;
      for (int i = mm - 1; i >= l; --i) {
        const double f = s * e[i], b = c * e[i];
        r = hypot(f, g);
        e[i + 1] = r;
        if (r == 0.0) {
          d[i + 1] -= p;
          e[mm] = 0.0;
          deflated = true;
          break;
        }
        s = f / r;
        c = g / r;
        g = d[i + 1] - p;
        r = (d[i] - g) * s + 2.0 * c * b;
        p = s * r;
        d[i + 1] = g + p;
        g = c * r - b;
        const double zi = z[i], zi1 = z[i + 1];
        z[i + 1] = s * zi + c * zi1;
        z[i] = c * zi - s * zi1;
      }
      if (deflated) continue;
      d[l] -= p;
      e[l] = g;
      e[mm] = 0.0;
    }
  }
}

// c = nrm exp(dt T) e_1 for the m x m symmetric tridiagonal T (diagonal alpha,
// off-diagonal beta[0..m-2]), by one warp: lane l holds entries l and l + 32.
// Scaling and Taylor on the vector: with h = dt / 2^s and |h| |T|_1 <= 1/2, each of
// the 2^s factors exp(h T) is summed to degree 16 (remainder below 2e-20 of the
// vector). exp(dt T) e_1 is the same vector U exp(dt Lambda) U^T e_1 that
// expm_krylov forms from eigh (pytenet/krylov.py:133-136); here it costs a chain of
// tridiagonal products instead of the serial FP64 sqrt / division chain of a QL
// eigensolver. Writes out[0..m-1] when out != null; returns c_{m-1} to all lanes.
// Beyond |dt| |T|_1 > 2^(EXPM_MAX_SCALE - 1) it does nothing and returns ok = false
// (the caller then takes the eigen-decomposition route or the full depth).
constexpr int EXPM_MAX_SCALE = 12;
__device__ double2 expm_e1_warp(const double* alpha, const double* beta, int m, double nrm,
                                double dt_re, double dt_im, ptn_c128* out, bool& ok) {
  const int lane = threadIdx.x & 31;
  double a[2], bl[2], br[2];   // diagonal, left and right off-diagonal of my rows
  double tn = 0.0;
#pragma unroll
  for (int q = 0; q < 2; ++q) {
    const int k = lane + 32 * q;
    a[q] = (k < m) ? alpha[k] : 0.0;
    bl[q] = (k < m && k > 0) ? beta[k - 1] : 0.0;
    br[q] = (k < m - 1) ? beta[k] : 0.0;
    tn = fmax(tn, fabs(a[q]) + fabs(bl[q]) + fabs(br[q]));
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) tn = fmax(tn, __shfl_xor_sync(0xffffffffu, tn, o));
  const double dta = sqrt(dt_re * dt_re + dt_im * dt_im);
  int sc = 0;
  double nt = dta * tn;
  while (nt > 0.5 && sc <= EXPM_MAX_SCALE) {
    nt *= 0.5;
    ++sc;
  }
  ok = (sc <= EXPM_MAX_SCALE) && (nt == nt);
  if (!ok) return make_double2(0.0, 0.0);
  const double hs = ldexp(1.0, -sc);
  const double hr = dt_re * hs, hi = dt_im * hs;
  // v = e_1
  double vr[2] = {lane == 0 ? 1.0 : 0.0, 0.0}, vi[2] = {0.0, 0.0};
  const long reps = 1L << sc;
  for (long rep = 0; rep < reps; ++rep) {
    double yr[2] = {vr[0], vr[1]}, yi[2] = {vi[0], vi[1]};
    double tr[2] = {vr[0], vr[1]}, ti[2] = {vi[0], vi[1]};
    for (int k = 1; k <= 16; ++k) {
      // neighbours: entry k-1 and k+1 of both halves
      double pr[2], pi[2], nr[2], ni[2];
      const double up_r0 = __shfl_up_sync(0xffffffffu, tr[0], 1), up_i0 = __shfl_up_sync(0xffffffffu, ti[0], 1);
      const double up_r1 = __shfl_up_sync(0xffffffffu, tr[1], 1), up_i1 = __shfl_up_sync(0xffffffffu, ti[1], 1);
      const double dn_r0 = __shfl_down_sync(0xffffffffu, tr[0], 1), dn_i0 = __shfl_down_sync(0xffffffffu, ti[0], 1);
      const double dn_r1 = __shfl_down_sync(0xffffffffu, tr[1], 1), dn_i1 = __shfl_down_sync(0xffffffffu, ti[1], 1);
      const double w31_r0 = __shfl_sync(0xffffffffu, tr[0], 31), w31_i0 = __shfl_sync(0xffffffffu, ti[0], 31);
      const double w0_r1 = __shfl_sync(0xffffffffu, tr[1], 0), w0_i1 = __shfl_sync(0xffffffffu, ti[1], 0);
      pr[0] = lane > 0 ? up_r0 : 0.0;
      pi[0] = lane > 0 ? up_i0 : 0.0;
      pr[1] = lane > 0 ? up_r1 : w31_r0;
      pi[1] = lane > 0 ? up_i1 : w31_i0;
      nr[0] = lane < 31 ? dn_r0 : w0_r1;
      ni[0] = lane < 31 ? dn_i0 : w0_i1;
      nr[1] = lane < 31 ? dn_r1 : 0.0;
      ni[1] = lane < 31 ? dn_i1 : 0.0;
      const double inv = 1.0 / (double)k;
#pragma unroll
      for (int q = 0; q < 2; ++q) {
        // u = T t (real T), then t <- (h / k) u
        const double ur = fma(bl[q], pr[q], fma(a[q], tr[q], br[q] * nr[q]));
        const double ui = fma(bl[q], pi[q], fma(a[q], ti[q], br[q] * ni[q]));
        const double cr = hr * inv, ci = hi * inv;
        tr[q] = fma(cr, ur, -ci * ui);
        ti[q] = fma(cr, ui, ci * ur);
        yr[q] += tr[q];
        yi[q] += ti[q];
      }
    }
#pragma unroll
    for (int q = 0; q < 2; ++q) {
      const int kk = lane + 32 * q;
      vr[q] = (kk < m) ? yr[q] : 0.0;
      vi[q] = (kk < m) ? yi[q] : 0.0;
    }
  }
#pragma unroll
  for (int q = 0; q < 2; ++q) {
    const int k = lane + 32 * q;
    if (out != nullptr && k < m) {
      out[k].re = nrm * vr[q];
      out[k].im = nrm * vi[q];
    }
  }
  const int ql = (m - 1) >> 5, ll = (m - 1) & 31;
  const double lr = __shfl_sync(0xffffffffu, ql ? vr[1] : vr[0], ll);
  const double li = __shfl_sync(0xffffffffu, ql ? vi[1] : vi[0], ll);
  return make_double2(nrm * lr, nrm * li);
}

// mode 0: expm coefficients c = nrm U exp(dt Lambda) U^T e_1;
// mode 1: lowest Ritz vector coefficients c = U[:, argmin], eval0 = min eigenvalue.
__global__ void k_tridiag(KState* st, double dt_re, double dt_im, int mode) {
  const int lane = threadIdx.x;  // one warp
  if (st->s.status != PTN_OK) return;
  const int m = st->s.m_used;
  bool ok = true;
  if (mode == 0 && !st->coef_ready)
    expm_e1_warp(st->s.alpha, st->s.beta, m, st->s.nrm, dt_re, dt_im, st->s.coef, ok);
  if (mode == 0 && ok) {
    __syncwarp();
    if (lane == 0) {
      const ptn_c128 cl = st->s.coef[m - 1];
      // relative estimate beta_m |c_m| / |v| (the coefficients carry the factor |v|);
      // an accepted learned depth already stored its own
      if (!st->coef_ready)
        st->s.resid = st->s.beta_next * sqrt(cl.re * cl.re + cl.im * cl.im) / st->s.nrm;
      st->s.iters_total += m;
    }
    return;
  }
  double d[PTN_KRYLOV_MAXITER], e[PTN_KRYLOV_MAXITER], z[PTN_KRYLOV_MAXITER];
  for (int i = 0; i < m; ++i) {
    d[i] = st->s.alpha[i];
    e[i] = (i < m - 1) ? st->s.beta[i] : 0.0;
  }
  // lanes >= 32 never exist; rows k >= 32 are handled by a second pass below
  for (int pass = 0; pass * 32 < m; ++pass) {
    const int k = pass * 32 + lane;
    double dd[PTN_KRYLOV_MAXITER], ee[PTN_KRYLOV_MAXITER];
    for (int i = 0; i < m; ++i) { dd[i] = d[i]; ee[i] = e[i]; z[i] = (i == k) ? 1.0 : 0.0; }
    tridiag_ql(dd, ee, m, z);
    // row 0 of U (lane 0 of pass 0 owns it): broadcast through shared memory
    __shared__ double u0[PTN_KRYLOV_MAXITER];
    __shared__ double lam[PTN_KRYLOV_MAXITER];
    if (pass == 0 && lane == 0)
      for (int i = 0; i < m; ++i) { u0[i] = z[i]; lam[i] = dd[i]; }
    __syncwarp();
    if (k < m) {
      if (mode == 0) {
        double cr = 0.0, ci = 0.0;
        for (int jj = 0; jj < m; ++jj) {
          const double a = exp(dt_re * lam[jj]);
          double sn, cs;
          sincos(dt_im * lam[jj], &sn, &cs);
          const double f = st->s.nrm * u0[jj] * z[jj];
          cr = fma(f * a, cs, cr);
          ci = fma(f * a, sn, ci);
        }
        st->s.coef[k].re = cr;
        st->s.coef[k].im = ci;
      } else {
        int jmin = 0;
        for (int jj = 1; jj < m; ++jj)
          if (lam[jj] < lam[jmin]) jmin = jj;
        st->s.coef[k].re = z[jmin];
        st->s.coef[k].im = 0.0;
        if (k == 0) st->s.eval0 = lam[jmin];
      }
    }
    __syncwarp();
  }
  __syncwarp();
  if (lane == 0) {
    const ptn_c128 cl = st->s.coef[m - 1];
    // relative estimate beta_m |c_m| / |v| (the coefficients carry the factor |v|);
    // an accepted learned depth already stored its own
    if (st->s.m_target == 0 || st->s.m_used != st->s.m_target)
      st->s.resid = st->s.beta_next * sqrt(cl.re * cl.re + cl.im * cl.im) / st->s.nrm;
    st->s.iters_total += m;
  }
}

// ------------------------------------------------------------------ learned depth
typedef ptn_depth_ctx DepthArgs;

// c_{m-1} of nrm exp(dt T_m) e_1 for the leading m x m block (all lanes get it)
__device__ double2 last_coef(const double* alpha, const double* beta, int m, double nrm,
                             double dt_re, double dt_im) {
  bool ok;
  const double2 c = expm_e1_warp(alpha, beta, m, nrm, dt_re, dt_im, nullptr, ok);
  return ok ? c : make_double2(HUGE_VAL, 0.0);   // no estimate: never accepted
}

// after iteration 0: features of this local step, and the predicted depth
__global__ void k_predict(KState* st, DepthArgs a, int Dl, int Dr, double dt_abs, int numiter) {
  __shared__ float x[12];
  const int lane = threadIdx.x;
  if (st->s.status != PTN_OK) return;
  if (lane == 0) {
    const double a0 = st->s.alpha[0];
    const double b0 = (st->s.m_used >= 2) ? st->s.beta[0] : st->s.beta_next;
    const double hv = sqrt(a0 * a0 + b0 * b0);
    x[0] = (float)a.site / (float)max(1, a.nsites - 1);
    x[1] = log2f((float)Dl) * 0.1f;
    x[2] = log2f((float)Dr) * 0.1f;
    x[3] = (float)a.kind;
    x[4] = (float)(log10(dt_abs * hv + 1e-300) * 0.25);
    const float* h = a.history + (long)a.slot * 8;
    const bool valid = h[7] != 0.f;
    for (int i = 0; i < 4; ++i) x[5 + i] = valid ? h[i] : (float)(dt_abs * a0);
    for (int i = 0; i < 3; ++i) x[9 + i] = valid ? h[4 + i] : (float)(dt_abs * b0);
    for (int i = 0; i < 12; ++i) st->s.feat[i] = x[i];
  }
  __syncwarp();
  if (st->s.stopped) return;
  if (a.params == nullptr) {
    // residual-only criterion: the estimate is tested from depth check_from on
    if (lane == 0 && a.check_from > 0) {
      const int m = max(a.check_from, 2);
      st->s.m_target = (m >= numiter) ? 0 : m;
    }
    return;
  }
  const float y = mlpdef::forward_warp(a.params, x);
  if (lane == 0) {
    // targets are depth / 20; rounded to nearest: a depth one short costs a
    // residual check, not more iterations
    int m = (int)rintf(y * 20.0f);
    m = max(m, 2);
    st->s.m_target = (m >= numiter) ? 0 : m;
  }
}

// after step j: from the learned depth on, accept the first depth whose residual
// estimate is small (a prediction one short costs one more check, not the full depth)
__global__ void k_depth_check(KState* st, int j, double dt_re, double dt_im, double tol) {
  if (st->s.stopped || st->s.m_target != j + 1) return;
  const int m = j + 1;
  const double nrm = st->s.nrm;
  // coefficients of the truncated run straight into coef[]: used as they are if
  // the depth is accepted, overwritten by the full-depth run otherwise
  bool ok;
  const double2 c = expm_e1_warp(st->s.alpha, st->s.beta, m, nrm, dt_re, dt_im, st->s.coef, ok);
  const double est = ok ? st->s.beta[j] * sqrt(c.x * c.x + c.y * c.y) / nrm : HUGE_VAL;
  __syncwarp();
  if (threadIdx.x == 0) {
    if (est <= tol) {
      st->s.m_used = m;
      st->s.stopped = 1;
      st->s.early_exits += 1;
      st->s.resid = est;
      st->coef_ready = 1;
    } else {
      st->s.m_target = j + 2;   // check again after the next iteration (up to the full depth)
    }
  }
}

// after the coefficients: history of this slot and, optionally, a training record
__global__ void k_record(KState* st, DepthArgs a, double dt_re, double dt_im) {
  if (threadIdx.x != 0 || st->s.status != PTN_OK) return;
  const int m = st->s.m_used;
  const double dta = sqrt(dt_re * dt_re + dt_im * dt_im);
  float* h = a.history + (long)a.slot * 8;
  for (int i = 0; i < 4; ++i) h[i] = (i < m) ? (float)(dta * st->s.alpha[i]) : 0.f;
  for (int i = 0; i < 3; ++i) h[4 + i] = (i < m - 1) ? (float)(dta * st->s.beta[i]) : 0.f;
  h[7] = 1.f;
  if (a.log == nullptr) return;
  const int idx = atomicAdd(a.log_count, 1);
  if (idx >= a.log_capacity) return;
  double* r = a.log + (long)idx * PTN_DEPTH_RECORD;
  for (int i = 0; i < 12; ++i) r[i] = st->s.feat[i];
  for (int i = 0; i < 24; ++i) {
    r[12 + i] = (i < m) ? st->s.alpha[i] : 0.0;
    r[36 + i] = (i < m - 1) ? st->s.beta[i] : ((i == m - 1) ? st->s.beta_next : 0.0);
  }
  r[60] = st->s.nrm;
  r[61] = dt_re;
  r[62] = dt_im;
  r[63] = m;
}

// labels: smallest depth whose residual estimate meets tol (one warp per record)
__global__ void k_labels(const double* log, int count, int m_max, double tol, int* labels) {
  const int rec = blockIdx.x;
  if (rec >= count) return;
  const double* r = log + (long)rec * PTN_DEPTH_RECORD;
  const int mu = min((int)r[63], min(m_max, 24));
  const double nrm = r[60];
  int label = m_max;
  for (int m = 1; m <= mu; ++m) {
    const double2 c = last_coef(r + 12, r + 36, m, nrm, r[61], r[62]);
    const double est = r[36 + m - 1] * sqrt(c.x * c.x + c.y * c.y) / nrm;
    if (est <= tol) { label = m; break; }
  }
  if (threadIdx.x == 0) labels[rec] = label;
}

// Full eigen-decomposition of the tridiagonal matrix, eigenvalues ascending as
// numpy.linalg.eigh returns them: evals[j], evecs[k * m + j] = U[k][j].
__global__ void k_tridiag_eig(const KState* st, double* evals, double* evecs) {
  const int lane = threadIdx.x;
  if (st->s.status != PTN_OK) return;
  const int m = st->s.m_used;
  __shared__ int perm[PTN_KRYLOV_MAXITER];
  double d[PTN_KRYLOV_MAXITER], e[PTN_KRYLOV_MAXITER], z[PTN_KRYLOV_MAXITER];
  for (int pass = 0; pass * 32 < m; ++pass) {
    const int k = pass * 32 + lane;
    for (int i = 0; i < m; ++i) {
      d[i] = st->s.alpha[i];
      e[i] = (i < m - 1) ? st->s.beta[i] : 0.0;
      z[i] = (i == k) ? 1.0 : 0.0;
    }
    tridiag_ql(d, e, m, z);
    if (pass == 0 && lane == 0) {
      for (int i = 0; i < m; ++i) perm[i] = i;
      for (int i = 1; i < m; ++i) {           // insertion sort, stable
        const int p = perm[i];
        int j = i - 1;
        while (j >= 0 && d[perm[j]] > d[p]) { perm[j + 1] = perm[j]; --j; }
        perm[j + 1] = p;
      }
      for (int i = 0; i < m; ++i) evals[i] = d[perm[i]];
    }
    __syncwarp();
    if (k < m)
      for (int j = 0; j < m; ++j) evecs[(long)k * m + j] = z[perm[j]];
    __syncwarp();
  }
}

__global__ void __launch_bounds__(VT) k_combine(const KState* st, const double2* __restrict__ V,
                                                long n, double2* __restrict__ out) {
  if (st->s.status != PTN_OK) return;
  const int m = st->s.m_used;
  for (long i = blockIdx.x * (long)VT + threadIdx.x; i < n; i += (long)gridDim.x * VT) {
    double2 acc = make_double2(0.0, 0.0);
    for (int k = 0; k < m; ++k) {
      const ptn_c128 c = st->s.coef[k];
      acc = cfma(make_double2(c.re, c.im), V[(long)k * n + i], acc);
    }
    out[i] = acc;
  }
}

int vec_blocks(long n) {
  long b = (n + 4L * VT - 1) / (4L * VT);
  b = std::max(1L, std::min(b, (long)std::min(RED_MAX, 8 * num_sms())));
  return (int)b;
}

}  // namespace

ptn_status depth_predict(void* state, const void* args, int Dl, int Dr, double dt_abs, int numiter,
                         cudaStream_t st) {
  k_predict<<<1, 32, 0, st>>>(static_cast<KState*>(state), *static_cast<const DepthArgs*>(args), Dl,
                              Dr, dt_abs, numiter);
  PTN_LAUNCH_CHECK();
  note_launches(1);
  return PTN_OK;
}

ptn_status depth_check(void* state, int j, double dt_re, double dt_im, double tol, cudaStream_t st) {
  k_depth_check<<<1, 32, 0, st>>>(static_cast<KState*>(state), j, dt_re, dt_im, tol);
  PTN_LAUNCH_CHECK();
  note_launches(1);
  return PTN_OK;
}

ptn_status depth_record(void* state, const void* args, double dt_re, double dt_im, cudaStream_t st) {
  k_record<<<1, 32, 0, st>>>(static_cast<KState*>(state), *static_cast<const DepthArgs*>(args), dt_re,
                             dt_im);
  PTN_LAUNCH_CHECK();
  note_launches(1);
  return PTN_OK;
}

size_t krylov_state_bytes() { return (sizeof(KState) + 255) & ~size_t(255); }
const int32_t* krylov_stop_flag(const void* state) {
  return &static_cast<const KState*>(state)->s.stopped;
}

ptn_status krylov_start(void* state, const double2* vstart, double2* V, long n, int maxiter,
                        cudaStream_t st) {
  PTN_CHECK_ARG(n > 0, "krylov: empty vector");
  PTN_CHECK_ARG(maxiter >= 1 && maxiter <= PTN_KRYLOV_MAXITER,
                "krylov: numiter must be in [1, %d]", PTN_KRYLOV_MAXITER);
  KState* s = static_cast<KState*>(state);
  const int nb = vec_blocks(n);
  k_norm_partial<<<nb, VT, 0, st>>>(s, vstart, n);
  k_start_finish<<<nb, VT, 0, st>>>(s, vstart, V, n, maxiter);
  PTN_LAUNCH_CHECK();
  note_launches(2);
  return PTN_OK;
}

// CTAs of the fused Lanczos step for vectors of n entries: all co-resident
// (cooperative launch), FR entries per thread; 0 when the knob is off or n needs
// more CTAs than can be resident (the three-launch step is used then)
int fused_blocks(long n) {
  // below ~2^18 entries the two grid barriers cost more than the two launches they
  // replace (measured on GB300 under graph replay: n = 4096: 16.5 us fused, 13.5 us
  // in three launches; n = 524288: 31.8 us fused, 33.8 us in three launches)
  constexpr long FUSED_MIN_N = 1L << 18;
  if (tune(PTN_TUNE_KRYLOV_FUSED) == 0 || n < FUSED_MIN_N) return 0;
  static int per_sm = -1;
  if (per_sm < 0) {
    int v = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&v, k_lanczos_fused, FT, 0) != cudaSuccess) {
      cudaGetLastError();
      v = 0;
    }
    per_sm = v;
  }
  const long resident = (long)per_sm * num_sms();
  const long need = (n + (long)FT * FR - 1) / ((long)FT * FR);
  if (per_sm <= 0 || need > resident || need > RED_MAX) return 0;
  // about two entries per thread (up to one CTA per SM, for bandwidth), never fewer
  // CTAs than the registers need, never more than can be resident: small vectors
  // synchronise few CTAs
  const long want = std::min<long>((n + 2L * FT - 1) / (2L * FT), std::min<long>(num_sms(), RED_MAX));
  return (int)std::max<long>(need, want);
}

ptn_status krylov_step(void* state, double2* V, long n, int j, cudaStream_t st) {
  KState* s = static_cast<KState*>(state);
  const int nb = vec_blocks(n);
  const double thresh = 100.0 * (double)n * DBL_EPSILON;
  double2* w = V + (long)(j + 1) * n;
  const double2* vj = V + (long)j * n;
  const double2* vjm1 = j > 0 ? V + (long)(j - 1) * n : vj;
  const int fb = fused_blocks(n);
  if (fb > 0) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(fb);
    cfg.blockDim = dim3(FT);
    cfg.dynamicSmemBytes = 0;
    cfg.stream = st;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeCooperative;
    attr[0].val.cooperative = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    const int prof = prof_begin(st, PROF_KRYLOV, 0.0, 64.0 * (double)n);
    PTN_CUDA_TRY(cudaLaunchKernelEx(&cfg, k_lanczos_fused, s, w, vj, vjm1, n, j, thresh));
    prof_end(st, prof);
    note_launches(1);
    return PTN_OK;
  }
  k_dot_partial<<<nb, VT, 0, st>>>(s, w, vj, n);
  k_update<<<nb, VT, 0, st>>>(s, w, vj, vjm1, n, j, 1);
  k_scale<<<nb, VT, 0, st>>>(s, w, n, j, thresh);
  PTN_LAUNCH_CHECK();
  note_launches(3);
  return PTN_OK;
}

ptn_status krylov_last(void* state, const double2* V, const double2* w, long n, int j, bool resid,
                       cudaStream_t st) {
  KState* s = static_cast<KState*>(state);
  const int nb = vec_blocks(n);
  const double2* vj = V + (long)j * n;
  const double2* vjm1 = j > 0 ? V + (long)(j - 1) * n : vj;
  k_dot_partial<<<nb, VT, 0, st>>>(s, w, vj, n);
  int launches = 1;
  if (resid) {
    k_update<<<nb, VT, 0, st>>>(s, const_cast<double2*>(w), vj, vjm1, n, j, 0);
    k_last_resid<<<1, 256, 0, st>>>(s);
    launches += 2;
  } else {
    k_last_alpha<<<1, 256, 0, st>>>(s, j);
    launches += 1;
  }
  PTN_LAUNCH_CHECK();
  note_launches(launches);
  return PTN_OK;
}

ptn_status krylov_coef(void* state, double dt_re, double dt_im, int mode, cudaStream_t st) {
  k_tridiag<<<1, 32, 0, st>>>(static_cast<KState*>(state), dt_re, dt_im, mode);
  PTN_LAUNCH_CHECK();
  note_launches(1);
  return PTN_OK;
}

ptn_status krylov_tridiag_eig(const void* state, double* evals, double* evecs, cudaStream_t st) {
  k_tridiag_eig<<<1, 32, 0, st>>>(static_cast<const KState*>(state), evals, evecs);
  PTN_LAUNCH_CHECK();
  note_launches(1);
  return PTN_OK;
}

ptn_status krylov_combine(const void* state, const double2* V, long n, double2* out,
                          cudaStream_t st) {
  k_combine<<<vec_blocks(n), VT, 0, st>>>(static_cast<const KState*>(state), V, n, out);
  PTN_LAUNCH_CHECK();
  note_launches(1);
  return PTN_OK;
}

}  // namespace ptn

using namespace ptn;

extern "C" {

size_t ptn_krylov_state_bytes(void) { return krylov_state_bytes(); }
const int32_t* ptn_krylov_stop_flag(const void* state) { return krylov_stop_flag(state); }

ptn_status ptn_krylov_start(void* state, const ptn_c128* vstart, ptn_c128* V, long n, int maxiter,
                            void* stream) {
  return krylov_start(state, reinterpret_cast<const double2*>(vstart),
                      reinterpret_cast<double2*>(V), n, maxiter, as_stream(stream));
}

ptn_status ptn_krylov_step(void* state, ptn_c128* V, long n, int j, void* stream) {
  return krylov_step(state, reinterpret_cast<double2*>(V), n, j, as_stream(stream));
}

ptn_status ptn_krylov_last(void* state, const ptn_c128* V, const ptn_c128* w, long n, int j,
                           void* stream) {
  // the generic path always reports the residual norm (one extra vector pass)
  return krylov_last(state, reinterpret_cast<const double2*>(V),
                     reinterpret_cast<const double2*>(w), n, j, true, as_stream(stream));
}

ptn_status ptn_krylov_expm_coef(void* state, double dt_re, double dt_im, void* stream) {
  return krylov_coef(state, dt_re, dt_im, 0, as_stream(stream));
}

ptn_status ptn_krylov_eigh_coef(void* state, void* stream) {
  return krylov_coef(state, 0.0, 0.0, 1, as_stream(stream));
}

ptn_status ptn_depth_labels(const double* log, int count, int m_max, double tol, int* labels,
                            void* stream) {
  PTN_CHECK_ARG(m_max >= 1 && m_max <= 24, "depth labels: m_max must be in [1, 24]");
  if (count <= 0) return PTN_OK;
  k_labels<<<count, 32, 0, as_stream(stream)>>>(log, count, m_max, tol, labels);
  PTN_LAUNCH_CHECK();
  note_launches(1);
  return PTN_OK;
}

ptn_status ptn_krylov_tridiag_eig(const void* state, double* evals, double* evecs, void* stream) {
  return krylov_tridiag_eig(state, evals, evecs, as_stream(stream));
}

ptn_status ptn_krylov_combine(const void* state, const ptn_c128* V, long n, ptn_c128* out,
                              void* stream) {
  return krylov_combine(state, reinterpret_cast<const double2*>(V), n,
                        reinterpret_cast<double2*>(out), as_stream(stream));
}

}  // extern "C"
