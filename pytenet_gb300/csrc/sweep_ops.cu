// Fused local steps of the sweep: one C call runs a whole Krylov exponential (or
// Ritz-vector) step of a site or bond tensor on the stream, with no host round
// trip: _local_hamiltonian_step / _local_bond_step (pytenet/tdvp.py:223-238) and
// _minimize_local_energy (pytenet/dmrg.py:181-189).
//
// The operator applies of iteration j are launched with the Krylov stop flag as
// their skip predicate, so after a Lanczos breakdown the remaining launches of
// the (possibly graph-captured) sequence retire immediately on the device.
#include "ptn_common.cuh"
#include <algorithm>

namespace ptn {

size_t krylov_state_bytes();
const int32_t* krylov_stop_flag(const void* state);
ptn_status krylov_start(void*, const double2*, double2*, long, int, cudaStream_t);
ptn_status krylov_step(void*, double2*, long, int, cudaStream_t);
ptn_status krylov_last(void*, const double2*, const double2*, long, int, bool, cudaStream_t);
ptn_status krylov_coef(void*, double, double, int, cudaStream_t);
ptn_status krylov_combine(const void*, const double2*, long, double2*, cudaStream_t);
ptn_status depth_predict(void*, const void*, int, int, double, int, cudaStream_t);
ptn_status depth_check(void*, int, double, double, double, cudaStream_t);
ptn_status depth_record(void*, const void*, double, double, cudaStream_t);

size_t heff_workspace_bytes_f64(int Dl, int d, int Dr, int chil, int chir);
size_t bond_workspace_bytes_f64(int Dl, int Dr, int chi);
ptn_status heff_apply_f64(const double2*, const double2*, const double2*, const double2*, double2*,
                          int, int, int, int, int, void*, size_t, const int*, cudaStream_t);
ptn_status bond_apply_f64(const double2*, const double2*, const double2*, double2*, int, int, int,
                          void*, size_t, const int*, cudaStream_t);

// mixed-precision operator (BF16-digit tcgen05 contractions), see mixed.cu
size_t heff_workspace_bytes_mixed(int Dl, int d, int Dr, int chil, int chir);
size_t bond_workspace_bytes_mixed(int Dl, int Dr, int chi);
ptn_status heff_prepare_mixed(const double2* w, const double2* l, const double2* r, int Dl, int d,
                              int Dr, int chil, int chir, void* ws, size_t ws_bytes,
                              cudaStream_t st);
ptn_status heff_apply_mixed(const double2* x, double2* y, const double2* w, int Dl, int d, int Dr,
                            int chil, int chir, void* ws, size_t ws_bytes, const int* skip,
                            cudaStream_t st);
ptn_status bond_prepare_mixed(const double2* l, const double2* r, int Dl, int Dr, int chi, void* ws,
                              size_t ws_bytes, cudaStream_t st);
ptn_status bond_apply_mixed(const double2* x, double2* y, int Dl, int Dr, int chi, void* ws,
                            size_t ws_bytes, const int* skip, cudaStream_t st);

namespace {

struct LocalOp {
  bool site;
  int Dl, d, Dr, chil, chir, prec;
  const double2 *w, *l, *r;
  void* ws;
  size_t ws_bytes;

  long n() const { return site ? (long)Dl * d * Dr : (long)Dl * Dr; }

  ptn_status prepare(cudaStream_t st) const {
    if (prec == PTN_PREC_FP64) return PTN_OK;
    return site ? heff_prepare_mixed(w, l, r, Dl, d, Dr, chil, chir, ws, ws_bytes, st)
                : bond_prepare_mixed(l, r, Dl, Dr, chil, ws, ws_bytes, st);
  }

  ptn_status apply(const double2* x, double2* y, const int* skip, cudaStream_t st) const {
    if (prec == PTN_PREC_FP64)
      return site ? heff_apply_f64(x, w, l, r, y, Dl, d, Dr, chil, chir, ws, ws_bytes, skip, st)
                  : bond_apply_f64(x, l, r, y, Dl, Dr, chil, ws, ws_bytes, skip, st);
    return site ? heff_apply_mixed(x, y, w, Dl, d, Dr, chil, chir, ws, ws_bytes, skip, st)
                : bond_apply_mixed(x, y, Dl, Dr, chil, ws, ws_bytes, skip, st);
  }
};

// mode 0: out = expm(dt H) x; mode 1: out = lowest Ritz vector
ptn_status krylov_run(const LocalOp& op, double2* x, double dt_re, double dt_im, int numiter,
                      int mode, double2* V, void* state, cudaStream_t st,
                      const ptn_depth_ctx* depth = nullptr) {
  PTN_CHECK_ARG(numiter >= 1 && numiter < PTN_KRYLOV_MAXITER, "numiter must be in [1, %d)",
                PTN_KRYLOV_MAXITER);
  const long n = op.n();
  const int* skip = krylov_stop_flag(state);
  PTN_TRY(op.prepare(st));
  PTN_TRY(krylov_start(state, x, V, n, numiter, st));
  const double dt_abs = sqrt(dt_re * dt_re + dt_im * dt_im);
  for (int j = 0; j + 1 < numiter; ++j) {
    PTN_TRY(op.apply(V + (long)j * n, V + (long)(j + 1) * n, skip, st));
    PTN_TRY(krylov_step(state, V, n, j, st));
    if (depth != nullptr) {
      if (j == 0)
        PTN_TRY(depth_predict(state, depth, op.Dl, op.Dr, dt_abs, numiter, st));
      if ((depth->params != nullptr || depth->check_from > 0) && j >= 1)
        PTN_TRY(depth_check(state, j, dt_re, dt_im, depth->tol, st));
    }
  }
  double2* w = V + (long)numiter * n;
  PTN_TRY(op.apply(V + (long)(numiter - 1) * n, w, skip, st));
  PTN_TRY(krylov_last(state, V, w, n, numiter - 1, true, st));
  PTN_TRY(krylov_coef(state, dt_re, dt_im, mode, st));
  if (depth != nullptr) PTN_TRY(depth_record(state, depth, dt_re, dt_im, st));
  PTN_TRY(krylov_combine(state, V, n, x, st));
  return PTN_OK;
}

}  // namespace
}  // namespace ptn

using namespace ptn;

extern "C" {

size_t ptn_site_step_workspace_bytes(int Dl, int d, int Dr, int chil, int chir, int prec) {
  return prec == PTN_PREC_FP64 ? heff_workspace_bytes_f64(Dl, d, Dr, chil, chir)
                               : heff_workspace_bytes_mixed(Dl, d, Dr, chil, chir);
}

size_t ptn_bond_step_workspace_bytes(int Dl, int Dr, int chi, int prec) {
  return prec == PTN_PREC_FP64 ? bond_workspace_bytes_f64(Dl, Dr, chi)
                               : bond_workspace_bytes_mixed(Dl, Dr, chi);
}

ptn_status ptn_expm_site(ptn_c128* a, const ptn_c128* w, const ptn_c128* l, const ptn_c128* r,
                         int Dl, int d, int Dr, int chil, int chir, double dt_re, double dt_im,
                         int numiter, int prec, ptn_c128* V, void* state, void* ws,
                         size_t ws_bytes, void* stream) {
  PTN_CHECK_ARG(Dl > 0 && d > 0 && Dr > 0 && chil > 0 && chir > 0, "expm_site: bad dims");
  LocalOp op{true, Dl, d, Dr, chil, chir, prec, reinterpret_cast<const double2*>(w),
             reinterpret_cast<const double2*>(l), reinterpret_cast<const double2*>(r), ws,
             ws_bytes};
  return krylov_run(op, reinterpret_cast<double2*>(a), dt_re, dt_im, numiter, 0,
                    reinterpret_cast<double2*>(V), state, as_stream(stream));
}

ptn_status ptn_expm_bond(ptn_c128* c, const ptn_c128* l, const ptn_c128* r, int Dl, int Dr,
                         int chi, double dt_re, double dt_im, int numiter, int prec, ptn_c128* V,
                         void* state, void* ws, size_t ws_bytes, void* stream) {
  PTN_CHECK_ARG(Dl > 0 && Dr > 0 && chi > 0, "expm_bond: bad dims");
  LocalOp op{false, Dl, 1, Dr, chi, chi, prec, nullptr, reinterpret_cast<const double2*>(l),
             reinterpret_cast<const double2*>(r), ws, ws_bytes};
  return krylov_run(op, reinterpret_cast<double2*>(c), dt_re, dt_im, numiter, 0,
                    reinterpret_cast<double2*>(V), state, as_stream(stream));
}

ptn_status ptn_expm_site_ex(ptn_c128* a, const ptn_c128* w, const ptn_c128* l, const ptn_c128* r,
                            int Dl, int d, int Dr, int chil, int chir, double dt_re, double dt_im,
                            int numiter, int prec, const ptn_depth_ctx* depth, ptn_c128* V,
                            void* state, void* ws, size_t ws_bytes, void* stream) {
  PTN_CHECK_ARG(Dl > 0 && d > 0 && Dr > 0 && chil > 0 && chir > 0, "expm_site: bad dims");
  PTN_CHECK_ARG(depth == nullptr || depth->history != nullptr, "expm_site: depth context needs a history buffer");
  LocalOp op{true, Dl, d, Dr, chil, chir, prec, reinterpret_cast<const double2*>(w),
             reinterpret_cast<const double2*>(l), reinterpret_cast<const double2*>(r), ws,
             ws_bytes};
  return krylov_run(op, reinterpret_cast<double2*>(a), dt_re, dt_im, numiter, 0,
                    reinterpret_cast<double2*>(V), state, as_stream(stream), depth);
}

ptn_status ptn_expm_bond_ex(ptn_c128* c, const ptn_c128* l, const ptn_c128* r, int Dl, int Dr,
                            int chi, double dt_re, double dt_im, int numiter, int prec,
                            const ptn_depth_ctx* depth, ptn_c128* V, void* state, void* ws,
                            size_t ws_bytes, void* stream) {
  PTN_CHECK_ARG(Dl > 0 && Dr > 0 && chi > 0, "expm_bond: bad dims");
  PTN_CHECK_ARG(depth == nullptr || depth->history != nullptr, "expm_bond: depth context needs a history buffer");
  LocalOp op{false, Dl, 1, Dr, chi, chi, prec, nullptr, reinterpret_cast<const double2*>(l),
             reinterpret_cast<const double2*>(r), ws, ws_bytes};
  return krylov_run(op, reinterpret_cast<double2*>(c), dt_re, dt_im, numiter, 0,
                    reinterpret_cast<double2*>(V), state, as_stream(stream), depth);
}

ptn_status ptn_eigh_site(ptn_c128* a, const ptn_c128* w, const ptn_c128* l, const ptn_c128* r,
                         int Dl, int d, int Dr, int chil, int chir, int numiter, int prec,
                         ptn_c128* V, void* state, void* ws, size_t ws_bytes, void* stream) {
  PTN_CHECK_ARG(Dl > 0 && d > 0 && Dr > 0 && chil > 0 && chir > 0, "eigh_site: bad dims");
  LocalOp op{true, Dl, d, Dr, chil, chir, prec, reinterpret_cast<const double2*>(w),
             reinterpret_cast<const double2*>(l), reinterpret_cast<const double2*>(r), ws,
             ws_bytes};
  return krylov_run(op, reinterpret_cast<double2*>(a), 0.0, 0.0, numiter, 1,
                    reinterpret_cast<double2*>(V), state, as_stream(stream));
}

}  // extern "C"
