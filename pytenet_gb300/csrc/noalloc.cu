// H_eff . A without caller-provided scratch memory.
//
// Some callers cannot allocate device memory: a host that binds this library
// through a foreign-function interface and has no CUDA allocator of its own, a
// process whose device memory is owned by another framework's pool, or code that
// runs while another component forbids allocation. For them this file offers
// ptn_heff_apply_noalloc, the plain FP64 H_eff . A of ptn_heff_apply, whose two
// intermediate tensors (and split-K partial sums) live in one file-scope device
// array instead of a workspace argument. The caller still passes inputs and
// output.
//
// Cost of the convenience: every GPU that loads this library keeps the array
// (PTN_HEFF_NOALLOC_BYTES) resident until the process exits, and all calls share
// it, so calls that overlap on the GPU (different streams, or different host
// threads without ordering) race on it. The first call on a device looks the
// array's device address up (cudaGetSymbolAddress, with that device current) and
// caches it together with the device's current context; make that first call
// before any stream capture. A call that finds another context current (after a
// cudaDeviceReset, say, which reloads the module) looks the address up again.
#include "ptn_common.cuh"
#include <algorithm>
#include <mutex>

namespace ptn {
ptn_status heff_apply_f64(const double2*, const double2*, const double2*, const double2*, double2*,
                          int, int, int, int, int, void*, size_t, const int*, cudaStream_t);
}

namespace {

constexpr size_t kScratchBytes = (size_t)PTN_HEFF_NOALLOC_BYTES;
constexpr int kMaxDevices = 64;

__device__ __align__(256) unsigned char g_heff_scratch[kScratchBytes];

void* g_scratch_addr[kMaxDevices] = {};
void* g_scratch_ctx[kMaxDevices] = {};   // context the cached address belongs to
std::mutex g_scratch_mu;

typedef int (*CtxGetCurrentFn)(void**);

// the driver's current context (CUcontext) of the calling thread, or null
void* current_context() {
  static CtxGetCurrentFn fn = nullptr;
  static std::once_flag once;
  std::call_once(once, [] {
    void* f = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f, 12000, cudaEnableDefault, &q) ==
            cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<CtxGetCurrentFn>(f);
  });
  void* ctx = nullptr;
  if (fn == nullptr || fn(&ctx) != 0) return nullptr;
  return ctx;
}

size_t align256(size_t b) { return (b + 255) & ~size_t(255); }

// device address of the scratch array on the current device: looked up once per
// device and context (a re-created context reloads the module at a new address)
ptn_status scratch_address(void** out) {
  int dev = -1;
  PTN_CUDA_TRY(cudaGetDevice(&dev));
  if (dev < 0 || dev >= kMaxDevices) {
    ptn::set_error("heff_apply_noalloc: device ordinal %d out of range", dev);
    return PTN_UNSUPPORTED;
  }
  std::lock_guard<std::mutex> lk(g_scratch_mu);
  void* ctx = current_context();
  if (g_scratch_addr[dev] == nullptr || ctx == nullptr || ctx != g_scratch_ctx[dev]) {
    void* p = nullptr;
    PTN_CUDA_TRY(cudaGetSymbolAddress(&p, g_heff_scratch));
    g_scratch_addr[dev] = p;
    // the lookup made the device's context current if none was
    g_scratch_ctx[dev] = current_context();
  }
  *out = g_scratch_addr[dev];
  return PTN_OK;
}

}  // namespace

extern "C" {

size_t ptn_heff_noalloc_capacity_bytes(void) { return kScratchBytes; }

ptn_status ptn_heff_apply_noalloc(const ptn_c128* a, const ptn_c128* w, const ptn_c128* l,
                                  const ptn_c128* r, ptn_c128* out, int Dl, int d, int Dr,
                                  int chil, int chir, void* stream) {
  PTN_CHECK_ARG(Dl > 0 && d > 0 && Dr > 0 && chil > 0 && chir > 0, "heff_apply_noalloc: bad dims");
  // the two intermediates T1 (Dl, d*chir, Dr) and T2 (Dl, chil*d, Dr)
  const size_t inter = (size_t)Dl * std::max(d * chir, chil * d) * Dr * sizeof(double2);
  const size_t need = 2 * align256(inter);
  PTN_CHECK_ARG(need <= kScratchBytes,
                "heff_apply_noalloc: needs %zu bytes of scratch, the built-in array holds %zu "
                "(2 * Dl * max(d*chir, chil*d) * Dr * 16 bytes must fit); use ptn_heff_apply "
                "with a workspace for this size",
                need, kScratchBytes);
  void* scratch = nullptr;
  PTN_TRY(scratch_address(&scratch));
  // every scratch byte that is read is written first in the same call (the GEMMs
  // run with beta = 0 and the MPO stage writes all of T2): nothing needs clearing
  return ptn::heff_apply_f64(reinterpret_cast<const double2*>(a), reinterpret_cast<const double2*>(w),
                             reinterpret_cast<const double2*>(l), reinterpret_cast<const double2*>(r),
                             reinterpret_cast<double2*>(out), Dl, d, Dr, chil, chir, scratch,
                             kScratchBytes, nullptr, ptn::as_stream(stream));
}

}  // extern "C"
