// Library plumbing (errors, version, launch counter) and the data-movement
// kernels of the sweep: gather / scatter of quantum-number blocks for the block
// QR (pytenet/block_sparse_util.py:67-103 sort + slice, done as index maps),
// the (2,1,0) transpose of the right-to-left sweep (pytenet/tdvp.py:95,104) and
// scaling.
#include "ptn_common.cuh"
#include <atomic>
#include <cstdarg>
#include <cstdio>
#include <algorithm>

namespace ptn {

static thread_local char g_err[512] = "";
static std::atomic<uint64_t> g_launches{0};

void set_error(const char* fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(g_err, sizeof(g_err), fmt, ap);
  va_end(ap);
}

void note_launches(int n) { g_launches.fetch_add((uint64_t)n, std::memory_order_relaxed); }

namespace {
std::atomic<int> g_tune[PTN_TUNE_COUNT] = {{1}, {2}, {0}, {0}, {1}, {0}, {0}, {0}};
constexpr int kTuneMax[PTN_TUNE_COUNT] = {16, 16, 5, 16, 1, 3, 1, 1};
}  // namespace

int tune(int key) { return (key >= 0 && key < PTN_TUNE_COUNT) ? g_tune[key].load() : 0; }

int num_sms() {
  static int cached = 0;
  if (cached == 0) {
    int dev = 0, v = 0;
    if (cudaGetDevice(&dev) == cudaSuccess &&
        cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev) == cudaSuccess && v > 0)
      cached = v;
    else
      return 132;
  }
  return cached;
}

// ------------------------------------------------------------------ live timing
namespace {
constexpr int PROF_SLOTS = 1 << 15;
struct ProfSlot {
  cudaEvent_t a = nullptr, b = nullptr;
  int kind = 0;
  double flops = 0, bytes = 0;
};
ProfSlot g_prof[PROF_SLOTS];
int g_prof_used = 0;
unsigned g_prof_mask = 0;
}  // namespace

int prof_begin(cudaStream_t st, int kind, double flops, double bytes) {
  if (!(g_prof_mask & (1u << kind)) || g_prof_used >= PROF_SLOTS) return -1;
  cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
  if (cudaStreamIsCapturing(st, &cs) != cudaSuccess || cs != cudaStreamCaptureStatusNone) return -1;
  ProfSlot& p = g_prof[g_prof_used];
  if (p.a == nullptr) {
    if (cudaEventCreate(&p.a) != cudaSuccess || cudaEventCreate(&p.b) != cudaSuccess) return -1;
  }
  p.kind = kind;
  p.flops = flops;
  p.bytes = bytes;
  if (cudaEventRecord(p.a, st) != cudaSuccess) return -1;
  return g_prof_used++;
}

void prof_end(cudaStream_t st, int slot) {
  if (slot >= 0) cudaEventRecord(g_prof[slot].b, st);
}

namespace {

int grid_for(long n, int threads = 256) {
  long b = (n + threads - 1) / threads;
  return (int)std::max(1L, std::min(b, 8L * num_sms()));
}

__global__ void gather_kernel(const double2* __restrict__ src, const int64_t* __restrict__ ro,
                              const int64_t* __restrict__ co, int nr, int nc,
                              double2* __restrict__ dst) {
  const long total = (long)nr * nc;
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < total;
       i += (long)gridDim.x * blockDim.x) {
    const int p = (int)(i / nc), c = (int)(i % nc);
    dst[i] = src[ro[p] + co[c]];
  }
}

__global__ void scatter_kernel(const double2* __restrict__ src, long ld,
                               const int64_t* __restrict__ ro, const int64_t* __restrict__ co,
                               int nr, int nc, double2* __restrict__ dst) {
  const long total = (long)nr * nc;
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < total;
       i += (long)gridDim.x * blockDim.x) {
    const int p = (int)(i / nc), c = (int)(i % nc);
    dst[ro[p] + co[c]] = src[(long)p * ld + c];
  }
}

__global__ void scale_kernel(const double2* __restrict__ in, double2* __restrict__ out, long n,
                             double2 alpha) {
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n;
       i += (long)gridDim.x * blockDim.x)
    out[i] = cmul(alpha, in[i]);
}

__global__ void sign_fix_kernel(double2* __restrict__ a, long n, const double2* __restrict__ r00,
                                double* __restrict__ nrm_out) {
  const double nrm = r00->x;
  if (blockIdx.x == 0 && threadIdx.x == 0) *nrm_out = fabs(nrm);
  if (!(nrm < 0.0)) return;
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n;
       i += (long)gridDim.x * blockDim.x) {
    const double2 v = a[i];
    a[i] = make_double2(-v.x, -v.y);
  }
}

// out[c][b][a] = in[a][b][c]; tiles of 32 x 32 over (a, c) per b
__global__ void transpose210_kernel(const double2* __restrict__ in, double2* __restrict__ out,
                                    int n0, int n1, int n2) {
  __shared__ double2 tile[32][33];
  const int b = blockIdx.z;
  const int a0 = blockIdx.y * 32, c0 = blockIdx.x * 32;
  for (int r = threadIdx.y; r < 32; r += blockDim.y) {
    const int a = a0 + r, c = c0 + threadIdx.x;
    if (a < n0 && c < n2) tile[r][threadIdx.x] = in[((long)a * n1 + b) * n2 + c];
  }
  __syncthreads();
  for (int r = threadIdx.y; r < 32; r += blockDim.y) {
    const int c = c0 + r, a = a0 + threadIdx.x;
    if (a < n0 && c < n2) out[((long)c * n1 + b) * n0 + a] = tile[threadIdx.x][r];
  }
}

}  // namespace

ptn_status gather(const double2* src, const int64_t* ro, const int64_t* co, int nr, int nc,
                  double2* dst, cudaStream_t st) {
  if ((long)nr * nc == 0) return PTN_OK;
  gather_kernel<<<grid_for((long)nr * nc), 256, 0, st>>>(src, ro, co, nr, nc, dst);
  PTN_LAUNCH_CHECK();
  note_launches(1);
  return PTN_OK;
}

ptn_status scatter(const double2* src, long ld, const int64_t* ro, const int64_t* co, int nr,
                   int nc, double2* dst, cudaStream_t st) {
  if ((long)nr * nc == 0) return PTN_OK;
  scatter_kernel<<<grid_for((long)nr * nc), 256, 0, st>>>(src, ld, ro, co, nr, nc, dst);
  PTN_LAUNCH_CHECK();
  note_launches(1);
  return PTN_OK;
}

ptn_status scale(const double2* in, double2* out, long n, double2 alpha, cudaStream_t st) {
  if (n == 0) return PTN_OK;
  scale_kernel<<<grid_for(n), 256, 0, st>>>(in, out, n, alpha);
  PTN_LAUNCH_CHECK();
  note_launches(1);
  return PTN_OK;
}

ptn_status sign_fix(double2* a, long n, const double2* r00, double* nrm_out, cudaStream_t st) {
  sign_fix_kernel<<<grid_for(n), 256, 0, st>>>(a, n, r00, nrm_out);
  PTN_LAUNCH_CHECK();
  note_launches(1);
  return PTN_OK;
}

ptn_status transpose210(const double2* in, double2* out, int n0, int n1, int n2, cudaStream_t st) {
  PTN_CHECK_ARG(n0 > 0 && n1 > 0 && n2 > 0 && n1 <= 65535, "transpose: bad shape");
  dim3 grid((n2 + 31) / 32, (n0 + 31) / 32, n1);
  PTN_CHECK_ARG(grid.y <= 65535, "transpose: n0 too large");
  transpose210_kernel<<<grid, dim3(32, 8), 0, st>>>(in, out, n0, n1, n2);
  PTN_LAUNCH_CHECK();
  note_launches(1);
  return PTN_OK;
}

}  // namespace ptn

using namespace ptn;

extern "C" {

int ptn_abi_version(void) { return PTN_ABI_VERSION; }
const char* ptn_version(void) { return "pytenet_gb300 0.1 (sm_103a)"; }
const char* ptn_last_error(void) { return g_err; }
uint64_t ptn_launch_count(void) { return g_launches.load(); }

ptn_status ptn_tune_set(int key, int value) {
  if (key < 0 || key >= PTN_TUNE_COUNT || value < 0 || value > kTuneMax[key]) {
    set_error("ptn_tune_set: bad key %d or value %d", key, value);
    return PTN_BAD_SHAPE;
  }
  g_tune[key].store(value);
  return PTN_OK;
}

int ptn_tune_get(int key) { return tune(key); }

void ptn_prof_start(unsigned kind_mask) {
  g_prof_used = 0;
  g_prof_mask = kind_mask;
}

ptn_status ptn_prof_read(int kind, double* total_ms, double* flops, double* bytes,
                         long* launches) {
  double ms = 0, fl = 0, by = 0;
  long n = 0;
  for (int i = 0; i < g_prof_used; ++i) {
    ProfSlot& p = g_prof[i];
    if (p.kind != kind) continue;
    float t = 0.f;
    PTN_CUDA_TRY(cudaEventElapsedTime(&t, p.a, p.b));
    ms += t;
    fl += p.flops;
    by += p.bytes;
    ++n;
  }
  *total_ms = ms;
  *flops = fl;
  *bytes = by;
  *launches = n;
  return PTN_OK;
}

void ptn_prof_stop(void) { g_prof_mask = 0; }

ptn_status ptn_gather(const ptn_c128* src, const int64_t* row_off, const int64_t* col_off, int nr,
                      int nc, ptn_c128* dst, void* stream) {
  return gather(reinterpret_cast<const double2*>(src), row_off, col_off, nr, nc,
                reinterpret_cast<double2*>(dst), as_stream(stream));
}

ptn_status ptn_scatter(const ptn_c128* src, long ld, const int64_t* row_off, const int64_t* col_off,
                       int nr, int nc, ptn_c128* dst, void* stream) {
  return scatter(reinterpret_cast<const double2*>(src), ld, row_off, col_off, nr, nc,
                 reinterpret_cast<double2*>(dst), as_stream(stream));
}

ptn_status ptn_scale(const ptn_c128* in, ptn_c128* out, long n, ptn_c128 alpha, void* stream) {
  return scale(reinterpret_cast<const double2*>(in), reinterpret_cast<double2*>(out), n,
               make_double2(alpha.re, alpha.im), as_stream(stream));
}

ptn_status ptn_sign_fix(ptn_c128* a, long n, const ptn_c128* r00, double* nrm_out, void* stream) {
  return sign_fix(reinterpret_cast<double2*>(a), n, reinterpret_cast<const double2*>(r00), nrm_out,
                  as_stream(stream));
}

ptn_status ptn_transpose_210(const ptn_c128* in, ptn_c128* out, int n0, int n1, int n2,
                             void* stream) {
  return transpose210(reinterpret_cast<const double2*>(in), reinterpret_cast<double2*>(out), n0,
                      n1, n2, as_stream(stream));
}

}  // extern "C"
