// gla_dsyev_static: the single-matrix FP64 eigensolver of gla_dsyev, with
// every piece of scratch memory it needs taken from one file-scope device
// array instead of cudaMalloc.
//
// Why: some callers cannot allocate device memory at the moment they need an
// eigen-decomposition. Examples are an application whose allocator has
// already reserved the whole device, a latency-critical loop where
// cudaMalloc/cudaFree would synchronize the device, and a process whose
// memory budget is fixed at start-up. Such callers still own the inputs and
// outputs (A, w) and pass them in; everything else lives in g_scratch.
//
// The array is sized for orders up to GLA_STATIC_MAX_N (128): rotation log
// (2 n^2 + 4 rotations), sweep headers, d, e, chase state, the packed matrix
// and a few counters, about 660 KB. Every GPU that loads this library holds
// it until the process exits. All calls share it and it keeps the contents
// of the last call: the entry point re-initialises everything that must
// start at zero (descriptor, chase state, counters) on each call, and calls
// whose work overlaps on the GPU (concurrent streams, or several host
// threads on one device) race on it and must be serialised by the caller.
#include <cuda_runtime.h>

#include <algorithm>
#include <mutex>

#include "../../include/glagpu.h"
#include "gla_launch.h"

namespace gla {
cudaError_t tridiag_kernels_init();
cudaError_t chase_kernels_init();
cudaError_t apply_kernels_init();
}  // namespace gla

using namespace gla;

namespace {

constexpr int kN = GLA_STATIC_MAX_N;
constexpr size_t al256(size_t x) { return (x + 255) / 256 * 256; }
constexpr size_t kOffDesc = 0;
constexpr size_t kOffPerm = kOffDesc + al256(sizeof(SmallDesc));
constexpr size_t kOffD = kOffPerm + al256(sizeof(int));
constexpr size_t kOffE = kOffD + al256(sizeof(double) * kN);
constexpr size_t kOffCst = kOffE + al256(sizeof(double) * kN);
constexpr size_t kOffPend = kOffCst + al256(sizeof(ChaseState));
constexpr size_t kOffStats = kOffPend + al256(sizeof(int));
constexpr size_t kOffInfo = kOffStats + al256(4 * sizeof(unsigned long long));
constexpr size_t kOffHdr = kOffInfo + al256(sizeof(int));
constexpr size_t kOffRot = kOffHdr + al256(sizeof(unsigned) * (3 * kN + 4));
constexpr size_t kOffQ = kOffRot + al256(2 * sizeof(double) * (2 * (size_t)kN * kN + 4));
constexpr size_t kScratchBytes = kOffQ + al256(sizeof(double) * (size_t)kN * kN);

__device__ __align__(256) unsigned char g_scratch[kScratchBytes];

constexpr int kMaxDevices = 64;
std::mutex g_mu;
char* g_addr[kMaxDevices] = {};
bool g_init[kMaxDevices] = {};

// Device address of g_scratch on the current device (host code cannot use the
// symbol itself as a device pointer). Looked up once per device, together
// with the kernels' shared-memory limits.
int scratch_base(char** out) {
  int dev = -1;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return -1000 - (int)e;
  if (dev < 0 || dev >= kMaxDevices) return -1000 - (int)cudaErrorInvalidDevice;
  std::lock_guard<std::mutex> lk(g_mu);
  if (!g_addr[dev]) {
    void* p = nullptr;
    e = cudaGetSymbolAddress(&p, g_scratch);
    if (e != cudaSuccess) return -1000 - (int)e;
    g_addr[dev] = static_cast<char*>(p);
  }
  if (!g_init[dev]) {
    if ((e = tridiag_kernels_init()) != cudaSuccess) return -1000 - (int)e;
    if ((e = chase_kernels_init()) != cudaSuccess) return -1000 - (int)e;
    if ((e = apply_kernels_init()) != cudaSuccess) return -1000 - (int)e;
    g_init[dev] = true;
  }
  *out = g_addr[dev];
  return 0;
}

// Writes the one-matrix descriptor and permutation (reset on every call).
__global__ void k_static_setup(SmallDesc* desc, int* perm, int n) {
  SmallDesc d;
  d.n = n;
  d.pad = 0;
  d.a_off = 0;
  d.w_off = 0;
  d.rot_off = 0;
  d.hdr_off = 0;
  d.rot_cap = 2 * n * n + 4;
  d.hdr_cap = 3 * n + 4;
  *desc = d;
  *perm = 0;
}

#define GLA_CUDA(x)                                \
  do {                                             \
    cudaError_t e_ = (x);                          \
    if (e_ != cudaSuccess) return -1000 - (int)e_; \
  } while (0)

}  // namespace

extern "C" int gla_dsyev_static(char jobz, char uplo, int64_t n, double* A, int64_t lda, double* w, int* info,
                                void* stream) {
  if (jobz != 'V' && jobz != 'N') return -1;
  if (uplo != 'L' && uplo != 'U') return -2;
  if (n < 0) return -3;
  if (n > GLA_STATIC_MAX_N) return GLA_ERR_STATIC_TOO_LARGE;
  if (!A && n) return -4;
  if (lda < std::max<int64_t>(1, n)) return -5;
  if (!w && n) return -6;
  if (!info) return -7;
  *info = 0;
  if (n == 0) return 0;
  char* base = nullptr;
  int rc = scratch_base(&base);
  if (rc) return rc;
  cudaStream_t st = (cudaStream_t)stream;
  SmallDesc* desc = reinterpret_cast<SmallDesc*>(base + kOffDesc);
  int* perm = reinterpret_cast<int*>(base + kOffPerm);
  double* d = reinterpret_cast<double*>(base + kOffD);
  double* e = reinterpret_cast<double*>(base + kOffE);
  ChaseState* cst = reinterpret_cast<ChaseState*>(base + kOffCst);
  int* pending = reinterpret_cast<int*>(base + kOffPend);
  unsigned long long* stats = reinterpret_cast<unsigned long long*>(base + kOffStats);
  int* dinfo = reinterpret_cast<int*>(base + kOffInfo);
  unsigned* hdr = reinterpret_cast<unsigned*>(base + kOffHdr);
  double* rot = reinterpret_cast<double*>(base + kOffRot);
  double* Q = reinterpret_cast<double*>(base + kOffQ);
  const int nn = (int)n;
  const int nt = std::max(32, (nn + 31) / 32 * 32);
  const bool wantq = jobz == 'V';

  k_static_setup<<<1, 1, 0, st>>>(desc, perm, nn);
  GLA_CUDA(cudaGetLastError());
  GLA_CUDA(cudaMemsetAsync(stats, 0, 4 * sizeof(unsigned long long), st));
  GLA_CUDA(cudaMemsetAsync(dinfo, 0, sizeof(int), st));
  GLA_CUDA(cudaMemcpy2DAsync(Q, sizeof(double) * n, A, sizeof(double) * lda, sizeof(double) * n, n,
                             cudaMemcpyDeviceToDevice, st));
  GLA_CUDA(launch_tridiag(kF64, wantq, 1, nt, tridiag_smem_bytes(nn, nt, 8), st, desc, perm, Q, uplo == 'L', d, e, Q,
                          dinfo, cst, nullptr));
  if (wantq) {
    for (int pass = 0; pass < kMaxPasses; pass++) {
      GLA_CUDA(cudaMemsetAsync(pending, 0, sizeof(int), st));
      GLA_CUDA(launch_chase(kF64, kAlgoQL, 1, chase_smem_bytes(nn, 8), st, desc, perm, d, e, cst, rot, hdr, dinfo,
                            kTolF64, kMaxSweepsPerN, pending, stats));
      GLA_CUDA(launch_apply(kF64, 1, nt, apply_smem_bytes(nn, 8), st, desc, perm, Q, d, w, cst, rot, hdr, dinfo,
                            nullptr));
      int more = 0;
      GLA_CUDA(cudaMemcpyAsync(&more, pending, sizeof(int), cudaMemcpyDeviceToHost, st));
      GLA_CUDA(cudaStreamSynchronize(st));
      if (more == 0) break;
    }
    GLA_CUDA(cudaMemcpy2DAsync(A, sizeof(double) * lda, Q, sizeof(double) * n, sizeof(double) * n, n,
                               cudaMemcpyDeviceToDevice, st));
  } else {
    GLA_CUDA(launch_chase(kF64, kAlgoPWK, 1, chase_smem_bytes(nn, 8), st, desc, perm, d, e, cst, nullptr, nullptr,
                          dinfo, kTolF64, kMaxSweepsPerN, pending, stats));
    GLA_CUDA(launch_sort_values(kF64, 1, st, desc, perm, d, w, dinfo, nullptr));
  }
  GLA_CUDA(cudaMemcpyAsync(info, dinfo, sizeof(int), cudaMemcpyDeviceToHost, st));
  GLA_CUDA(cudaStreamSynchronize(st));
  return *info != 0;
}
