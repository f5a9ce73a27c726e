// Spectrum slicing on a symmetric tridiagonal matrix T = SymTridiagonal(a, b):
//
//   gla_numnegevals: the reference's numnegevals (src/tridiag.jl:20-36), the
//     number of negative eigenvalues of T - sigma I, for many shifts at once
//     (one thread per shift). The Sturm (LDL') recurrence of Parlett, "The
//     symmetric eigenvalue problem" 3.3.1,
//       delta_1 = a_1 - sigma,
//       delta_{k+1} = (a_{k+1} - sigma) - b_k (b_k / delta_k),
//     with a zero delta replaced by eps (b_k + eps) as the reference does, is
//     evaluated with explicitly rounded operations (no contraction into
//     fused multiply-adds), so the counts equal the reference's bit for bit.
//   gla_dstebz: eigenvalues il..iu (ascending, 1-based) by multisection: one
//     warp per eigenvalue, its 32 lanes evaluating the count at 32 interior
//     points of the current bracket, which shrinks 33-fold per step, from the
//     Gershgorin interval down to max(abstol, 2 eps max|bracket ends|).
#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/glagpu.h"

namespace {

constexpr double kEps = 0x1p-52;  // eps(Float64)

__device__ __forceinline__ int64_t sturm_count(const double* __restrict__ a, const double* __restrict__ b, int64_t n,
                                               double sigma) {
  double delta = __dsub_rn(a[0], sigma);
  int64_t nu = delta < 0.0 ? 1 : 0;
  for (int64_t k = 0; k + 1 < n; k++) {
    if (delta == 0.0) delta = __dmul_rn(kEps, __dadd_rn(b[k], kEps));
    const double bk = b[k];
    delta = __dsub_rn(__dsub_rn(a[k + 1], sigma), __dmul_rn(bk, __ddiv_rn(bk, delta)));
    nu += delta < 0.0 ? 1 : 0;
  }
  return nu;
}

__global__ void __launch_bounds__(128) k_sturm_counts(int64_t n, const double* __restrict__ a,
                                                      const double* __restrict__ b, int64_t m,
                                                      const double* __restrict__ sigma, int64_t* __restrict__ counts) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i < m) counts[i] = sturm_count(a, b, n, sigma[i]);
}

// One warp per eigenvalue index il - 1 + warp.
__global__ void __launch_bounds__(128) k_stebz(int64_t n, const double* __restrict__ a, const double* __restrict__ b,
                                               int64_t il, int64_t count, double abstol, double* __restrict__ w) {
  const int lane = threadIdx.x & 31;
  const int64_t j = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
  if (j >= count) return;
  const int64_t target = il - 1 + j;  // 0-based index: count(lo) <= target < count(hi)
  // Gershgorin interval, widened so that count(lo) = 0 and count(hi) = n
  double glo = INFINITY, ghi = -INFINITY;
  for (int64_t k = lane; k < n; k += 32) {
    const double r = (k > 0 ? fabs(b[k - 1]) : 0.0) + (k + 1 < n ? fabs(b[k]) : 0.0);
    glo = fmin(glo, a[k] - r);
    ghi = fmax(ghi, a[k] + r);
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    glo = fmin(glo, __shfl_xor_sync(0xffffffffu, glo, o));
    ghi = fmax(ghi, __shfl_xor_sync(0xffffffffu, ghi, o));
  }
  const double span = fmax(ghi - glo, fmax(fabs(glo), fabs(ghi)) * kEps);
  double lo = glo - 2.0 * span * kEps - 2.0 * abstol - 1e-300;
  double hi = ghi + 2.0 * span * kEps + 2.0 * abstol + 1e-300;
  for (int step = 0; step < 64; step++) {
    const double tol = fmax(abstol, 2.0 * kEps * fmax(fabs(lo), fabs(hi)));
    if (hi - lo <= tol) break;
    const double x = lo + (hi - lo) * ((double)(lane + 1) / 33.0);
    const bool inside = x > lo && x < hi;
    const int64_t c = inside ? sturm_count(a, b, n, x) : 0;
    // lanes whose point has at most `target` eigenvalues below it move lo up,
    // the others move hi down; points are increasing in the lane index
    const unsigned below = __ballot_sync(0xffffffffu, inside && c <= target);
    const unsigned above = __ballot_sync(0xffffffffu, inside && c > target);
    double nlo = lo, nhi = hi;
    if (below) nlo = __shfl_sync(0xffffffffu, x, 31 - __clz(below));
    if (above) nhi = __shfl_sync(0xffffffffu, x, __ffs(above) - 1);
    if (nlo == lo && nhi == hi) break;  // no representable interior point left
    lo = nlo;
    hi = nhi;
  }
  if (lane == 0) w[j] = 0.5 * (lo + hi);
}

}  // namespace

extern "C" {

int gla_numnegevals(int64_t n, const double* d, const double* e, int64_t m, const double* sigma, int64_t* counts,
                    void* stream) {
  if (n < 0) return -1;
  if (!d && n) return -2;
  if (!e && n > 1) return -3;
  if (m < 0) return -4;
  if (!sigma && m) return -5;
  if (!counts && m) return -6;
  if (m == 0) return 0;
  cudaStream_t st = (cudaStream_t)stream;
  if (n == 0) {
    cudaError_t err = cudaMemsetAsync(counts, 0, sizeof(int64_t) * m, st);
    return err == cudaSuccess ? 0 : -1000 - (int)err;
  }
  k_sturm_counts<<<(unsigned)((m + 127) / 128), 128, 0, st>>>(n, d, e, m, sigma, counts);
  const cudaError_t err = cudaGetLastError();
  return err == cudaSuccess ? 0 : -1000 - (int)err;
}

int gla_dstebz(int64_t n, const double* d, const double* e, int64_t il, int64_t iu, double abstol, double* w,
               void* stream) {
  if (n < 0) return -1;
  if (!d && n) return -2;
  if (!e && n > 1) return -3;
  if (il < 1 || (n > 0 && il > n)) return -4;
  if (iu < il - 1 || iu > n) return -5;
  if (!(abstol >= 0.0)) return -6;
  const int64_t count = iu - il + 1;
  if (count <= 0) return 0;
  if (!w) return -7;
  const int64_t threads = count * 32;
  k_stebz<<<(unsigned)((threads + 127) / 128), 128, 0, (cudaStream_t)stream>>>(n, d, e, il, count, abstol, w);
  const cudaError_t err = cudaGetLastError();
  return err == cudaSuccess ? 0 : -1000 - (int)err;
}

// Host-buffer forms (stage through the device, synchronize).
int gla_numnegevals_host(int64_t n, const double* d, const double* e, int64_t m, const double* sigma,
                         int64_t* counts) {
  if (n < 0) return -1;
  if (!d && n) return -2;
  if (!e && n > 1) return -3;
  if (m < 0) return -4;
  if (!sigma && m) return -5;
  if (!counts && m) return -6;
  if (m == 0) return 0;
  const int64_t ne = n > 1 ? n - 1 : 0;
  double* buf = nullptr;
  int64_t* dc = nullptr;
  cudaError_t err = cudaMalloc((void**)&buf, sizeof(double) * (n + ne + m + 1));
  if (err == cudaSuccess) err = cudaMalloc((void**)&dc, sizeof(int64_t) * m);
  if (err == cudaSuccess && n) err = cudaMemcpy(buf, d, sizeof(double) * n, cudaMemcpyHostToDevice);
  if (err == cudaSuccess && ne) err = cudaMemcpy(buf + n, e, sizeof(double) * ne, cudaMemcpyHostToDevice);
  if (err == cudaSuccess) err = cudaMemcpy(buf + n + ne, sigma, sizeof(double) * m, cudaMemcpyHostToDevice);
  int rc = err == cudaSuccess ? gla_numnegevals(n, buf, buf + n, m, buf + n + ne, dc, nullptr) : -1000 - (int)err;
  if (rc == 0) {
    err = cudaMemcpy(counts, dc, sizeof(int64_t) * m, cudaMemcpyDeviceToHost);
    if (err != cudaSuccess) rc = -1000 - (int)err;
  }
  cudaFree(buf);
  cudaFree(dc);
  return rc;
}

int gla_dstebz_host(int64_t n, const double* d, const double* e, int64_t il, int64_t iu, double abstol, double* w) {
  if (n < 0) return -1;
  if (!d && n) return -2;
  if (!e && n > 1) return -3;
  if (il < 1 || (n > 0 && il > n)) return -4;
  if (iu < il - 1 || iu > n) return -5;
  if (!(abstol >= 0.0)) return -6;
  const int64_t count = iu - il + 1;
  if (count <= 0) return 0;
  if (!w) return -7;
  const int64_t ne = n > 1 ? n - 1 : 0;
  double* buf = nullptr;
  cudaError_t err = cudaMalloc((void**)&buf, sizeof(double) * (n + ne + count + 1));
  if (err == cudaSuccess) err = cudaMemcpy(buf, d, sizeof(double) * n, cudaMemcpyHostToDevice);
  if (err == cudaSuccess && ne) err = cudaMemcpy(buf + n, e, sizeof(double) * ne, cudaMemcpyHostToDevice);
  int rc = err == cudaSuccess ? gla_dstebz(n, buf, buf + n, il, iu, abstol, buf + n + ne, nullptr) : -1000 - (int)err;
  if (rc == 0) {
    err = cudaMemcpy(w, buf + n + ne, sizeof(double) * count, cudaMemcpyDeviceToHost);
    if (err != cudaSuccess) rc = -1000 - (int)err;
  }
  cudaFree(buf);
  return rc;
}

}  // extern "C"
