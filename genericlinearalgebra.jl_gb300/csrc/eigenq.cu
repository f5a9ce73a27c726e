// The Householder factorisation of the self-adjoint path exposed on its own:
// the counterparts of the reference's symtri! / SymmetricTridiagonalFactorization
// and of lmul! / rmul! with its EigenQ (src/eigenSelfAdjoint.jl:6-118, 446-504),
// for FP64 matrices in device memory.
//
//   gla_dsytrd: A = Q T Q' from the referenced triangle. On return, like the
//     reference's symtriLower!: d on the diagonal of A, e (the reflector
//     betas) on its first subdiagonal, reflector k stored in A[k+2:n, k]
//     below its implicit unit at row k+1, and tau. The other triangle is not
//     touched. An upper-stored input (uplo 'U') is read as its symmetric
//     lower counterpart and factored in the same lower layout.
//   gla_dormtr: C := op(Q) C (side 'L', C nq x ncol) or C op(Q) (side 'R',
//     C mrow x nq), op = identity ('N') or transpose ('T'), Q of order nq from
//     gla_dsytrd's A and tau (the reference's lmul!(Q, B) and rmul!(B, Q)).
//
// Both run on the large path's kernels (cooperative panel reduction, blocked
// compact-WY application) with a cached context per order.
#include <cuda_runtime.h>
#include <stdint.h>

#include <map>
#include <mutex>

#include "../../include/glagpu.h"
#include "gla_large.h"

namespace gla {
namespace {

// Lower-stored working copy (zeros above the diagonal) of the referenced
// triangle.
__global__ void k_q_load(const double* __restrict__ A, long long lda, int n, int lower, double* __restrict__ W) {
  const int j = blockIdx.y;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    W[i + (long long)j * n] = i < j ? 0.0 : (lower ? A[i + (long long)j * lda] : A[j + (long long)i * lda]);
}

// A's lower triangle := the factorisation: d on the diagonal, e below it,
// the reflectors' stored parts below that.
__global__ void k_q_store(const double* __restrict__ W, int n, const double* __restrict__ d,
                          const double* __restrict__ e, double* __restrict__ A, long long lda) {
  const int j = blockIdx.y;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    if (i < j) continue;
    double v;
    if (i == j)
      v = d[j];
    else if (i == j + 1)
      v = e[j];
    else
      v = W[i + (long long)j * n];
    A[i + (long long)j * lda] = v;
  }
}

// out (cols x rows, leading dimension ldo) = in' (in: rows x cols, ldi).
__global__ void k_q_transpose(const double* __restrict__ in, long long ldi, int rows, int cols,
                              double* __restrict__ out, long long ldo) {
  __shared__ double t[32][33];
  const int r0 = blockIdx.x * 32, c0 = blockIdx.y * 32;
  for (int k = threadIdx.y; k < 32; k += 8) {
    const int r = r0 + threadIdx.x, c = c0 + k;
    if (r < rows && c < cols) t[k][threadIdx.x] = in[r + (long long)c * ldi];
  }
  __syncthreads();
  for (int k = threadIdx.y; k < 32; k += 8) {
    const int c = c0 + threadIdx.x, r = r0 + k;
    if (r < rows && c < cols) out[c + (long long)r * ldo] = t[threadIdx.x][k];
  }
}

struct QCtx {
  LargeCtx* c = nullptr;
  double* tmp = nullptr;  // gla_dormtr side 'R': the transposed C
  size_t tmp_elems = 0;
};
std::mutex g_q_mu;
std::map<int, QCtx> g_q;

int q_ctx(int n, QCtx** out) {
  auto it = g_q.find(n);
  if (it == g_q.end()) {
    QCtx q;
    int rc = large_create(&q.c, n, true);
    if (rc) return rc;
    it = g_q.emplace(n, q).first;
  }
  *out = &it->second;
  return 0;
}

#define Q_CUDA(x)                                   \
  do {                                              \
    cudaError_t e_ = (x);                           \
    if (e_ != cudaSuccess) return -1000 - (int)e_;  \
  } while (0)

}  // namespace
}  // namespace gla

using namespace gla;

extern "C" {

int gla_dsytrd(char uplo, int64_t n, double* A, int64_t lda, double* d, double* e, double* tau, void* stream) {
  if (uplo != 'L' && uplo != 'U') return -1;
  if (n < 0 || n > GLA_MAX_N) return -2;
  if (!A && n) return -3;
  if (lda < (n > 1 ? n : 1)) return -4;
  if (!d && n) return -5;
  if (!e && n > 1) return -6;
  if (!tau && n > 1) return -7;
  if (n == 0) return 0;
  cudaStream_t st = (cudaStream_t)stream;
  std::lock_guard<std::mutex> lk(g_q_mu);
  QCtx* q = nullptr;
  int rc = q_ctx((int)n, &q);
  if (rc) return rc;
  const int nn = (int)n;
  const dim3 g2((nn + 255) / 256, nn);
  double* W = (double*)large_work_matrix(q->c);
  k_q_load<<<g2, 256, 0, st>>>(A, lda, nn, uplo == 'L', W);
  Q_CUDA(cudaGetLastError());
  if (n == 1) {
    Q_CUDA(cudaMemcpyAsync(d, W, sizeof(double), cudaMemcpyDeviceToDevice, st));
  } else {
    rc = large_sytrd(q->c, W, nn, d, e, tau, st);
    if (rc) return rc;
  }
  k_q_store<<<g2, 256, 0, st>>>(W, nn, d, n > 1 ? e : d, A, lda);
  Q_CUDA(cudaGetLastError());
  return 0;
}

int gla_dormtr(char side, char trans, int64_t m, int64_t n, const double* A, int64_t lda, const double* tau,
               double* C, int64_t ldc, void* stream) {
  if (side != 'L' && side != 'R') return -1;
  if (trans != 'N' && trans != 'T') return -2;
  if (m < 0) return -3;
  if (n < 0) return -4;
  const int64_t nq = side == 'L' ? m : n;
  if (nq > GLA_MAX_N) return side == 'L' ? -3 : -4;
  if (!A && nq) return -5;
  if (lda < (nq > 1 ? nq : 1)) return -6;
  if (!tau && nq > 1) return -7;
  if (!C && m && n) return -8;
  if (ldc < (m > 1 ? m : 1)) return -9;
  if (m == 0 || n == 0 || nq < 2) return 0;  // Q of order 0 or 1 is the identity
  cudaStream_t st = (cudaStream_t)stream;
  std::lock_guard<std::mutex> lk(g_q_mu);
  QCtx* q = nullptr;
  int rc = q_ctx((int)nq, &q);
  if (rc) return rc;
  if (side == 'L') return large_ormtr(q->c, A, lda, tau, C, ldc, st, (int)n, trans == 'T');
  // C op(Q) = (op(Q)' C')': transpose C (m x nq) into nq x m, apply op(Q)',
  // transpose back
  const size_t need = (size_t)nq * (size_t)m;
  if (q->tmp_elems < need) {
    Q_CUDA(cudaStreamSynchronize(st));
    cudaFree(q->tmp);
    q->tmp = nullptr;
    q->tmp_elems = 0;
    Q_CUDA(cudaMalloc((void**)&q->tmp, sizeof(double) * need));
    q->tmp_elems = need;
  }
  const dim3 tb(32, 8);
  k_q_transpose<<<dim3((unsigned)((m + 31) / 32), (unsigned)((nq + 31) / 32)), tb, 0, st>>>(C, ldc, (int)m, (int)nq,
                                                                                            q->tmp, nq);
  Q_CUDA(cudaGetLastError());
  rc = large_ormtr(q->c, A, lda, tau, q->tmp, nq, st, (int)m, trans == 'N');
  if (rc) return rc;
  k_q_transpose<<<dim3((unsigned)((nq + 31) / 32), (unsigned)((m + 31) / 32)), tb, 0, st>>>(q->tmp, nq, (int)nq,
                                                                                             (int)m, C, ldc);
  Q_CUDA(cudaGetLastError());
  return 0;
}

// Host-buffer forms (stage through the device, synchronize).
int gla_dsytrd_host(char uplo, int64_t n, double* A, int64_t lda, double* d, double* e, double* tau) {
  if (uplo != 'L' && uplo != 'U') return -1;
  if (n < 0 || n > GLA_MAX_N) return -2;
  if (!A && n) return -3;
  if (lda < (n > 1 ? n : 1)) return -4;
  if (!d && n) return -5;
  if (!e && n > 1) return -6;
  if (!tau && n > 1) return -7;
  if (n == 0) return 0;
  const size_t nn = (size_t)n * n, ne = n > 1 ? (size_t)n - 1 : 1;
  double* buf = nullptr;
  Q_CUDA(cudaMalloc((void**)&buf, sizeof(double) * (nn + n + 2 * ne)));
  double *dA = buf, *dd = buf + nn, *de = dd + n, *dt = de + ne;
  cudaError_t err = cudaMemcpy2D(dA, sizeof(double) * n, A, sizeof(double) * lda, sizeof(double) * n, n,
                                 cudaMemcpyHostToDevice);
  int rc = err == cudaSuccess ? gla_dsytrd(uplo, n, dA, n, dd, de, dt, nullptr) : -1000 - (int)err;
  if (rc == 0) {
    err = cudaMemcpy2D(A, sizeof(double) * lda, dA, sizeof(double) * n, sizeof(double) * n, n, cudaMemcpyDeviceToHost);
    if (err == cudaSuccess) err = cudaMemcpy(d, dd, sizeof(double) * n, cudaMemcpyDeviceToHost);
    if (err == cudaSuccess && n > 1) err = cudaMemcpy(e, de, sizeof(double) * (n - 1), cudaMemcpyDeviceToHost);
    if (err == cudaSuccess && n > 1) err = cudaMemcpy(tau, dt, sizeof(double) * (n - 1), cudaMemcpyDeviceToHost);
    if (err != cudaSuccess) rc = -1000 - (int)err;
  }
  cudaFree(buf);
  return rc;
}

int gla_dormtr_host(char side, char trans, int64_t m, int64_t n, const double* A, int64_t lda, const double* tau,
                    double* C, int64_t ldc) {
  if (side != 'L' && side != 'R') return -1;
  if (trans != 'N' && trans != 'T') return -2;
  if (m < 0) return -3;
  if (n < 0) return -4;
  const int64_t nq = side == 'L' ? m : n;
  if (nq > GLA_MAX_N) return side == 'L' ? -3 : -4;
  if (!A && nq) return -5;
  if (lda < (nq > 1 ? nq : 1)) return -6;
  if (!tau && nq > 1) return -7;
  if (!C && m && n) return -8;
  if (ldc < (m > 1 ? m : 1)) return -9;
  if (m == 0 || n == 0 || nq < 2) return 0;
  const size_t qa = (size_t)nq * nq, cc = (size_t)m * n;
  double* buf = nullptr;
  Q_CUDA(cudaMalloc((void**)&buf, sizeof(double) * (qa + nq + cc)));
  double *dA = buf, *dt = buf + qa, *dC = dt + nq;
  cudaError_t err = cudaMemcpy2D(dA, sizeof(double) * nq, A, sizeof(double) * lda, sizeof(double) * nq, nq,
                                 cudaMemcpyHostToDevice);
  if (err == cudaSuccess) err = cudaMemcpy(dt, tau, sizeof(double) * (nq - 1), cudaMemcpyHostToDevice);
  if (err == cudaSuccess)
    err = cudaMemcpy2D(dC, sizeof(double) * m, C, sizeof(double) * ldc, sizeof(double) * m, n, cudaMemcpyHostToDevice);
  int rc = err == cudaSuccess ? gla_dormtr(side, trans, m, n, dA, nq, dt, dC, m, nullptr) : -1000 - (int)err;
  if (rc == 0) {
    err = cudaMemcpy2D(C, sizeof(double) * ldc, dC, sizeof(double) * m, sizeof(double) * m, n, cudaMemcpyDeviceToHost);
    if (err != cudaSuccess) rc = -1000 - (int)err;
  }
  cudaFree(buf);
  return rc;
}

}  // extern "C"
