// The Householder factorisation of the self-adjoint path exposed on its own:
// the counterparts of the reference's symtri! / SymmetricTridiagonalFactorization
// and of lmul! / rmul! with its EigenQ (src/eigenSelfAdjoint.jl:6-118, 446-504),
// for FP64 matrices in device memory.
//
//   gla_dsytrd: A = Q T Q' from the referenced triangle, in that triangle's
//     layout. uplo 'L' (symtriLower!, :450-504): d on the diagonal of A, e
//     (the reflector betas) on its first subdiagonal, reflector k stored in
//     A[k+2:n, k] below its implicit unit at row k+1. uplo 'U'
//     (symtriUpper!, :507-564): e on the first superdiagonal, reflector k in
//     A[1:n-k-1, n-k+1] above its implicit unit at row n-k. tau in both. The
//     other triangle is not touched.
//   gla_dormtr: C := op(Q) C (side 'L', C nq x ncol) or C op(Q) (side 'R',
//     C mrow x nq), op = identity ('N') or transpose ('T'), Q of order nq from
//     gla_dsytrd's A and tau with the same uplo (the reference's lmul!(Q, B)
//     and rmul!(B, Q)).
//
// Both run on the large path's kernels (cooperative panel reduction, blocked
// compact-WY application) with a cached context per order. The upper form
// is the lower one of the reversed matrix: with P the reversal permutation,
// symtriUpper!(A) takes the same reflectors, in the same order, as
// symtriLower!(P A P) (reflector k of the upper form is the reversed column
// of the lower one), so its factors are the lower factors reversed in both
// indices, its d and e the lower ones reversed, tau the same, and
// Q_U = P Q_L P. The two differ only in the summation order of the products
// inside each step.
#include <cuda_runtime.h>
#include <stdint.h>

#include <algorithm>
#include <map>
#include <mutex>

#include "../../include/glagpu.h"
#include "gla_large.h"

namespace gla {
namespace {

// Lower-stored working copy W (zeros above the diagonal) of the lower
// triangle (lower) or of the reversed upper triangle, W[i, j] =
// A[n-1-i, n-1-j] (!lower).
__global__ void k_q_load(const double* __restrict__ A, long long lda, int n, int lower, double* __restrict__ W) {
  const int j = blockIdx.y;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    W[i + (long long)j * n] =
        i < j ? 0.0 : (lower ? A[i + (long long)j * lda] : A[(n - 1 - i) + (long long)(n - 1 - j) * lda]);
}

// The factorisation into A's referenced triangle: d on the diagonal, e next
// to it, the reflectors' stored parts beyond (reversed back for !lower).
__global__ void k_q_store(const double* __restrict__ W, int n, const double* __restrict__ d,
                          const double* __restrict__ e, int lower, double* __restrict__ A, long long lda) {
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
    if (lower)
      A[i + (long long)j * lda] = v;
    else
      A[(n - 1 - i) + (long long)(n - 1 - j) * lda] = v;
  }
}

// x[0 .. len-1] reversed in place
__global__ void k_q_reverse(double* __restrict__ x, int len) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < len / 2; i += gridDim.x * blockDim.x) {
    const double t = x[i];
    x[i] = x[len - 1 - i];
    x[len - 1 - i] = t;
  }
}

// F (nq x nq, lower part) = the lower-layout factors of an upper
// factorisation: F[i, j] = A[nq-1-i, nq-1-j] for i >= j.
__global__ void k_q_revfactors(const double* __restrict__ A, long long lda, int nq, double* __restrict__ F) {
  const int j = blockIdx.y;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < nq; i += gridDim.x * blockDim.x)
    F[i + (long long)j * nq] = i < j ? 0.0 : A[(nq - 1 - i) + (long long)(nq - 1 - j) * lda];
}

// out = P in (rows reversed; in, out: rows x cols)
__global__ void k_q_revrows(const double* __restrict__ in, long long ldi, int rows, int cols,
                            double* __restrict__ out, long long ldo) {
  for (int c = blockIdx.y; c < cols; c += gridDim.y)
    for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < rows; r += gridDim.x * blockDim.x)
      out[r + (long long)c * ldo] = in[(rows - 1 - r) + (long long)c * ldi];
}

// out (cols x rows, leading dimension ldo) = in' (in: rows x cols, ldi);
// flip 1: out's rows reversed (out = P in'); flip 2: in's rows reversed
// (out = (P in)').
__global__ void k_q_transpose(const double* __restrict__ in, long long ldi, int rows, int cols,
                              double* __restrict__ out, long long ldo, int flip) {
  __shared__ double t[32][33];
  const int r0 = blockIdx.x * 32;
  for (int c0 = blockIdx.y * 32; c0 < cols; c0 += gridDim.y * 32) {  // column tiles beyond the grid's y limit
    for (int k = threadIdx.y; k < 32; k += 8) {
      const int r = r0 + threadIdx.x, c = c0 + k;
      if (r < rows && c < cols) t[k][threadIdx.x] = in[(flip == 2 ? rows - 1 - r : r) + (long long)c * ldi];
    }
    __syncthreads();
    for (int k = threadIdx.y; k < 32; k += 8) {
      const int c = c0 + threadIdx.x, r = r0 + k;
      if (r < rows && c < cols) out[(flip == 1 ? cols - 1 - c : c) + (long long)r * ldo] = t[threadIdx.x][k];
    }
    __syncthreads();
  }
}

unsigned grid_y(long long n) { return (unsigned)std::min<long long>(std::max<long long>(n, 1), 65535); }

struct QCtx {
  LargeCtx* c = nullptr;
  double* tmp = nullptr;  // gla_dormtr: C transposed or reversed
  size_t tmp_elems = 0;
  double* frev = nullptr;  // gla_dormtr uplo 'U': the factors in the lower layout
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

// q->tmp holds at least need doubles (the stream is drained before a
// reallocation).
cudaError_t q_tmp(QCtx* q, size_t need, cudaStream_t st) {
  if (q->tmp_elems >= need) return cudaSuccess;
  cudaError_t e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) return e;
  cudaFree(q->tmp);
  q->tmp = nullptr;
  q->tmp_elems = 0;
  e = cudaMalloc((void**)&q->tmp, sizeof(double) * need);
  if (e == cudaSuccess) q->tmp_elems = need;
  return e;
}

}  // namespace

// Frees the per-order contexts cached by gla_dsytrd / gla_dormtr (the caller
// has drained the device).
void release_eigenq_cache() {
  std::lock_guard<std::mutex> lk(g_q_mu);
  for (auto& kv : g_q) {
    large_destroy(kv.second.c);
    cudaFree(kv.second.tmp);
    cudaFree(kv.second.frev);
  }
  g_q.clear();
}

namespace {

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
  const int nn = (int)n, lower = uplo == 'L';
  const dim3 g2((nn + 255) / 256, nn);
  double* W = (double*)large_work_matrix(q->c);
  k_q_load<<<g2, 256, 0, st>>>(A, lda, nn, lower, W);
  Q_CUDA(cudaGetLastError());
  if (n == 1) {
    Q_CUDA(cudaMemcpyAsync(d, W, sizeof(double), cudaMemcpyDeviceToDevice, st));
  } else {
    rc = large_sytrd(q->c, W, nn, d, e, tau, st);
    if (rc) return rc;
  }
  k_q_store<<<g2, 256, 0, st>>>(W, nn, d, n > 1 ? e : d, lower, A, lda);
  Q_CUDA(cudaGetLastError());
  if (!lower) {  // the upper form's d and e are the reversed matrix's, reversed
    k_q_reverse<<<(nn + 511) / 512, 256, 0, st>>>(d, nn);
    Q_CUDA(cudaGetLastError());
    if (n > 1) {
      k_q_reverse<<<(nn + 511) / 512, 256, 0, st>>>(e, nn - 1);
      Q_CUDA(cudaGetLastError());
    }
  }
  return 0;
}

int gla_dormtr(char side, char uplo, char trans, int64_t m, int64_t n, const double* A, int64_t lda,
               const double* tau, double* C, int64_t ldc, void* stream) {
  if (side != 'L' && side != 'R') return -1;
  if (uplo != 'L' && uplo != 'U') return -2;
  if (trans != 'N' && trans != 'T') return -3;
  if (m < 0) return -4;
  if (n < 0) return -5;
  const int64_t nq = side == 'L' ? m : n;
  if (nq > GLA_MAX_N) return side == 'L' ? -4 : -5;
  if (!A && nq) return -6;
  if (lda < (nq > 1 ? nq : 1)) return -7;
  if (!tau && nq > 1) return -8;
  if (!C && m && n) return -9;
  if (ldc < (m > 1 ? m : 1)) return -10;
  if (m == 0 || n == 0 || nq < 2) return 0;  // Q of order 0 or 1 is the identity
  cudaStream_t st = (cudaStream_t)stream;
  std::lock_guard<std::mutex> lk(g_q_mu);
  QCtx* q = nullptr;
  int rc = q_ctx((int)nq, &q);
  if (rc) return rc;
  const int nqi = (int)nq, mi = (int)m, ni = (int)n;
  const bool upper = uplo == 'U';
  // the lower-layout factors: A itself, or the reversed upper factors
  const double* F = A;
  long long ldf = lda;
  if (upper) {
    if (!q->frev) {  // set only on success, so a failed allocation is retried
      void* f = nullptr;
      Q_CUDA(cudaMalloc(&f, sizeof(double) * (size_t)nq * nq));
      q->frev = static_cast<double*>(f);
    }
    k_q_revfactors<<<dim3((nqi + 255) / 256, nqi), 256, 0, st>>>(A, lda, nqi, q->frev);
    Q_CUDA(cudaGetLastError());
    F = q->frev;
    ldf = nq;
  }
  if (side == 'L') {
    if (!upper) return large_ormtr(q->c, A, lda, tau, C, ldc, st, ni, trans == 'T');
    // op(Q_U) C = P op(Q_L) (P C)
    Q_CUDA(q_tmp(q, (size_t)nq * n, st));
    const dim3 g2((nqi + 255) / 256, grid_y(ni));
    k_q_revrows<<<g2, 256, 0, st>>>(C, ldc, nqi, ni, q->tmp, nq);
    Q_CUDA(cudaGetLastError());
    rc = large_ormtr(q->c, F, ldf, tau, q->tmp, nq, st, ni, trans == 'T');
    if (rc) return rc;
    k_q_revrows<<<g2, 256, 0, st>>>(q->tmp, nq, nqi, ni, C, ldc);
    Q_CUDA(cudaGetLastError());
    return 0;
  }
  // C op(Q) = (op(Q)' C')': transpose C (m x nq) into nq x m, apply op(Q)',
  // transpose back; for Q_U = P Q_L P the transposes also reverse the nq rows
  Q_CUDA(q_tmp(q, (size_t)nq * m, st));
  const dim3 tb(32, 8);
  k_q_transpose<<<dim3((unsigned)((m + 31) / 32), grid_y((nq + 31) / 32)), tb, 0, st>>>(C, ldc, mi, nqi, q->tmp, nq,
                                                                                       upper ? 1 : 0);
  Q_CUDA(cudaGetLastError());
  rc = large_ormtr(q->c, F, ldf, tau, q->tmp, nq, st, mi, trans == 'N');
  if (rc) return rc;
  k_q_transpose<<<dim3((unsigned)((nq + 31) / 32), grid_y((m + 31) / 32)), tb, 0, st>>>(q->tmp, nq, nqi, mi, C, ldc,
                                                                                        upper ? 2 : 0);
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

int gla_dormtr_host(char side, char uplo, char trans, int64_t m, int64_t n, const double* A, int64_t lda,
                    const double* tau, double* C, int64_t ldc) {
  if (side != 'L' && side != 'R') return -1;
  if (uplo != 'L' && uplo != 'U') return -2;
  if (trans != 'N' && trans != 'T') return -3;
  if (m < 0) return -4;
  if (n < 0) return -5;
  const int64_t nq = side == 'L' ? m : n;
  if (nq > GLA_MAX_N) return side == 'L' ? -4 : -5;
  if (!A && nq) return -6;
  if (lda < (nq > 1 ? nq : 1)) return -7;
  if (!tau && nq > 1) return -8;
  if (!C && m && n) return -9;
  if (ldc < (m > 1 ? m : 1)) return -10;
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
  int rc = err == cudaSuccess ? gla_dormtr(side, uplo, trans, m, n, dA, nq, dt, dC, m, nullptr) : -1000 - (int)err;
  if (rc == 0) {
    err = cudaMemcpy2D(C, sizeof(double) * ldc, dC, sizeof(double) * m, sizeof(double) * m, n, cudaMemcpyDeviceToHost);
    if (err != cudaSuccess) rc = -1000 - (int)err;
  }
  cudaFree(buf);
  return rc;
}

}  // extern "C"
