// Complex Hermitian input (the reference's eigen!/eigvals! on
// Hermitian{<:Complex}, src/eigenSelfAdjoint.jl:620-630 with the complex
// loop bound of :462) through the real symmetric embedding
//
//   A = B + i C (B symmetric, C antisymmetric)  ->  E = [ B  -C ]
//                                                     [ C   B ]   (order 2n),
//
// whose eigenvalues are those of A, each twice, and whose eigenvectors [x; y]
// map to eigenvectors x + i y of A (a unit [x; y] gives a unit x + i y). E is
// solved by this library's real FP64 path. The sorted eigenvalues of E are
// grouped at gaps above 32 (2n) eps max|lambda|; a group of 2k values holds k
// eigenvalues of A (the means of consecutive pairs). Each group of two gives
// the complex vector of its first real eigenvector; a larger group's 2k
// complex candidates span a k-dimensional space (the candidates come in
// pairs u, i u), from which a modified Gram-Schmidt pass with re-
// orthogonalisation keeps k orthonormal vectors. The complex inner
// products of vectors from different groups carry the real subspaces'
// departure from invariance under [x; y] -> [-y; x], about u ||A|| / gap,
// so one symmetric Newton-Schulz step V <- V (I + R/2), R = I - V^H V, in
// real FP64 GEMMs on the real and imaginary parts, squares that defect (the
// residual moves by (lambda_a - lambda_b) r_ab / 2 ~ u ||A||).
//
// Costs: the real problem has order 2n (8 times the n^3 work of a real
// solve of order n, twice that of complex Householder arithmetic), in
// exchange for the real path's kernels unchanged.
#include <cuda_runtime.h>
#include <stdint.h>

#include <algorithm>
#include <cmath>
#include <mutex>
#include <vector>

#include "../../include/glagpu.h"
#include "gla_large.h"

namespace {

#define Z_CUDA(x)                                   \
  do {                                              \
    cudaError_t e_ = (x);                           \
    if (e_ != cudaSuccess) return -1000 - (int)e_;  \
  } while (0)

// E (2n x 2n, leading dimension 2n) from the referenced triangle of the
// complex matrix A (interleaved re, im; column-major, leading dimension lda).
__global__ void k_zembed(const double* __restrict__ A, long long lda, int n, int lower, double* __restrict__ E) {
  const int j = blockIdx.y;
  const long long n2 = 2LL * n;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    double re, im;
    const bool own = lower ? i >= j : i <= j;
    if (own) {
      re = A[2 * (i + (long long)j * lda)];
      im = A[2 * (i + (long long)j * lda) + 1];
    } else {  // the Hermitian mirror
      re = A[2 * (j + (long long)i * lda)];
      im = -A[2 * (j + (long long)i * lda) + 1];
    }
    if (i == j) im = 0.0;  // a Hermitian diagonal is real
    E[i + (long long)j * n2] = re;
    E[(i + n) + (long long)(j + n) * n2] = re;
    E[(i + n) + (long long)j * n2] = im;
    E[i + (long long)(j + n) * n2] = -im;
  }
}

// V[:, c] = x + i y for the real eigenvector src[c] = [x; y] of E.
__global__ void k_zpairs(const double* __restrict__ E, int n, const int* __restrict__ src, const int* __restrict__ dst,
                         double* __restrict__ V, long long ldv) {
  const int c = blockIdx.y;
  const long long s = src[c], d = dst[c];
  const long long n2 = 2LL * n;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    V[2 * (i + d * ldv)] = E[i + s * n2];
    V[2 * (i + d * ldv) + 1] = E[(i + n) + s * n2];
  }
}

__device__ double2 block_sum2(double2 v, double2* red) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    v.x += __shfl_xor_sync(0xffffffffu, v.x, o);
    v.y += __shfl_xor_sync(0xffffffffu, v.y, o);
  }
  __syncthreads();
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
  __syncthreads();
  double2 s = make_double2(0.0, 0.0);
  for (int w = 0; w < (int)(blockDim.x >> 5); w++) {
    s.x += red[w].x;
    s.y += red[w].y;
  }
  return s;
}

// One CTA per group of 2k real eigenvectors (columns g0 .. g0 + 2k - 1 of E):
// k orthonormal complex vectors into V[:, out0 .. out0 + k - 1] by modified
// Gram-Schmidt (two passes) over the candidates in order. A first sweep
// keeps candidates whose residual norm exceeds 1/2. Were it to end short (it
// cannot for k < 4), a second sweep keeps those above 1/(2 sqrt k): the 2k
// candidates are an orthonormal basis of the group's space, so with j < k
// vectors kept their residuals' squares sum to 2 (k - j) and some
// candidate's residual is at least 1/sqrt k. Scratch: n complex per CTA in r.
__global__ void __launch_bounds__(256) k_zgroup(const double* __restrict__ E, int n, const int* __restrict__ g0s,
                                                const int* __restrict__ ks, const int* __restrict__ outs,
                                                double* __restrict__ V, long long ldv, double* __restrict__ scratch) {
  __shared__ double2 red[8];
  __shared__ int kept_s;
  const int g = blockIdx.x, g0 = g0s[g], k = ks[g], out0 = outs[g];
  double* r = scratch + 2LL * n * g;
  const long long n2 = 2LL * n;
  if (threadIdx.x == 0) kept_s = 0;
  __syncthreads();
  for (int sweep = 0; sweep < 2; sweep++) {
    const double thr = sweep == 0 ? 0.5 : 0.5 / sqrt((double)k);
    for (int cand = 0; cand < 2 * k; cand++) {
      if (kept_s >= k) break;
      const long long s = g0 + cand;
      for (int i = threadIdx.x; i < n; i += blockDim.x) {
        r[2 * i] = E[i + s * n2];
        r[2 * i + 1] = E[(i + n) + s * n2];
      }
      __syncthreads();
      const int kept = kept_s;
      for (int pass = 0; pass < 2; pass++)
        for (int q = 0; q < kept; q++) {
          const double* vq = V + 2 * (out0 + q) * ldv;
          // h = vq^H r
          double2 h = make_double2(0.0, 0.0);
          for (int i = threadIdx.x; i < n; i += blockDim.x) {
            const double ar = vq[2 * i], ai = vq[2 * i + 1], br = r[2 * i], bi = r[2 * i + 1];
            h.x += ar * br + ai * bi;
            h.y += ar * bi - ai * br;
          }
          h = block_sum2(h, red);
          for (int i = threadIdx.x; i < n; i += blockDim.x) {
            const double ar = vq[2 * i], ai = vq[2 * i + 1];
            r[2 * i] -= h.x * ar - h.y * ai;
            r[2 * i + 1] -= h.x * ai + h.y * ar;
          }
          __syncthreads();
        }
      double2 nn = make_double2(0.0, 0.0);
      for (int i = threadIdx.x; i < n; i += blockDim.x) nn.x += r[2 * i] * r[2 * i] + r[2 * i + 1] * r[2 * i + 1];
      nn = block_sum2(nn, red);
      const double nrm = sqrt(nn.x);
      if (nrm > thr) {
        double* vo = V + 2 * (out0 + kept) * ldv;
        for (int i = threadIdx.x; i < n; i += blockDim.x) {
          vo[2 * i] = r[2 * i] / nrm;
          vo[2 * i + 1] = r[2 * i + 1] / nrm;
        }
        __syncthreads();
        if (threadIdx.x == 0) kept_s = kept + 1;
      }
      __syncthreads();
    }
  }
}

// X = re V, Y = im V (V interleaved, leading dimension ldv; X, Y n x n, ld n)
__global__ void k_zsplit(const double* __restrict__ V, long long ldv, int n, double* __restrict__ X,
                         double* __restrict__ Y) {
  const int j = blockIdx.y;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    X[i + (long long)j * n] = V[2 * (i + j * ldv)];
    Y[i + (long long)j * n] = V[2 * (i + j * ldv) + 1];
  }
}
__global__ void k_zmerge(const double* __restrict__ X, const double* __restrict__ Y, int n, double* __restrict__ V,
                         long long ldv) {
  const int j = blockIdx.y;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    V[2 * (i + j * ldv)] = X[i + (long long)j * n];
    V[2 * (i + j * ldv) + 1] = Y[i + (long long)j * n];
  }
}
// R = I - V^H V from P = re(V^H V), Q = im(V^H V): Rr = I - P, Ri = -Q (in place)
__global__ void k_zresid(int n, double* __restrict__ P, double* __restrict__ Q) {
  const int j = blockIdx.y;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const long long idx = i + (long long)j * n;
    P[idx] = (i == j ? 1.0 : 0.0) - P[idx];
    Q[idx] = -Q[idx];
  }
}

// One Newton-Schulz step on V (n x n complex, interleaved), with six n x n
// real work arrays in W.
int z_orthonormalise(double* V, long long ldv, int n, double* W, cudaStream_t st) {
  const long long nn = (long long)n * n;
  double *X = W, *Y = W + nn, *P = W + 2 * nn, *Q = W + 3 * nn, *X2 = W + 4 * nn, *Y2 = W + 5 * nn;
  const dim3 g2((n + 255) / 256, n);
  k_zsplit<<<g2, 256, 0, st>>>(V, ldv, n, X, Y);
  Z_CUDA(cudaGetLastError());
  auto gemm = [&](bool ta, const double* A, const double* B, double* C, double alpha, double beta) {
    gla::GemmDesc g{};
    g.m = g.n = g.k = n;
    g.A = A;
    g.lda = n;
    g.B = B;
    g.ldb = n;
    g.C = C;
    g.ldc = n;
    g.alpha = alpha;
    g.beta = beta;
    return gla::gemm_launch(true, ta, false, false, g, 1, st);
  };
  // V^H V = (X'X + Y'Y) + i (X'Y - Y'X)
  Z_CUDA(gemm(true, X, X, P, 1.0, 0.0));
  Z_CUDA(gemm(true, Y, Y, P, 1.0, 1.0));
  Z_CUDA(gemm(true, X, Y, Q, 1.0, 0.0));
  Z_CUDA(gemm(true, Y, X, Q, -1.0, 1.0));
  k_zresid<<<g2, 256, 0, st>>>(n, P, Q);
  Z_CUDA(cudaGetLastError());
  // V (I + R/2): X2 = X + (X Rr - Y Ri)/2, Y2 = Y + (X Ri + Y Rr)/2
  Z_CUDA(cudaMemcpyAsync(X2, X, sizeof(double) * nn, cudaMemcpyDeviceToDevice, st));
  Z_CUDA(cudaMemcpyAsync(Y2, Y, sizeof(double) * nn, cudaMemcpyDeviceToDevice, st));
  Z_CUDA(gemm(false, X, P, X2, 0.5, 1.0));
  Z_CUDA(gemm(false, Y, Q, X2, -0.5, 1.0));
  Z_CUDA(gemm(false, X, Q, Y2, 0.5, 1.0));
  Z_CUDA(gemm(false, Y, P, Y2, 0.5, 1.0));
  k_zmerge<<<g2, 256, 0, st>>>(X2, Y2, n, V, ldv);
  Z_CUDA(cudaGetLastError());
  return 0;
}

struct ZWork {
  double* E = nullptr;
  double* w2 = nullptr;
  double* scratch = nullptr;
  int* idx = nullptr;
  size_t cap_E = 0, cap_w2 = 0, cap_scratch = 0, cap_idx = 0;
};
std::mutex g_z_mu;
ZWork g_z;

template <class P>
cudaError_t grow(P** p, size_t* cap, size_t need) {
  if (*cap >= need) return cudaSuccess;
  cudaFree(*p);
  *p = nullptr;
  *cap = 0;
  cudaError_t e = cudaMalloc((void**)p, sizeof(P) * need);
  if (e == cudaSuccess) *cap = need;
  return e;
}

}  // namespace

namespace gla {
// Frees the buffers cached by gla_zheev (the caller has drained the device).
void release_complex_cache() {
  std::lock_guard<std::mutex> lk(g_z_mu);
  cudaFree(g_z.E);
  cudaFree(g_z.w2);
  cudaFree(g_z.scratch);
  cudaFree(g_z.idx);
  g_z = ZWork();
}
}  // namespace gla

extern "C" {

int gla_zheev(char jobz, char uplo, int64_t n, const double* A, int64_t lda, double* w, double* V, int64_t ldv,
              int* info, void* stream) {
  if (jobz != 'V' && jobz != 'N') return -1;
  if (uplo != 'L' && uplo != 'U') return -2;
  if (n < 0 || 2 * n > GLA_MAX_N) return -3;
  if (!A && n) return -4;
  if (lda < (n > 1 ? n : 1)) return -5;
  if (!w && n) return -6;
  if (jobz == 'V' && !V && n) return -7;
  if (jobz == 'V' && ldv < (n > 1 ? n : 1)) return -8;
  if (!info) return -9;
  *info = 0;
  if (n == 0) return 0;
  cudaStream_t st = (cudaStream_t)stream;
  std::lock_guard<std::mutex> lk(g_z_mu);
  const int nn = (int)n, n2 = 2 * nn;
  Z_CUDA(cudaStreamSynchronize(st));  // the buffers may be reallocated
  Z_CUDA(grow(&g_z.E, &g_z.cap_E, (size_t)6 * nn * nn));  // E (4 n^2), later the 6 n^2 work arrays
  Z_CUDA(grow(&g_z.w2, &g_z.cap_w2, (size_t)n2));
  k_zembed<<<dim3((nn + 255) / 256, nn), 256, 0, st>>>(A, lda, nn, uplo == 'L', g_z.E);
  Z_CUDA(cudaGetLastError());
  int inf2 = 0;
  int rc = gla_dsyev(jobz, 'L', n2, g_z.E, n2, g_z.w2, &inf2, stream);  // synchronizes
  if (rc < 0) return rc;
  if (inf2 != 0) {
    *info = inf2;
    return 1;
  }
  std::vector<double> h(n2);
  Z_CUDA(cudaMemcpy(h.data(), g_z.w2, sizeof(double) * n2, cudaMemcpyDeviceToHost));
  double amax = 0.0;
  for (double x : h) amax = std::max(amax, std::fabs(x));
  const double tol = 32.0 * n2 * 0x1p-52 * std::max(amax, 1e-300);
  // groups of the sorted eigenvalues of E; odd groups (pairs split by more
  // than tol) are merged with their successor
  std::vector<int> gs;  // group starts
  for (int i = 0; i < n2;) {
    int j = i + 1;
    while (j < n2 && (h[j] - h[j - 1] <= tol || (j - i) % 2 == 1)) j++;
    gs.push_back(i);
    i = j;
  }
  gs.push_back(n2);
  std::vector<double> hw(nn);
  std::vector<int> psrc, pdst, g0s, ks, outs;
  int out = 0;
  for (size_t g = 0; g + 1 < gs.size(); g++) {
    const int a = gs[g], len = gs[g + 1] - gs[g], k = len / 2;
    for (int m = 0; m < k; m++) hw[out + m] = 0.5 * (h[a + 2 * m] + h[a + 2 * m + 1]);
    if (k == 1) {
      psrc.push_back(a);
      pdst.push_back(out);
    } else {
      g0s.push_back(a);
      ks.push_back(k);
      outs.push_back(out);
    }
    out += k;
  }
  Z_CUDA(cudaMemcpyAsync(w, hw.data(), sizeof(double) * nn, cudaMemcpyHostToDevice, st));
  if (jobz == 'V') {
    const size_t nidx = psrc.size() * 2 + g0s.size() * 3;
    Z_CUDA(grow(&g_z.idx, &g_z.cap_idx, std::max<size_t>(nidx, 1)));
    std::vector<int> all;
    all.insert(all.end(), psrc.begin(), psrc.end());
    all.insert(all.end(), pdst.begin(), pdst.end());
    all.insert(all.end(), g0s.begin(), g0s.end());
    all.insert(all.end(), ks.begin(), ks.end());
    all.insert(all.end(), outs.begin(), outs.end());
    if (!all.empty()) Z_CUDA(cudaMemcpyAsync(g_z.idx, all.data(), sizeof(int) * all.size(), cudaMemcpyHostToDevice, st));
    const int np = (int)psrc.size(), ng = (int)g0s.size();
    if (np)
      k_zpairs<<<dim3((nn + 255) / 256, np), 256, 0, st>>>(g_z.E, nn, g_z.idx, g_z.idx + np, V, ldv);
    Z_CUDA(cudaGetLastError());
    if (ng) {
      Z_CUDA(grow(&g_z.scratch, &g_z.cap_scratch, (size_t)2 * nn * ng));
      k_zgroup<<<ng, 256, 0, st>>>(g_z.E, nn, g_z.idx + 2 * np, g_z.idx + 2 * np + ng, g_z.idx + 2 * np + 2 * ng, V,
                                   ldv, g_z.scratch);
      Z_CUDA(cudaGetLastError());
    }
    // E's real eigenvectors are consumed (stream order); its 6 n^2 doubles
    // hold the work arrays of the orthonormalisation step
    if (nn > 1) {
      int rc2 = z_orthonormalise(V, ldv, nn, g_z.E, st);
      if (rc2) return rc2;
    }
  }
  Z_CUDA(cudaStreamSynchronize(st));  // the index tables live in host memory until here
  return 0;
}

// Host-buffer form (stages through the device).
int gla_zheev_host(char jobz, char uplo, int64_t n, const double* A, int64_t lda, double* w, double* V, int64_t ldv,
                   int* info) {
  if (jobz != 'V' && jobz != 'N') return -1;
  if (uplo != 'L' && uplo != 'U') return -2;
  if (n < 0 || 2 * n > GLA_MAX_N) return -3;
  if (!A && n) return -4;
  if (lda < (n > 1 ? n : 1)) return -5;
  if (!w && n) return -6;
  if (jobz == 'V' && !V && n) return -7;
  if (jobz == 'V' && ldv < (n > 1 ? n : 1)) return -8;
  if (!info) return -9;
  *info = 0;
  if (n == 0) return 0;
  const size_t cn = 2 * (size_t)n * n;
  double* buf = nullptr;
  Z_CUDA(cudaMalloc((void**)&buf, sizeof(double) * (2 * cn + n)));
  double *dA = buf, *dV = buf + cn, *dw = buf + 2 * cn;
  cudaError_t err = cudaMemcpy2D(dA, 2 * sizeof(double) * n, A, 2 * sizeof(double) * lda, 2 * sizeof(double) * n, n,
                                 cudaMemcpyHostToDevice);
  int rc = err == cudaSuccess ? gla_zheev(jobz, uplo, n, dA, n, dw, dV, n, info, nullptr) : -1000 - (int)err;
  if (rc >= 0) {
    err = cudaMemcpy(w, dw, sizeof(double) * n, cudaMemcpyDeviceToHost);
    if (err == cudaSuccess && jobz == 'V')
      err = cudaMemcpy2D(V, 2 * sizeof(double) * ldv, dV, 2 * sizeof(double) * n, 2 * sizeof(double) * n, n,
                         cudaMemcpyDeviceToHost);
    if (err != cudaSuccess) rc = -1000 - (int)err;
  }
  cudaFree(buf);
  return rc;
}

}  // extern "C"
