// Quaternion Hermitian input (the reference's eigen!/eigvals! on
// Hermitian{Quaternion{Float64}}, src/eigenSelfAdjoint.jl:620-630 with the
// non-real loop bound of :462; tested at test/eigenselfadjoint.jl:54-84)
// through the real symmetric matrix of left multiplication:
//
//   A = A0 + A1 i + A2 j + A3 k  ->  L(A) = [ A0 -A1 -A2 -A3 ]
//                                          [ A1  A0 -A3  A2 ]
//                                          [ A2  A3  A0 -A1 ]
//                                          [ A3 -A2  A1  A0 ]   (order 4n),
//
// block (r, c) = sign(r, c) A_{r xor c}, acting on v = x0 + x1 i + x2 j + x3 k
// stored as [x0; x1; x2; x3] (the Hamilton product row by row). L(AB) =
// L(A) L(B) and L(A^H) = L(A)', so L(A) is symmetric for Hermitian A, and a
// unit real eigenvector of L(A) is a unit quaternion eigenvector of A with
// the same (real) eigenvalue. Every eigenvalue of A appears four times in
// L(A): with A v = v lambda, the vectors v, v i, v j, v k are eigenvectors
// too and are orthogonal in the real inner product.
//
// L(A) is solved by this library's real FP64 path. Its sorted eigenvalues
// are grouped at gaps above 32 (4n) eps max|lambda|, in groups of 4k that
// hold k eigenvalues of A (the means of consecutive quadruples). A group of
// four gives the quaternion vector of its first real eigenvector; a larger
// group's 4k candidates span a k-dimensional (right) quaternion space, from
// which modified Gram-Schmidt with re-orthogonalisation keeps k orthonormal
// vectors. One symmetric Newton-Schulz step V <- V (I + R/2), R = I - V^H V,
// then squares the departure from orthogonality between groups (about
// u ||A|| / gap). It runs as two real FP64 GEMMs of order 4n on L(V):
// L(V)' [V0; V1; V2; V3] is the first block column [M0; M1; M2; M3] of
// L(V^H V), and L(V) [R0; R1; R2; R3] that of L(V R).
//
// The layout of a quaternion is 4 doubles (s, i, j, k), the field order of
// Julia's Quaternion{Float64}; matrices are column-major with the leading
// dimension counted in quaternions.
#include <cuda_runtime.h>
#include <stdint.h>

#include <algorithm>
#include <cmath>
#include <mutex>
#include <vector>

#include "../../include/glagpu.h"
#include "gla_large.h"

namespace {

#define Q_CUDA(x)                                   \
  do {                                              \
    cudaError_t e_ = (x);                           \
    if (e_ != cudaSuccess) return -1000 - (int)e_;  \
  } while (0)

// sign(r, c) of block (r, c) of L: bit (4 r + c) set means -1
constexpr unsigned kSignMask = (0xEu << 0) | (0x4u << 4) | (0x8u << 8) | (0x2u << 12);
__device__ __forceinline__ double lsign(int r, int c) { return (kSignMask >> (4 * r + c)) & 1u ? -1.0 : 1.0; }

// A quaternion s + x i + y j + z k in registers.
struct Quat {
  double s, x, y, z;
};
__device__ __forceinline__ Quat quat(double s, double x, double y, double z) {
  Quat q;
  q.s = s;
  q.x = x;
  q.y = y;
  q.z = z;
  return q;
}
// One Hamilton product p q.
__device__ __forceinline__ Quat hmul(Quat p, Quat q) {
  return quat(p.s * q.s - p.x * q.x - p.y * q.y - p.z * q.z, p.s * q.x + p.x * q.s + p.y * q.z - p.z * q.y,
              p.s * q.y - p.x * q.z + p.y * q.s + p.z * q.x, p.s * q.z + p.x * q.y - p.y * q.x + p.z * q.s);
}
__device__ __forceinline__ Quat hconj(Quat p) { return quat(p.s, -p.x, -p.y, -p.z); }
__device__ __forceinline__ Quat ld4(const double* p) { return quat(p[0], p[1], p[2], p[3]); }

// E = L(A) (4n x 4n, leading dimension 4n) from the referenced triangle of
// the quaternion matrix A (leading dimension lda quaternions).
__global__ void k_qembed(const double* __restrict__ A, long long lda, int n, int lower, double* __restrict__ E) {
  const int j = blockIdx.y;
  const long long n4 = 4LL * n;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const bool own = lower ? i >= j : i <= j;
    double a[4];
    if (own) {
      const double* p = A + 4 * (i + (long long)j * lda);
      a[0] = p[0];
      a[1] = p[1];
      a[2] = p[2];
      a[3] = p[3];
    } else {  // the Hermitian mirror: conj(A[j, i])
      const double* p = A + 4 * (j + (long long)i * lda);
      a[0] = p[0];
      a[1] = -p[1];
      a[2] = -p[2];
      a[3] = -p[3];
    }
    if (i == j) a[1] = a[2] = a[3] = 0.0;  // a Hermitian diagonal is real
#pragma unroll
    for (int r = 0; r < 4; r++)
#pragma unroll
      for (int c = 0; c < 4; c++) E[(r * n + i) + (long long)(c * n + j) * n4] = lsign(r, c) * a[r ^ c];
  }
}

// V[:, dst[c]] = the quaternion vector of the real eigenvector src[c] of E.
__global__ void k_qfour(const double* __restrict__ E, int n, const int* __restrict__ src, const int* __restrict__ dst,
                        double* __restrict__ V, long long ldv) {
  const int c = blockIdx.y;
  const long long s = src[c], d = dst[c], n4 = 4LL * n;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
#pragma unroll
    for (int m = 0; m < 4; m++) V[4 * (i + d * ldv) + m] = E[(m * n + i) + s * n4];
}

__device__ Quat block_sum4(Quat v, Quat* red) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    v.s += __shfl_xor_sync(0xffffffffu, v.s, o);
    v.x += __shfl_xor_sync(0xffffffffu, v.x, o);
    v.y += __shfl_xor_sync(0xffffffffu, v.y, o);
    v.z += __shfl_xor_sync(0xffffffffu, v.z, o);
  }
  __syncthreads();
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
  __syncthreads();
  Quat s = quat(0.0, 0.0, 0.0, 0.0);
  for (int w = 0; w < (int)(blockDim.x >> 5); w++) {
    s.s += red[w].s;
    s.x += red[w].x;
    s.y += red[w].y;
    s.z += red[w].z;
  }
  return s;
}

// One CTA per group of 4k real eigenvectors (columns g0 .. g0 + 4k - 1 of
// E): k orthonormal quaternion vectors into V[:, out0 .. out0 + k - 1] by
// modified Gram-Schmidt (two passes, r -= v (v^H r)) over the candidates in
// order. A first sweep keeps candidates whose residual norm exceeds 1/2.
// Were it to end short (it cannot for k < 4), a second sweep keeps those
// above 1/(2 sqrt k): the 4k candidates are an orthonormal basis of the
// group's space, so with j < k vectors kept their residuals' squares sum to
// 4 (k - j) and some candidate's residual is at least 1/sqrt k. Scratch: 4n
// doubles per CTA in r.
__global__ void __launch_bounds__(256) k_qgroup(const double* __restrict__ E, int n, const int* __restrict__ g0s,
                                                const int* __restrict__ ks, const int* __restrict__ outs,
                                                double* __restrict__ V, long long ldv, double* __restrict__ scratch) {
  __shared__ Quat red[8];
  __shared__ int kept_s;
  const int g = blockIdx.x, g0 = g0s[g], k = ks[g], out0 = outs[g];
  double* r = scratch + 4LL * n * g;
  const long long n4 = 4LL * n;
  if (threadIdx.x == 0) kept_s = 0;
  __syncthreads();
  for (int sweep = 0; sweep < 2; sweep++) {
    const double thr = sweep == 0 ? 0.5 : 0.5 / sqrt((double)k);
    for (int cand = 0; cand < 4 * k; cand++) {
      if (kept_s >= k) break;
      const long long s = g0 + cand;
      for (int i = threadIdx.x; i < n; i += blockDim.x)
#pragma unroll
        for (int m = 0; m < 4; m++) r[4 * i + m] = E[(m * n + i) + s * n4];
      __syncthreads();
      const int kept = kept_s;
      for (int pass = 0; pass < 2; pass++)
        for (int q = 0; q < kept; q++) {
          const double* vq = V + 4 * (out0 + q) * ldv;
          Quat h = quat(0.0, 0.0, 0.0, 0.0);  // vq^H r
          for (int i = threadIdx.x; i < n; i += blockDim.x) {
            const Quat t = hmul(hconj(ld4(vq + 4 * i)), ld4(r + 4 * i));
            h.s += t.s;
            h.x += t.x;
            h.y += t.y;
            h.z += t.z;
          }
          h = block_sum4(h, red);
          for (int i = threadIdx.x; i < n; i += blockDim.x) {
            const Quat t = hmul(ld4(vq + 4 * i), h);
            r[4 * i] -= t.s;
            r[4 * i + 1] -= t.x;
            r[4 * i + 2] -= t.y;
            r[4 * i + 3] -= t.z;
          }
          __syncthreads();
        }
      Quat nn = quat(0.0, 0.0, 0.0, 0.0);
      for (int i = threadIdx.x; i < n; i += blockDim.x)
#pragma unroll
        for (int m = 0; m < 4; m++) nn.s += r[4 * i + m] * r[4 * i + m];
      nn = block_sum4(nn, red);
      const double nrm = sqrt(nn.s);
      if (nrm > thr) {
        double* vo = V + 4 * (out0 + kept) * ldv;
        for (int i = threadIdx.x; i < 4 * n; i += blockDim.x) vo[i] = r[i] / nrm;
        __syncthreads();
        if (threadIdx.x == 0) kept_s = kept + 1;
      }
      __syncthreads();
    }
  }
}

// Cc (4n x n, leading dimension 4n) = [V0; V1; V2; V3], the components of V
__global__ void k_qsplit(const double* __restrict__ V, long long ldv, int n, double* __restrict__ Cc) {
  const int j = blockIdx.y;
  const long long n4 = 4LL * n;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
#pragma unroll
    for (int m = 0; m < 4; m++) Cc[(m * n + i) + j * n4] = V[4 * (i + j * ldv) + m];
}
__global__ void k_qmerge(const double* __restrict__ Cc, int n, double* __restrict__ V, long long ldv) {
  const int j = blockIdx.y;
  const long long n4 = 4LL * n;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
#pragma unroll
    for (int m = 0; m < 4; m++) V[4 * (i + j * ldv) + m] = Cc[(m * n + i) + j * n4];
}
// Lv = L(V) (4n x 4n) from its first block column Cc
__global__ void k_qlmat(const double* __restrict__ Cc, int n, double* __restrict__ Lv) {
  const int j = blockIdx.y;
  const long long n4 = 4LL * n;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    double a[4];
#pragma unroll
    for (int m = 0; m < 4; m++) a[m] = Cc[(m * n + i) + j * n4];
#pragma unroll
    for (int r = 0; r < 4; r++)
#pragma unroll
      for (int c = 0; c < 4; c++) Lv[(r * n + i) + (long long)(c * n + j) * n4] = lsign(r, c) * a[r ^ c];
  }
}
// G = [M0; M1; M2; M3] -> R = I - M in place
__global__ void k_qresid(int n, double* __restrict__ G) {
  const int j = blockIdx.y;
  const long long n4 = 4LL * n;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
#pragma unroll
    for (int m = 0; m < 4; m++) {
      const long long idx = (m * n + i) + j * n4;
      G[idx] = (m == 0 && i == j ? 1.0 : 0.0) - G[idx];
    }
}

// One Newton-Schulz step on V (n x n quaternions); W holds 28 n^2 doubles.
int q_orthonormalise(double* V, long long ldv, int n, double* W, cudaStream_t st) {
  const long long nn = (long long)n * n, n4 = 4LL * n;
  double *Lv = W, *Cc = W + 16 * nn, *G = W + 20 * nn, *Out = W + 24 * nn;
  const dim3 g2((n + 255) / 256, n);
  k_qsplit<<<g2, 256, 0, st>>>(V, ldv, n, Cc);
  Q_CUDA(cudaGetLastError());
  k_qlmat<<<g2, 256, 0, st>>>(Cc, n, Lv);
  Q_CUDA(cudaGetLastError());
  gla::GemmDesc g{};
  g.m = (int)n4;
  g.n = n;
  g.k = (int)n4;
  g.A = Lv;
  g.lda = n4;
  g.B = Cc;
  g.ldb = n4;
  g.C = G;
  g.ldc = n4;
  g.alpha = 1.0;
  g.beta = 0.0;
  Q_CUDA(gla::gemm_launch(true, true, false, false, g, 1, st));  // G = L(V)' Cc
  k_qresid<<<g2, 256, 0, st>>>(n, G);
  Q_CUDA(cudaGetLastError());
  Q_CUDA(cudaMemcpyAsync(Out, Cc, sizeof(double) * 4 * nn, cudaMemcpyDeviceToDevice, st));
  g.B = G;
  g.C = Out;
  g.alpha = 0.5;
  g.beta = 1.0;
  Q_CUDA(gla::gemm_launch(true, false, false, false, g, 1, st));  // Out = Cc + L(V) R / 2
  k_qmerge<<<g2, 256, 0, st>>>(Out, n, V, ldv);
  Q_CUDA(cudaGetLastError());
  return 0;
}

struct QWork {
  double* E = nullptr;
  double* w4 = nullptr;
  double* scratch = nullptr;
  int* idx = nullptr;
  size_t cap_E = 0, cap_w4 = 0, cap_scratch = 0, cap_idx = 0;
};
std::mutex g_qh_mu;
QWork g_qh;

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

int check_args(char jobz, char uplo, int64_t n, const double* A, int64_t lda, const double* w, const double* V,
               int64_t ldv, const int* info) {
  if (jobz != 'V' && jobz != 'N') return -1;
  if (uplo != 'L' && uplo != 'U') return -2;
  if (n < 0 || 4 * n > GLA_MAX_N) return -3;
  if (!A && n) return -4;
  if (lda < (n > 1 ? n : 1)) return -5;
  if (!w && n) return -6;
  if (jobz == 'V' && !V && n) return -7;
  if (jobz == 'V' && ldv < (n > 1 ? n : 1)) return -8;
  if (!info) return -9;
  return 0;
}

}  // namespace

namespace gla {
// Frees the buffers cached by gla_qheev (the caller has drained the device).
void release_quaternion_cache() {
  std::lock_guard<std::mutex> lk(g_qh_mu);
  cudaFree(g_qh.E);
  cudaFree(g_qh.w4);
  cudaFree(g_qh.scratch);
  cudaFree(g_qh.idx);
  g_qh = QWork();
}
}  // namespace gla

extern "C" {

int gla_qheev(char jobz, char uplo, int64_t n, const double* A, int64_t lda, double* w, double* V, int64_t ldv,
              int* info, void* stream) {
  const int bad = check_args(jobz, uplo, n, A, lda, w, V, ldv, info);
  if (bad) return bad;
  *info = 0;
  if (n == 0) return 0;
  cudaStream_t st = (cudaStream_t)stream;
  std::lock_guard<std::mutex> lk(g_qh_mu);
  const int nn = (int)n, n4 = 4 * nn;
  Q_CUDA(cudaStreamSynchronize(st));  // the buffers may be reallocated
  // L(A) (16 n^2), later the 28 n^2 work arrays of the orthonormalisation
  Q_CUDA(grow(&g_qh.E, &g_qh.cap_E, (size_t)(jobz == 'V' ? 28 : 16) * nn * nn));
  Q_CUDA(grow(&g_qh.w4, &g_qh.cap_w4, (size_t)n4));
  k_qembed<<<dim3((nn + 255) / 256, nn), 256, 0, st>>>(A, lda, nn, uplo == 'L', g_qh.E);
  Q_CUDA(cudaGetLastError());
  int inf4 = 0;
  int rc = gla_dsyev(jobz, 'L', n4, g_qh.E, n4, g_qh.w4, &inf4, stream);  // synchronizes
  if (rc < 0) return rc;
  if (inf4 != 0) {
    *info = inf4;
    return 1;
  }
  std::vector<double> h(n4);
  Q_CUDA(cudaMemcpy(h.data(), g_qh.w4, sizeof(double) * n4, cudaMemcpyDeviceToHost));
  double amax = 0.0;
  for (double x : h) amax = std::max(amax, std::fabs(x));
  const double tol = 32.0 * n4 * 0x1p-52 * std::max(amax, 1e-300);
  // groups of the sorted eigenvalues of L(A), closed at gaps above tol and
  // only at multiples of four
  std::vector<int> gs;  // group starts
  for (int i = 0; i < n4;) {
    int j = i + 1;
    while (j < n4 && (h[j] - h[j - 1] <= tol || (j - i) % 4 != 0)) j++;
    gs.push_back(i);
    i = j;
  }
  gs.push_back(n4);
  std::vector<double> hw(nn);
  std::vector<int> fsrc, fdst, g0s, ks, outs;
  int out = 0;
  for (size_t g = 0; g + 1 < gs.size(); g++) {
    const int a = gs[g], len = gs[g + 1] - gs[g], k = len / 4;
    for (int m = 0; m < k; m++) {
      const double* q = &h[a + 4 * m];
      hw[out + m] = 0.25 * ((q[0] + q[1]) + (q[2] + q[3]));
    }
    if (k == 1) {
      fsrc.push_back(a);
      fdst.push_back(out);
    } else {
      g0s.push_back(a);
      ks.push_back(k);
      outs.push_back(out);
    }
    out += k;
  }
  Q_CUDA(cudaMemcpyAsync(w, hw.data(), sizeof(double) * nn, cudaMemcpyHostToDevice, st));
  if (jobz == 'V') {
    std::vector<int> all;
    all.insert(all.end(), fsrc.begin(), fsrc.end());
    all.insert(all.end(), fdst.begin(), fdst.end());
    all.insert(all.end(), g0s.begin(), g0s.end());
    all.insert(all.end(), ks.begin(), ks.end());
    all.insert(all.end(), outs.begin(), outs.end());
    Q_CUDA(grow(&g_qh.idx, &g_qh.cap_idx, std::max<size_t>(all.size(), 1)));
    if (!all.empty())
      Q_CUDA(cudaMemcpyAsync(g_qh.idx, all.data(), sizeof(int) * all.size(), cudaMemcpyHostToDevice, st));
    const int nf = (int)fsrc.size(), ng = (int)g0s.size();
    if (nf) {
      k_qfour<<<dim3((nn + 255) / 256, nf), 256, 0, st>>>(g_qh.E, nn, g_qh.idx, g_qh.idx + nf, V, ldv);
      Q_CUDA(cudaGetLastError());
    }
    if (ng) {
      Q_CUDA(grow(&g_qh.scratch, &g_qh.cap_scratch, (size_t)4 * nn * ng));
      k_qgroup<<<ng, 256, 0, st>>>(g_qh.E, nn, g_qh.idx + 2 * nf, g_qh.idx + 2 * nf + ng, g_qh.idx + 2 * nf + 2 * ng,
                                   V, ldv, g_qh.scratch);
      Q_CUDA(cudaGetLastError());
    }
    // L(A)'s real eigenvectors are consumed (stream order); its buffer holds
    // the work arrays of the orthonormalisation step
    if (nn > 1) {
      const int rc2 = q_orthonormalise(V, ldv, nn, g_qh.E, st);
      if (rc2) return rc2;
    }
  }
  Q_CUDA(cudaStreamSynchronize(st));  // the index tables live in host memory until here
  return 0;
}

// Host-buffer form (stages through the device).
int gla_qheev_host(char jobz, char uplo, int64_t n, const double* A, int64_t lda, double* w, double* V, int64_t ldv,
                   int* info) {
  const int bad = check_args(jobz, uplo, n, A, lda, w, V, ldv, info);
  if (bad) return bad;
  *info = 0;
  if (n == 0) return 0;
  const size_t qn = 4 * (size_t)n * n;
  double* buf = nullptr;
  Q_CUDA(cudaMalloc((void**)&buf, sizeof(double) * (2 * qn + n)));
  double *dA = buf, *dV = buf + qn, *dw = buf + 2 * qn;
  cudaError_t err = cudaMemcpy2D(dA, 4 * sizeof(double) * n, A, 4 * sizeof(double) * lda, 4 * sizeof(double) * n, n,
                                 cudaMemcpyHostToDevice);
  int rc = err == cudaSuccess ? gla_qheev(jobz, uplo, n, dA, n, dw, dV, n, info, nullptr) : -1000 - (int)err;
  if (rc >= 0) {
    err = cudaMemcpy(w, dw, sizeof(double) * n, cudaMemcpyDeviceToHost);
    if (err == cudaSuccess && jobz == 'V')
      err = cudaMemcpy2D(V, 4 * sizeof(double) * ldv, dV, 4 * sizeof(double) * n, 4 * sizeof(double) * n, n,
                         cudaMemcpyDeviceToHost);
    if (err != cudaSuccess) rc = -1000 - (int)err;
  }
  cudaFree(buf);
  return rc;
}

}  // extern "C"
