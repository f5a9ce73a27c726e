// Driver of the large-matrix path (orders above the small-matrix limit):
//   load  : the used triangle of A into a lower-stored working copy in the
//           working precision, scaled by an exact power of two so that its
//           largest entry lies in [1, 2) (no overflow in the Householder
//           norms, bit-exact unscaling of the eigenvalues); non-finite input
//           gives info = -1
//   sytrd : blocked Householder tridiagonalisation (large_sytrd.cu)
//   stedc : divide and conquer on (d, e) (large_dc.cu)
//   ormtr : Z := Q Z with compact-WY blocks (large_backtr.cu)
//   store : eigenvalues unscaled, eigenvectors copied out
// The sequence synchronises with the host once at the end (and inside the
// leaf solves) to collect the status words.
#include <cuda_runtime.h>

#include <algorithm>
#include <new>
#include <vector>

#include "gla_common.cuh"
#include "gla_large.h"
#include "gla_launch.h"

namespace gla {

struct LargeCtx {
  int n = 0;
  bool f64 = true;
  SytrdPlan* sy = nullptr;
  DcPlan* dc = nullptr;
  BacktrPlan* bt = nullptr;
  void* Aw = nullptr;   // working copy, n x n, leading dimension n
  void* Z = nullptr;    // eigenvectors, n x n
  void* d = nullptr;
  void* e = nullptr;
  void* tau = nullptr;
  int* flags = nullptr; // [0] max |a| bits (low word), [1] high word, [2] non-finite, [3] scale exponent
  int* leaf_info = nullptr;
  int* h_stat = nullptr;  // pinned status words
  cudaEvent_t ev[4] = {};  // stage boundaries: load+sytrd | stedc | ormtr+store
  float ms[3] = {0, 0, 0}; // last solve: tridiagonalisation, divide and conquer, back-transformation
};

namespace {

template <class Tin>
GLA_DEV unsigned long long abs_bits(Tin x);
template <>
GLA_DEV unsigned long long abs_bits<double>(double x) {
  return (unsigned long long)__double_as_longlong(fabs(x));
}
template <>
GLA_DEV unsigned long long abs_bits<float>(float x) {
  return (unsigned long long)__double_as_longlong((double)fabsf(x));
}

// max |a_ij| over the used triangle (as the bits of a non-negative double,
// which order like the values) and a non-finite flag.
template <class Tin>
__global__ void k_large_maxabs(const Tin* __restrict__ A, long long lda, int n, bool lower,
                               unsigned long long* amax, int* nonfinite) {
  unsigned long long m = 0;
  int bad = 0;
  const int j = blockIdx.y;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    if (lower ? i < j : i > j) continue;
    const Tin x = A[i + (long long)j * lda];
    if (!isfinite(x)) bad = 1;
    else m = max(m, abs_bits<Tin>(x));
  }
#pragma unroll
  for (int s = 16; s > 0; s >>= 1) {
    m = max(m, __shfl_xor_sync(0xffffffffu, m, s));
    bad |= __shfl_xor_sync(0xffffffffu, bad, s);
  }
  if ((threadIdx.x & 31) == 0) {
    if (m) atomicMax(amax, m);
    if (bad) atomicExch(nonfinite, 1);
  }
}

// Working copy: Aw[i, j] (i >= j) = A[i, j] (lower) or A[j, i] (upper),
// times 2^-e; zeros above the diagonal. Non-finite input: zeros.
template <class Tin, class T>
__global__ void k_large_load(const Tin* __restrict__ A, long long lda, int n, bool lower, T* __restrict__ Aw,
                             const unsigned long long* __restrict__ amax, const int* __restrict__ nonfinite,
                             int* __restrict__ scale_exp) {
  const double am = __longlong_as_double((long long)*amax);
  const int ex = (am > 0.0 && !*nonfinite) ? ilogb(am) : 0;
  const double sc = ldexp(1.0, -ex);
  if (blockIdx.x == 0 && blockIdx.y == 0 && threadIdx.x == 0) *scale_exp = ex;
  const bool bad = *nonfinite != 0;
  const int j = blockIdx.y;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    T v = T(0);
    if (i >= j && !bad) {
      const Tin x = lower ? A[i + (long long)j * lda] : A[j + (long long)i * lda];
      v = (T)((double)x * sc);
    }
    Aw[i + (long long)j * n] = v;
  }
}

// Eigenvalues unscaled (NaN for non-finite input), eigenvectors copied out.
template <class T, class Tout>
__global__ void k_large_store(const T* __restrict__ d, const T* __restrict__ Z, int n, Tout* __restrict__ w,
                              Tout* __restrict__ V, long long ldv, const int* __restrict__ nonfinite,
                              const int* __restrict__ scale_exp) {
  const bool bad = *nonfinite != 0;
  const int j = blockIdx.y;
  const double sc = ldexp(1.0, *scale_exp);
  if (blockIdx.x == 0 && threadIdx.x == 0) w[j] = bad ? (Tout)NAN : (Tout)((double)d[j] * sc);
  if (!V) return;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    V[i + (long long)j * ldv] = bad ? (Tout)NAN : (Tout)Z[i + (long long)j * n];
}

#define LG_CUDA(x)                                         \
  do {                                                     \
    cudaError_t e_ = (x);                                  \
    if (e_ != cudaSuccess) return -1000 - (int)e_;         \
  } while (0)

}  // namespace

int large_create(LargeCtx** out, int n, bool f64, bool refine_stage) {
  *out = nullptr;
  LargeCtx* c = new (std::nothrow) LargeCtx();
  if (!c) return -1000 - (int)cudaErrorMemoryAllocation;
  c->n = n;
  c->f64 = f64;
  const size_t el = f64 ? 8 : 4;
  cudaError_t err = sytrd_plan_create(&c->sy, n, f64, !f64 && refine_stage);
  int rc = err == cudaSuccess ? 0 : -1000 - (int)err;
  if (!rc) rc = dc_plan_create(&c->dc, n, f64, refine_stage);
  if (!rc) rc = backtr_plan_create(&c->bt, n, f64, !f64 && refine_stage);
  if (!rc) backtr_set_error_word(c->bt, sytrd_error_word(c->sy));
  auto alloc = [&](void** p, size_t bytes) {
    if (!rc) {
      cudaError_t e2 = cudaMalloc(p, std::max<size_t>(bytes, 16));
      if (e2 != cudaSuccess) rc = -1000 - (int)e2;
    }
  };
  alloc(&c->Aw, el * (size_t)n * n);
  alloc(&c->Z, el * (size_t)n * n);
  alloc(&c->d, el * n);
  alloc(&c->e, el * n);
  alloc(&c->tau, el * n);
  alloc((void**)&c->flags, 4 * sizeof(int));
  if (!rc) alloc((void**)&c->leaf_info, sizeof(int) * dc_leaf_count(c->dc));
  if (!rc) {
    cudaError_t e2 = cudaMallocHost((void**)&c->h_stat, 4 * sizeof(int));
    for (int i = 0; i < 4 && e2 == cudaSuccess; i++) e2 = cudaEventCreate(&c->ev[i]);
    if (e2 != cudaSuccess) rc = -1000 - (int)e2;
  }
  if (rc) {
    large_destroy(c);
    return rc;
  }
  *out = c;
  return 0;
}

void large_destroy(LargeCtx* c) {
  if (!c) return;
  sytrd_plan_destroy(c->sy);
  dc_plan_destroy(c->dc);
  backtr_plan_destroy(c->bt);
  cudaFree(c->Aw);
  cudaFree(c->Z);
  cudaFree(c->d);
  cudaFree(c->e);
  cudaFree(c->tau);
  cudaFree(c->flags);
  cudaFree(c->leaf_info);
  cudaFreeHost(c->h_stat);
  for (int i = 0; i < 4; i++)
    if (c->ev[i]) cudaEventDestroy(c->ev[i]);
  delete c;
}

void* large_work_matrix(LargeCtx* c) { return c->Aw; }

void large_stage_ms(const LargeCtx* c, float* ms3) {
  for (int i = 0; i < 3; i++) ms3[i] = c->ms[i];
}

size_t large_workspace_bytes(const LargeCtx* c) {
  const size_t el = c->f64 ? 8 : 4;
  return el * (size_t)c->n * c->n * 4 + dc_plan_bytes(c->dc);
}

int large_sytrd(LargeCtx* c, void* A, long long lda, void* d, void* e, void* tau, cudaStream_t st) {
  LG_CUDA(sytrd_enqueue(c->sy, A, lda, d, e, tau, st));
  return 0;
}

int large_stedc(LargeCtx* c, void* d, const void* e, void* Z, long long ldz, int* info, cudaStream_t st) {
  (void)ldz;
  return dc_enqueue(c->dc, d, e, Z, info, st);
}

int large_ormtr(LargeCtx* c, const void* A, long long lda, const void* tau, void* Z, long long ldz, cudaStream_t st,
                int ncol, bool trans) {
  return backtr_enqueue(c->bt, A, lda, tau, Z, ldz, st, ncol, trans);
}

int large_syev(LargeCtx* c, int tcode, bool wantv, bool lower, const void* Ain, long long lda, void* w, void* V,
               long long ldv, int* info_host, cudaStream_t st) {
  const int n = c->n;
  unsigned long long* amax = reinterpret_cast<unsigned long long*>(c->flags);
  int* nonfinite = c->flags + 2;
  int* sexp = c->flags + 3;
  LG_CUDA(cudaEventRecord(c->ev[0], st));
  LG_CUDA(cudaMemsetAsync(c->flags, 0, 4 * sizeof(int), st));
  const dim3 g2((n + 255) / 256, n);
  const bool in64 = tcode != kF32;
  if (in64)
    k_large_maxabs<double><<<g2, 256, 0, st>>>((const double*)Ain, lda, n, lower, amax, nonfinite);
  else
    k_large_maxabs<float><<<g2, 256, 0, st>>>((const float*)Ain, lda, n, lower, amax, nonfinite);
  LG_CUDA(cudaGetLastError());
  if (c->f64)
    k_large_load<double, double><<<g2, 256, 0, st>>>((const double*)Ain, lda, n, lower, (double*)c->Aw, amax,
                                                     nonfinite, sexp);
  else if (in64)
    k_large_load<double, float><<<g2, 256, 0, st>>>((const double*)Ain, lda, n, lower, (float*)c->Aw, amax,
                                                    nonfinite, sexp);
  else
    k_large_load<float, float><<<g2, 256, 0, st>>>((const float*)Ain, lda, n, lower, (float*)c->Aw, amax,
                                                   nonfinite, sexp);
  LG_CUDA(cudaGetLastError());
  int rc = large_sytrd(c, c->Aw, n, c->d, c->e, c->tau, st);
  if (rc) return rc;
  LG_CUDA(cudaEventRecord(c->ev[1], st));
  rc = large_stedc(c, c->d, c->e, c->Z, n, c->leaf_info, st);
  if (rc) return rc;
  LG_CUDA(cudaEventRecord(c->ev[2], st));
  if (wantv) {
    rc = large_ormtr(c, c->Aw, n, c->tau, c->Z, n, st);
    if (rc) return rc;
  }
  const dim3 gs((n + 255) / 256, n);
  if (c->f64)
    k_large_store<double, double><<<gs, 256, 0, st>>>((const double*)c->d, (const double*)c->Z, n, (double*)w,
                                                      wantv ? (double*)V : nullptr, ldv, nonfinite, sexp);
  else
    k_large_store<float, float><<<gs, 256, 0, st>>>((const float*)c->d, (const float*)c->Z, n, (float*)w,
                                                    wantv ? (float*)V : nullptr, ldv, nonfinite, sexp);
  LG_CUDA(cudaGetLastError());
  LG_CUDA(cudaEventRecord(c->ev[3], st));
  // status: barrier timeout, secular non-convergence, leaf non-convergence, non-finite input
  LG_CUDA(cudaMemcpyAsync(c->h_stat, sytrd_error_word(c->sy), sizeof(int), cudaMemcpyDeviceToHost, st));
  LG_CUDA(cudaMemcpyAsync(c->h_stat + 1, dc_fail_word(c->dc), sizeof(int), cudaMemcpyDeviceToHost, st));
  LG_CUDA(cudaMemcpyAsync(c->h_stat + 2, nonfinite, sizeof(int), cudaMemcpyDeviceToHost, st));
  const int nleaf = dc_leaf_count(c->dc);
  std::vector<int> li(nleaf);
  LG_CUDA(cudaMemcpyAsync(li.data(), c->leaf_info, sizeof(int) * nleaf, cudaMemcpyDeviceToHost, st));
  LG_CUDA(cudaStreamSynchronize(st));
  for (int i = 0; i < 3; i++) cudaEventElapsedTime(&c->ms[i], c->ev[i], c->ev[i + 1]);
  if (c->h_stat[0]) return -1000 - (int)cudaErrorLaunchTimeout;
  int inf = 0;
  if (c->h_stat[2])
    inf = -1;
  else {
    int bad = c->h_stat[1] ? 1 : 0;
    for (int x : li) bad += x > 0 ? x : 0;
    inf = bad;
  }
  *info_host = inf;
  return 0;
}

// SymTridiagonal input (the reference's eigen!(::SymTridiagonal),
// src/eigenSelfAdjoint.jl:602-612): divide and conquer on (d, e) as given
// (FP64 context), eigenvalues ascending into w, eigenvectors into Z (ldz)
// when wanted. Synchronises st.
int large_stev(LargeCtx* c, const double* d, const double* e, double* w, double* Z, long long ldz, int* info_host,
               cudaStream_t st) {
  const int n = c->n;
  if (!c->f64) return -1000 - (int)cudaErrorInvalidValue;
  LG_CUDA(cudaMemcpyAsync(c->d, d, sizeof(double) * n, cudaMemcpyDeviceToDevice, st));
  LG_CUDA(cudaMemsetAsync(c->e, 0, sizeof(double) * n, st));
  if (n > 1) LG_CUDA(cudaMemcpyAsync(c->e, e, sizeof(double) * (n - 1), cudaMemcpyDeviceToDevice, st));
  int rc = dc_enqueue(c->dc, c->d, c->e, c->Z, c->leaf_info, st);
  if (rc) return rc;
  LG_CUDA(cudaMemcpyAsync(w, c->d, sizeof(double) * n, cudaMemcpyDeviceToDevice, st));
  if (Z)
    LG_CUDA(cudaMemcpy2DAsync(Z, sizeof(double) * ldz, c->Z, sizeof(double) * n, sizeof(double) * n, n,
                              cudaMemcpyDeviceToDevice, st));
  LG_CUDA(cudaMemcpyAsync(c->h_stat + 1, dc_fail_word(c->dc), sizeof(int), cudaMemcpyDeviceToHost, st));
  const int nleaf = dc_leaf_count(c->dc);
  std::vector<int> li(nleaf);
  LG_CUDA(cudaMemcpyAsync(li.data(), c->leaf_info, sizeof(int) * nleaf, cudaMemcpyDeviceToHost, st));
  LG_CUDA(cudaStreamSynchronize(st));
  int bad = c->h_stat[1] ? 1 : 0;
  bool nonfinite = false;
  for (int x : li) {
    if (x < 0) nonfinite = true;
    if (x > 0) bad += x;
  }
  *info_host = nonfinite ? -1 : bad;
  return 0;
}

}  // namespace gla
