// Back-transformation Z := Q Z for the large path, Q = H_0 H_1 ... H_{n-2}
// from large_sytrd (the reference forms Array(Q) with lmul!(::EigenQ),
// src/eigenSelfAdjoint.jl:23-60,101, one reflector at a time). Here the
// reflectors are grouped in blocks of kBacktrNB into compact-WY factors
// H_j0 ... H_j1 = I - Y T Y' (T upper triangular, the LAPACK dlarft
// "forward, columnwise" form) and applied from the last block to the first:
//   W  = Y' Z        (split-K GEMM: Y has few columns, Z many rows)
//   W2 = T W
//   Z -= Y W2        (GEMM)
// All T factors are formed up front, one CTA per block.
#include <cuda_runtime.h>

#include <algorithm>

#include "gla_common.cuh"
#include "gla_large.h"
#include "tc_gemm.cuh"

namespace gla {

constexpr int kBT = kBacktrNB;

// Y (n x n): column j is reflector j with its unit element and zeros above.
// Y (and, when Yt is given, its transpose: the K-major operand of the
// tensor-core Z -= Y W2) from the reflectors stored below the subdiagonal.
template <class T>
__global__ void k_form_y(const T* __restrict__ A, long long lda, T* __restrict__ Y, int n, T* __restrict__ Yt) {
  const int j = blockIdx.y;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    T v;
    if (j >= n - 1 || i <= j)
      v = T(0);
    else if (i == j + 1)
      v = T(1);
    else
      v = A[i + (long long)j * lda];
    Y[i + (long long)j * n] = v;
    if (Yt) Yt[j + (long long)i * n] = v;
  }
}

// One CTA per block: G = Y_b' Y_b, then T (kb x kb, leading dimension kBT):
// T[i][i] = tau_i, T[0:i, i] = -tau_i T[0:i, 0:i] G[0:i, i]. Dynamic shared
// memory: G (kBT x kBT+1), then the staging tile of Y rows, later reused
// for T.
template <class T>
size_t larft_smem_bytes() {
  return sizeof(T) * (size_t)(2 * kBT * (kBT + 1));
}

template <class T>
__global__ void __launch_bounds__(256) k_larft(const T* __restrict__ Y, const T* __restrict__ tau, T* __restrict__ Tm,
                                               int n) {
  const int b = blockIdx.x, j0 = b * kBT, kb = min(kBT, n - 1 - j0);
  extern __shared__ __align__(16) unsigned char larft_sm[];
  T(*G)[kBT + 1] = reinterpret_cast<T(*)[kBT + 1]>(larft_sm);
  T(*Ys)[kBT + 1] = reinterpret_cast<T(*)[kBT + 1]>(larft_sm + sizeof(T) * kBT * (kBT + 1));
  T(*Ts)[kBT + 1] = Ys;
  const int tid = threadIdx.x;
  T acc[16];
#pragma unroll
  for (int q = 0; q < 16; q++) acc[q] = T(0);
  // thread owns entries (r, c) = (tid % 64, tid / 64 + 4 q) of the 64 x 64 Gram matrix
  const int r = tid % kBT, cb = tid / kBT;
  for (int i0 = j0 + 1; i0 < n; i0 += 32) {
    __syncthreads();
    for (int idx = tid; idx < 32 * kBT; idx += 256) {
      const int ii = idx % 32, c = idx / 32;
      const int i = i0 + ii;
      Ys[ii][c] = (i < n && c < kb) ? Y[i + (long long)(j0 + c) * n] : T(0);
    }
    __syncthreads();
#pragma unroll 4
    for (int ii = 0; ii < 32; ii++) {
      const T yr = Ys[ii][r];
#pragma unroll
      for (int q = 0; q < 16; q++) acc[q] = fma(yr, Ys[ii][cb + 4 * q], acc[q]);
    }
  }
#pragma unroll
  for (int q = 0; q < 16; q++) G[r][cb + 4 * q] = acc[q];
  __syncthreads();
  T* Tb = Tm + (long long)b * kBT * kBT;
  for (int idx = tid; idx < kBT * kBT; idx += 256) Ts[idx % kBT][idx / kBT] = T(0);
  __syncthreads();
  for (int i = 0; i < kb; i++) {  // the recurrence is sequential in i
    const T ti = tau[j0 + i];
    if (tid < i) {
      T s = T(0);
      for (int q = tid; q < i; q++) s = fma(Ts[tid][q], G[q][i], s);
      Ts[tid][i] = -ti * s;
    }
    if (tid == 0) Ts[i][i] = ti;
    __syncthreads();
  }
  for (int idx = tid; idx < kBT * kBT; idx += 256) Tb[idx] = Ts[idx % kBT][idx / kBT];
}

// W2 = op(T) * sum_s Wpart_s   (W is kb x ncol, partials of leading dimension
// kb; op(T) = T, or T' when trans)
template <class T>
__global__ void __launch_bounds__(256) k_tw(const T* __restrict__ Wp, int splits, long long pstride,
                                            const T* __restrict__ Tb, T* __restrict__ W2, int kb, int ncol,
                                            int trans) {
  constexpr int kC = 16;  // columns per CTA
  __shared__ T Ts[kBT][kBT + 1];
  __shared__ T ws[kBT][kC + 1];
  for (int idx = threadIdx.x; idx < kBT * kBT; idx += 256) Ts[idx % kBT][idx / kBT] = Tb[idx];
  const int c0 = blockIdx.x * kC;
  for (int idx = threadIdx.x; idx < kBT * kC; idx += 256) {
    const int i = idx % kBT, c = idx / kBT;
    T s = T(0);
    if (i < kb && c0 + c < ncol)
      for (int sp = 0; sp < splits; sp++) s += Wp[sp * pstride + i + (long long)(c0 + c) * kb];
    ws[i][c] = s;
  }
  __syncthreads();
  for (int idx = threadIdx.x; idx < kBT * kC; idx += 256) {
    const int i = idx % kBT, c = idx / kBT;
    if (i >= kb || c0 + c >= ncol) continue;
    T s = T(0);
    if (trans)
      for (int q = 0; q <= i; q++) s = fma(Ts[q][i], ws[q][c], s);
    else
      for (int q = i; q < kb; q++) s = fma(Ts[i][q], ws[q][c], s);
    W2[i + (long long)(c0 + c) * kBT] = s;
  }
}

struct BacktrPlan {
  int n = 0;
  bool f64 = true;
  int nblk = 0;
  int splits = 1;
  void* Y = nullptr;
  void* Tm = nullptr;
  void* Wp = nullptr;
  void* W2 = nullptr;   // T W, kBT x n (leading dimension kBT)
  float* Yt = nullptr;  // FP32 with tensor cores: Y transposed
  int* err = nullptr;   // error word of the tensor-core GEMMs (set by backtr_set_error_word)
};

void backtr_set_error_word(BacktrPlan* p, int* err) { p->err = err; }

int backtr_plan_create(BacktrPlan** out, int n, bool f64, bool tc) {
  *out = nullptr;
  BacktrPlan* p = new BacktrPlan();
  p->n = n;
  p->f64 = f64;
  p->nblk = (n - 1 + kBT - 1) / kBT;
  const int bn = f64 ? GemmCfg<double>::BN : GemmCfg<float>::BN;
  const int tiles = (n + bn - 1) / bn;
  p->splits = std::max(1, std::min(16, (2 * 152 + tiles - 1) / tiles));
  const size_t el = f64 ? 8 : 4;
  cudaError_t err = cudaSuccess;
  auto alloc = [&](void** q, size_t bytes) {
    if (err == cudaSuccess) err = cudaMalloc(q, std::max<size_t>(bytes, 16));
  };
  alloc(&p->Y, el * (size_t)n * n);
  alloc(&p->Tm, el * (size_t)p->nblk * kBT * kBT);
  alloc(&p->Wp, el * (size_t)p->splits * kBT * n);
  alloc(&p->W2, el * (size_t)kBT * n);
  if (!f64 && tc && n % 4 == 0 && tc::tc_available()) alloc((void**)&p->Yt, sizeof(float) * (size_t)n * n);
  if (err == cudaSuccess)
    err = f64 ? cudaFuncSetAttribute((const void*)k_larft<double>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     (int)larft_smem_bytes<double>())
              : cudaFuncSetAttribute((const void*)k_larft<float>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     (int)larft_smem_bytes<float>());
  if (err != cudaSuccess) {
    backtr_plan_destroy(p);
    return -1000 - (int)err;
  }
  *out = p;
  return 0;
}

void backtr_plan_destroy(BacktrPlan* p) {
  if (!p) return;
  cudaFree(p->Y);
  cudaFree(p->Tm);
  cudaFree(p->Wp);
  cudaFree(p->W2);
  cudaFree(p->Yt);
  delete p;
}

// Z := Q Z (trans: Q' Z) for Z with ncol columns, in chunks of at most n
// columns (the W buffers' width). Q = B_0 B_1 ... with the blocks
// B_b = I - Y_b T_b Y_b': Q Z applies the last block first, Q' Z applies
// B_0' = I - Y_0 T_0' Y_0' first.
template <class T>
int backtr_run(BacktrPlan& p, const T* A, long long lda, const T* tau, T* Zall, long long ldz, int ncol, bool trans,
               cudaStream_t st) {
  const int n = p.n;
  if (n < 2 || ncol <= 0) return 0;
  T* Y = (T*)p.Y;
  // FP32 with tensor cores: both GEMMs of a block on tcgen05 (3xTF32) when
  // the tensor maps of Y, Y' and Z can be built (16-byte-aligned columns)
  CUtensorMap mY, mYt;
  const bool tc = sizeof(T) == 4 && p.Yt && p.err && (ldz % 4) == 0 && ((uintptr_t)Zall & 15) == 0 &&
                  tc::tc_make_map(&mY, (const float*)Y, n, n, n, tc::kBM) &&
                  tc::tc_make_map(&mYt, p.Yt, n, n, n, tc::kBM);
  k_form_y<T><<<dim3((n + 255) / 256, n), 256, 0, st>>>(A, lda, Y, n, tc ? (T*)p.Yt : (T*)nullptr);
  cudaError_t err = cudaGetLastError();
  if (err != cudaSuccess) return -1000 - (int)err;
  k_larft<T><<<p.nblk, 256, larft_smem_bytes<T>(), st>>>(Y, tau, (T*)p.Tm, n);
  if ((err = cudaGetLastError()) != cudaSuccess) return -1000 - (int)err;
  const bool f64 = sizeof(T) == 8;
  const int bk = f64 ? GemmCfg<double>::BK : GemmCfg<float>::BK;
  for (int c0 = 0; c0 < ncol; c0 += n) {
  const int nc = std::min(n, ncol - c0);
  T* Z = Zall + (long long)c0 * ldz;
  CUtensorMap mZ;
  const bool tcz = tc && tc::tc_make_map(&mZ, (const float*)Z, n, nc, ldz, tc::kBN);
  for (int bi = 0; bi < p.nblk; bi++) {
    const int b = trans ? bi : p.nblk - 1 - bi;
    const int j0 = b * kBT, kb = std::min(kBT, n - 1 - j0);
    // rows from r0 (j0 + 1 rounded down to a 16-byte boundary: Y is zero
    // above its unit diagonal, so the extra rows add nothing) keep Z's
    // column segments aligned for vector access
    const int r0 = (j0 + 1) & ~(16 / (int)sizeof(T) - 1);
    const int mrows = n - r0;
    if (tcz) {
      // W = Y_b' Z[r0:, :]: A operand rows = columns j0.. of Y (K = rows of
      // Y), B operand = columns of Z; split K as the SIMT path does
      int splits = std::max(1, std::min(p.splits, mrows / (4 * tc::kBK)));
      const int ks = ((mrows + splits - 1) / splits + tc::kBK - 1) / tc::kBK * tc::kBK;
      splits = (mrows + ks - 1) / ks;
      tc::TcArgs g{};
      g.M = kb;
      g.N = nc;
      g.nseg = 1;
      g.K[0] = mrows;
      g.a_x[0] = r0;
      g.b_x[0] = r0;
      g.a_y = j0;
      g.b_y = 0;
      g.ksplit = splits > 1 ? ks : 0;
      g.split_stride = (long long)kb * n;
      g.D = (float*)p.Wp;
      g.ldd = kb;
      g.alpha = 1.f;
      g.beta = 0.f;
      g.err = p.err;
      if ((err = tc::tc_gemm_launch(mY, mZ, g, splits, st)) != cudaSuccess) return -1000 - (int)err;
      k_tw<T><<<(nc + 15) / 16, 256, 0, st>>>((const T*)p.Wp, splits, (long long)kb * n,
                                              (const T*)p.Tm + (long long)b * kBT * kBT, (T*)p.W2, kb, nc,
                                              trans ? 1 : 0);
      if ((err = cudaGetLastError()) != cudaSuccess) return -1000 - (int)err;
      // Z[r0:, :] -= Y_b W2: A operand rows = rows r0.. of Y (K-major through
      // Y'), B operand = W2 (K = the block's kb reflectors)
      CUtensorMap mW2;
      if (!tc::tc_make_map(&mW2, (const float*)p.W2, kb, nc, kBT, tc::kBN)) return -1000 - (int)cudaErrorInvalidValue;
      tc::TcArgs h{};
      h.M = mrows;
      h.N = nc;
      h.nseg = 1;
      h.K[0] = kb;
      h.a_x[0] = j0;
      h.b_x[0] = 0;
      h.a_y = r0;
      h.b_y = 0;
      h.D = (float*)Z + r0;
      h.ldd = ldz;
      h.alpha = -1.f;
      h.beta = 1.f;
      h.err = p.err;
      if ((err = tc::tc_gemm_launch(mYt, mW2, h, 1, st)) != cudaSuccess) return -1000 - (int)err;
      continue;
    }
    // W = Y_b' Z[r0:, :]
    GemmDesc g{};
    g.m = kb;
    g.n = nc;
    g.k = mrows;
    g.A = Y + r0 + (long long)j0 * n;
    g.lda = n;
    g.B = Z + r0;
    g.ldb = ldz;
    g.C = p.Wp;
    g.ldc = kb;
    g.alpha = 1.0;
    g.beta = 0.0;
    int splits = std::max(1, std::min(p.splits, mrows / (4 * bk)));
    g.ksplit = splits > 1 ? ((mrows + splits - 1) / splits + bk - 1) / bk * bk : 0;
    if (splits > 1) splits = (mrows + g.ksplit - 1) / g.ksplit;
    g.split_stride = (long long)kb * n;
    if ((err = gemm_launch(f64, true, false, false, g, splits, st)) != cudaSuccess) return -1000 - (int)err;
    k_tw<T><<<(nc + 15) / 16, 256, 0, st>>>((const T*)p.Wp, splits, (long long)kb * n,
                                            (const T*)p.Tm + (long long)b * kBT * kBT, (T*)p.W2, kb, nc,
                                            trans ? 1 : 0);
    if ((err = cudaGetLastError()) != cudaSuccess) return -1000 - (int)err;
    // Z[r0:, :] -= Y_b W2
    GemmDesc h{};
    h.m = mrows;
    h.n = nc;
    h.k = kb;
    h.A = Y + r0 + (long long)j0 * n;
    h.lda = n;
    h.B = p.W2;
    h.ldb = kBT;
    h.C = Z + r0;
    h.ldc = ldz;
    h.alpha = -1.0;
    h.beta = 1.0;
    if ((err = gemm_launch(f64, false, false, false, h, 1, st)) != cudaSuccess) return -1000 - (int)err;
  }
  }
  return 0;
}

int backtr_enqueue(BacktrPlan* p, const void* A, long long lda, const void* tau, void* Z, long long ldz,
                   cudaStream_t st, int ncol, bool trans) {
  if (ncol < 0) ncol = p->n;
  if (p->f64)
    return backtr_run<double>(*p, (const double*)A, lda, (const double*)tau, (double*)Z, ldz, ncol, trans, st);
  return backtr_run<float>(*p, (const float*)A, lda, (const float*)tau, (float*)Z, ldz, ncol, trans, st);
}

}  // namespace gla
