// Register-blocked SIMT GEMM used by the large-matrix path:
//
//   C(i, j) = alpha * sum_kk op(A)(i, kk) * op(B)(kk, j) + beta * C(i, j)
//
// column-major operands with leading dimensions, optional transposes, an
// optional lower-triangle-only output (symmetric rank-k updates), index
// remaps on the k dimension of A and B (gathered columns of a matrix) and
// on the output columns (scattered columns), and split-K into a partial
// buffer. FP64 runs 64x64 tiles with 4x4 per thread (the FP64 pipe is the
// bound); FP32 runs 128x128 tiles with 8x8 per thread. Tiles are double
// buffered in shared memory with a register prefetch of the next k-slab.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace gla {

struct GemmDesc {
  int m, n, k;
  int ksplit;          // k columns per split (0: no split); split s writes C + s * split_stride
  const void* A;
  long long lda;
  const void* B;
  long long ldb;
  void* C;
  long long ldc;
  long long split_stride;
  const int* a_kidx;   // physical k index of A (column if A is not transposed, row if it is)
  const int* b_kidx;   // physical k index of B (row if B is not transposed, column if it is)
  const int* c_nidx;   // physical column of C for output column j
  double alpha, beta;
};

template <class T>
struct GemmCfg;
template <>
struct GemmCfg<double> {
  static constexpr int BM = 64, BN = 64, BK = 16, TM = 4, TN = 4;
};
template <>
struct GemmCfg<float> {
  static constexpr int BM = 128, BN = 128, BK = 8, TM = 8, TN = 8;
};
constexpr int kGemmThreads = 256;

template <class T>
struct Vec16;
template <>
struct Vec16<double> {
  using type = double2;
};
template <>
struct Vec16<float> {
  using type = float4;
};

template <class T, bool TA, bool TB, bool LOWER>
__device__ __forceinline__ void gemm_body(const GemmDesc& g, int tile, int split) {
  using Cf = GemmCfg<T>;
  constexpr int BM = Cf::BM, BN = Cf::BN, BK = Cf::BK, TM = Cf::TM, TN = Cf::TN;
  constexpr int NTX = BN / TN, NTY = BM / TM, NT = NTX * NTY;
  static_assert(NT == kGemmThreads, "thread count");
  constexpr int VW = 16 / sizeof(T);
  constexpr int NVM = TM / VW, NVN = TN / VW;
  constexpr int LA = BM * BK / NT, LB = BK * BN / NT;
  using V = typename Vec16<T>::type;
  __shared__ __align__(16) T As[2][BK][BM];
  __shared__ __align__(16) T Bs[2][BK][BN];

  const int m = g.m, n = g.n;
  int kbeg = 0, kend = g.k;
  T* C = (T*)g.C;
  if (g.ksplit > 0) {
    kbeg = split * g.ksplit;
    kend = min(g.k, kbeg + g.ksplit);
    C += (size_t)split * (size_t)g.split_stride;
  }
  const int tiles_m = (m + BM - 1) / BM;
  const int bi = tile % tiles_m, bj = tile / tiles_m;
  const int row0 = bi * BM, col0 = bj * BN;
  if (LOWER && row0 + BM <= col0) return;  // tile wholly above the diagonal

  const int t = threadIdx.x, tx = t % NTX, ty = t / NTX;
  const T* A = (const T*)g.A;
  const T* B = (const T*)g.B;
  const long long lda = g.lda, ldb = g.ldb;
  const int* akx = g.a_kidx;
  const int* bkx = g.b_kidx;

  T ra[LA], rb[LB];
  auto load = [&](int k0) {
#pragma unroll
    for (int r = 0; r < LA; r++) {
      const int e = t + r * NT;
      const int i = TA ? e / BK : e % BM;
      const int kk = TA ? e % BK : e / BM;
      const int gi = row0 + i, gk = k0 + kk;
      T v = T(0);
      if (gi < m && gk < kend) {
        const long long pk = akx ? (long long)akx[gk] : (long long)gk;
        v = TA ? A[pk + (long long)gi * lda] : A[gi + pk * lda];
      }
      ra[r] = v;
    }
#pragma unroll
    for (int r = 0; r < LB; r++) {
      const int e = t + r * NT;
      const int j = TB ? e % BN : e / BK;
      const int kk = TB ? e / BN : e % BK;
      const int gj = col0 + j, gk = k0 + kk;
      T v = T(0);
      if (gj < n && gk < kend) {
        const long long pk = bkx ? (long long)bkx[gk] : (long long)gk;
        v = TB ? B[gj + pk * ldb] : B[pk + (long long)gj * ldb];
      }
      rb[r] = v;
    }
  };
  auto store = [&](int buf) {
#pragma unroll
    for (int r = 0; r < LA; r++) {
      const int e = t + r * NT;
      const int i = TA ? e / BK : e % BM;
      const int kk = TA ? e % BK : e / BM;
      As[buf][kk][i] = ra[r];
    }
#pragma unroll
    for (int r = 0; r < LB; r++) {
      const int e = t + r * NT;
      const int j = TB ? e % BN : e / BK;
      const int kk = TB ? e / BN : e % BK;
      Bs[buf][kk][j] = rb[r];
    }
  };

  T acc[TM][TN];
#pragma unroll
  for (int i = 0; i < TM; i++)
#pragma unroll
    for (int j = 0; j < TN; j++) acc[i][j] = T(0);

  const int nk = kend > kbeg ? (kend - kbeg + BK - 1) / BK : 0;
  if (nk > 0) {
    load(kbeg);
    store(0);
    __syncthreads();
    int buf = 0;
    for (int kt = 0; kt < nk; kt++) {
      if (kt + 1 < nk) load(kbeg + (kt + 1) * BK);
#pragma unroll
      for (int kk = 0; kk < BK; kk++) {
        T a[TM], b[TN];
#pragma unroll
        for (int v = 0; v < NVM; v++) {
          const V x = *reinterpret_cast<const V*>(&As[buf][kk][v * (BM / NVM) + ty * VW]);
          const T* xs = reinterpret_cast<const T*>(&x);
#pragma unroll
          for (int q = 0; q < VW; q++) a[v * VW + q] = xs[q];
        }
#pragma unroll
        for (int w = 0; w < NVN; w++) {
          const V x = *reinterpret_cast<const V*>(&Bs[buf][kk][w * (BN / NVN) + tx * VW]);
          const T* xs = reinterpret_cast<const T*>(&x);
#pragma unroll
          for (int q = 0; q < VW; q++) b[w * VW + q] = xs[q];
        }
#pragma unroll
        for (int i = 0; i < TM; i++)
#pragma unroll
          for (int j = 0; j < TN; j++) acc[i][j] = fma(a[i], b[j], acc[i][j]);
      }
      if (kt + 1 < nk) store(buf ^ 1);
      __syncthreads();
      buf ^= 1;
    }
  }

  const T alpha = (T)g.alpha, beta = (T)g.beta;
  const bool split_out = g.ksplit > 0;
#pragma unroll
  for (int v = 0; v < NVM; v++)
#pragma unroll
    for (int q = 0; q < VW; q++) {
      const int r = row0 + v * (BM / NVM) + ty * VW + q;
      if (r >= m) continue;
#pragma unroll
      for (int w = 0; w < NVN; w++)
#pragma unroll
        for (int s = 0; s < VW; s++) {
          const int c = col0 + w * (BN / NVN) + tx * VW + s;
          if (c >= n || (LOWER && r < c)) continue;
          const long long pc = g.c_nidx ? (long long)g.c_nidx[c] : (long long)c;
          T* p = C + r + pc * g.ldc;
          const T x = acc[v * VW + q][w * VW + s];
          if (split_out)
            *p = x;
          else
            *p = beta == T(0) ? alpha * x : fma(alpha, x, beta * *p);
        }
    }
}

}  // namespace gla
