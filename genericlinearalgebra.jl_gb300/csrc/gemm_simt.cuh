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

// REMAP: honour a_kidx / b_kidx / c_nidx (plain GEMMs skip the index loads
// and their registers).
template <class T, bool TA, bool TB, bool LOWER, bool REMAP>
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
  const int* akx = REMAP ? g.a_kidx : nullptr;
  const int* bkx = REMAP ? g.b_kidx : nullptr;

  T ra[LA], rb[LB];
  // Without remaps every load of a thread sits at a fixed offset from one
  // moving pointer (advanced by one k-slab per step).
  const int i_a0 = TA ? t / BK : t % BM, k_a0 = TA ? t % BK : t / BM;  // element r: e = t + r NT
  const int j_b0 = TB ? t % BN : t / BK, k_b0 = TB ? t / BN : t % BK;
  constexpr int DI_A = TA ? NT / BK : 0, DK_A = TA ? 0 : NT / BM;     // per-r steps
  constexpr int DJ_B = TB ? 0 : NT / BK, DK_B = TB ? NT / BN : 0;
  const T* pa = A + (TA ? (long long)(row0 + i_a0) * lda + (kbeg + k_a0) : (row0 + i_a0) + (long long)(kbeg + k_a0) * lda);
  const T* pb = B + (TB ? (col0 + j_b0) + (long long)(kbeg + k_b0) * ldb : (long long)(col0 + j_b0) * ldb + (kbeg + k_b0));
  const long long step_a = TA ? BK : (long long)BK * lda, step_b = TB ? (long long)BK * ldb : BK;
  auto load = [&](int k0) {
    if (!REMAP) {
      const int kofs = k0 - kbeg;
#pragma unroll
      for (int r = 0; r < LA; r++) {
        const int gi = row0 + i_a0 + r * DI_A, gk = k0 + k_a0 + r * DK_A;
        const long long off = TA ? (long long)r * DI_A * lda : (long long)r * DK_A * lda;
        ra[r] = (gi < m && gk < kend) ? pa[off + (TA ? kofs : (long long)kofs * lda)] : T(0);
      }
#pragma unroll
      for (int r = 0; r < LB; r++) {
        const int gj = col0 + j_b0 + r * DJ_B, gk = k0 + k_b0 + r * DK_B;
        const long long off = TB ? (long long)r * DK_B * ldb : (long long)r * DJ_B * ldb;
        rb[r] = (gj < n && gk < kend) ? pb[off + (TB ? (long long)kofs * ldb : kofs)] : T(0);
      }
      return;
    }
#pragma unroll
    for (int r = 0; r < LA; r++) {
      const int e = t + r * NT;
      const int i = TA ? e / BK : e % BM;
      const int kk = TA ? e % BK : e / BM;
      const int gi = row0 + i, gk = k0 + kk;
      T v = T(0);
      if (gi < m && gk < kend) {
        const long long pk = (REMAP && akx) ? (long long)akx[gk] : (long long)gk;
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
        const long long pk = (REMAP && bkx) ? (long long)bkx[gk] : (long long)gk;
        v = TB ? B[gj + pk * ldb] : B[pk + (long long)gj * ldb];
      }
      rb[r] = v;
    }
  };
  (void)step_a;
  (void)step_b;
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
  // rows r0 .. r0+VW-1 of an output column are contiguous: one 16-byte
  // access when the column start is aligned
  const bool vec = ((reinterpret_cast<unsigned long long>(C) & 15) == 0) && (g.ldc % VW == 0);
#pragma unroll
  for (int v = 0; v < NVM; v++) {
    const int r0 = row0 + v * (BM / NVM) + ty * VW;
    if (r0 >= m) continue;
#pragma unroll
    for (int w = 0; w < NVN; w++)
#pragma unroll
      for (int s = 0; s < VW; s++) {
        const int c = col0 + w * (BN / NVN) + tx * VW + s;
        if (c >= n) continue;
        const long long pc = (REMAP && g.c_nidx) ? (long long)g.c_nidx[c] : (long long)c;
        T* p = C + r0 + pc * g.ldc;
        if (vec && r0 + VW <= m && (!LOWER || r0 >= c)) {
          V out;
          T* o = reinterpret_cast<T*>(&out);
          if (split_out || beta == T(0)) {
#pragma unroll
            for (int q = 0; q < VW; q++) o[q] = (split_out ? T(1) : alpha) * acc[v * VW + q][w * VW + s];
          } else {
            const V old = *reinterpret_cast<const V*>(p);
            const T* po = reinterpret_cast<const T*>(&old);
#pragma unroll
            for (int q = 0; q < VW; q++) o[q] = fma(alpha, acc[v * VW + q][w * VW + s], beta * po[q]);
          }
          *reinterpret_cast<V*>(p) = out;
        } else {
#pragma unroll
          for (int q = 0; q < VW; q++) {
            const int r = r0 + q;
            if (r >= m || (LOWER && r < c)) continue;
            const T x = acc[v * VW + q][w * VW + s];
            if (split_out)
              p[q] = x;
            else
              p[q] = beta == T(0) ? alpha * x : fma(alpha, x, beta * p[q]);
          }
        }
      }
  }
}

}  // namespace gla
