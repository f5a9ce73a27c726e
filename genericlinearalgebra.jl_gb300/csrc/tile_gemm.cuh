// Batched small-matrix GEMM building blocks (one CTA of kTileThreads per
// matrix, 64 x 64 output tiles, 4 x 4 outputs per thread, operands read
// through accessor functors so that transposes, triangles and on-the-fly
// conversions cost nothing extra). Used by the eigenpair refinement and the
// adjoint kernel.
#pragma once
#include "df64.cuh"

namespace gla {

constexpr int kRT = 256;  // threads per CTA of the tile GEMMs

// C(i, j) = init(i, j) + sum_k la(i, k) * lb(k, j) over 64 x 64 output tiles;
// 256 threads, 4 x 4 outputs per thread, double-float accumulation.
// `upper` skips tiles strictly below the diagonal and stores i <= j only.
// Operand slices (16 x 64) are staged in shared memory with a padded row
// (kTP = 65 elements: conflict-free stores of the k-fastest global reads) and
// the next slice is prefetched into registers while the current one is used.
constexpr int kTP = 65;
template <class TB, class LA, class LB, class IN, class ST>
GLA_DEV void tile_gemm_df(int n, const LA& la, const LB& lb, const IN& init, const ST& store, df64* As, TB* Bs,
                          bool upper) {
  const int tid = threadIdx.x, tx = tid & 15, ty = tid >> 4;
  const int kk_ld = tid & 15, ii_ld = tid >> 4;  // this thread loads (kk_ld, ii_ld + 16 q), q < 4
  for (int i0 = 0; i0 < n; i0 += 64) {
    for (int j0 = 0; j0 < n; j0 += 64) {
      if (upper && j0 + 63 < i0) continue;
      df64 acc[4][4];
#pragma unroll
      for (int u = 0; u < 4; u++)
#pragma unroll
        for (int v = 0; v < 4; v++) {
          const int i = i0 + tx + 16 * u, j = j0 + ty + 16 * v;
          acc[u][v] = (i < n && j < n) ? init(i, j) : df_make(0.f, 0.f);
        }
      df64 ra[4];
      TB rb[4];
      auto fetch = [&](int k0) {
        const int k = k0 + kk_ld;
#pragma unroll
        for (int q = 0; q < 4; q++) {
          const int i = i0 + ii_ld + 16 * q, j = j0 + ii_ld + 16 * q;
          ra[q] = (i < n && k < n) ? la(i, k) : df_make(0.f, 0.f);
          rb[q] = (j < n && k < n) ? lb(k, j) : TB();
        }
      };
      fetch(0);
      for (int k0 = 0; k0 < n; k0 += 16) {
        __syncthreads();
#pragma unroll
        for (int q = 0; q < 4; q++) {
          As[kk_ld * kTP + ii_ld + 16 * q] = ra[q];
          Bs[kk_ld * kTP + ii_ld + 16 * q] = rb[q];
        }
        __syncthreads();
        if (k0 + 16 < n) fetch(k0 + 16);
#pragma unroll 2
        for (int kk = 0; kk < 16; kk++) {
          df64 a[4];
          TB b[4];
#pragma unroll
          for (int u = 0; u < 4; u++) a[u] = As[kk * kTP + tx + 16 * u];
#pragma unroll
          for (int v = 0; v < 4; v++) b[v] = Bs[kk * kTP + ty + 16 * v];
#pragma unroll
          for (int u = 0; u < 4; u++)
#pragma unroll
            for (int v = 0; v < 4; v++) acc[u][v] = df_mac(acc[u][v], a[u], b[v]);
        }
      }
#pragma unroll
      for (int u = 0; u < 4; u++)
#pragma unroll
        for (int v = 0; v < 4; v++) {
          const int i = i0 + tx + 16 * u, j = j0 + ty + 16 * v;
          if (i < n && j < n && (!upper || i <= j)) store(i, j, acc[u][v]);
        }
    }
  }
  __syncthreads();
}

// FP32 variant of tile_gemm_df (the X E update).
template <class LA, class LB, class ST>
GLA_DEV void tile_gemm_f32(int n, const LA& la, const LB& lb, const ST& store, float* As, float* Bs, bool upper) {
  const int tid = threadIdx.x, tx = tid & 15, ty = tid >> 4;
  const int kk_ld = tid & 15, ii_ld = tid >> 4;
  for (int i0 = 0; i0 < n; i0 += 64) {
    for (int j0 = 0; j0 < n; j0 += 64) {
      if (upper && j0 + 63 < i0) continue;
      float acc[4][4];
#pragma unroll
      for (int u = 0; u < 4; u++)
#pragma unroll
        for (int v = 0; v < 4; v++) acc[u][v] = 0.f;
      float ra[4], rb[4];
      auto fetch = [&](int k0) {
        const int k = k0 + kk_ld;
#pragma unroll
        for (int q = 0; q < 4; q++) {
          const int i = i0 + ii_ld + 16 * q, j = j0 + ii_ld + 16 * q;
          ra[q] = (i < n && k < n) ? la(i, k) : 0.f;
          rb[q] = (j < n && k < n) ? lb(k, j) : 0.f;
        }
      };
      fetch(0);
      for (int k0 = 0; k0 < n; k0 += 16) {
        __syncthreads();
#pragma unroll
        for (int q = 0; q < 4; q++) {
          As[kk_ld * kTP + ii_ld + 16 * q] = ra[q];
          Bs[kk_ld * kTP + ii_ld + 16 * q] = rb[q];
        }
        __syncthreads();
        if (k0 + 16 < n) fetch(k0 + 16);
#pragma unroll 4
        for (int kk = 0; kk < 16; kk++) {
          float a[4], b[4];
#pragma unroll
          for (int u = 0; u < 4; u++) a[u] = As[kk * kTP + tx + 16 * u];
#pragma unroll
          for (int v = 0; v < 4; v++) b[v] = Bs[kk * kTP + ty + 16 * v];
#pragma unroll
          for (int u = 0; u < 4; u++)
#pragma unroll
            for (int v = 0; v < 4; v++) acc[u][v] = fmaf(a[u], b[v], acc[u][v]);
        }
      }
#pragma unroll
      for (int u = 0; u < 4; u++)
#pragma unroll
        for (int v = 0; v < 4; v++) {
          const int i = i0 + tx + 16 * u, j = j0 + ty + 16 * v;
          if (i < n && j < n && (!upper || i <= j)) store(i, j, acc[u][v]);
        }
    }
  }
  __syncthreads();
}

}  // namespace gla
