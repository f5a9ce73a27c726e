// Double-float GEMM on the FP32 pipe for the large-matrix refinement:
//
//   C = op(A) B     with A = Ahi + Alo, B = Bhi + Blo (the lo parts optional),
//                   C returned as Chi + Clo (~2^-47 relative per element)
//
// Products: Ahi*Bhi exactly by TwoProduct (fma), the cross terms
// Ahi*Blo + Alo*Bhi in FP32 (they are 2^-24 smaller); sums by TwoSum.
// Each 16-wide k-slab is accumulated from zero into (s, c) (s by TwoSum, the
// error terms lazily into c) and then folded into the running tile total by
// an accurate double-float addition, so the rounding of the low parts grows
// with the slab length, not with k: for k = 4096 a single running
// accumulator would lose ~sqrt(k) * 2^-48, which is visible in an FP64-class
// residual of an order-4096 matrix.
//
// 64 x 64 output tiles, 256 threads with 4 x 4 outputs each, both operands
// staged in shared memory (hi and lo planes), double buffered.
#include "df64.cuh"
#include "gla_large.h"

namespace gla {

namespace {
constexpr int kDBM = 64, kDBN = 64, kDBK = 16, kDT = 256;

template <bool TA, bool ALO, bool BLO>
__global__ void __launch_bounds__(kDT) k_dfgemm(const DfGemmDesc g) {
  __shared__ __align__(16) float Ah[2][kDBK][kDBM], Al[2][kDBK][kDBM];
  __shared__ __align__(16) float Bh[2][kDBK][kDBN], Bl[2][kDBK][kDBN];
  const int m = g.m, n = g.n, K = g.k;
  const int tiles_m = (m + kDBM - 1) / kDBM;
  const int bi = blockIdx.x % tiles_m, bj = blockIdx.x / tiles_m;
  const int row0 = bi * kDBM, col0 = bj * kDBN;
  if (g.lower && row0 + kDBM <= col0) return;
  const int t = threadIdx.x, tx = t % 16, ty = t / 16;
  constexpr int L = kDBM * kDBK / kDT;  // 4 elements per operand per thread
  float rah[L], ral[L], rbh[L], rbl[L];
  auto load = [&](int k0) {
#pragma unroll
    for (int r = 0; r < L; r++) {
      const int e = t + r * kDT;
      const int i = TA ? e / kDBK : e % kDBM;
      const int kk = TA ? e % kDBK : e / kDBM;
      const int gi = row0 + i, gk = k0 + kk;
      float h = 0.f, l = 0.f;
      if (gi < m && gk < K) {
        const long long idx = TA ? (long long)gk + (long long)gi * g.lda : (long long)gi + (long long)gk * g.lda;
        h = g.Ahi[idx];
        if (ALO) l = g.Alo[idx];
      }
      rah[r] = h;
      ral[r] = l;
    }
#pragma unroll
    for (int r = 0; r < L; r++) {
      const int e = t + r * kDT;
      const int kk = e % kDBK, j = e / kDBK;
      const int gj = col0 + j, gk = k0 + kk;
      float h = 0.f, l = 0.f;
      if (gj < n && gk < K) {
        const long long idx = (long long)gk + (long long)gj * g.ldb;
        h = g.Bhi[idx];
        if (BLO) l = g.Blo[idx];
      }
      rbh[r] = h;
      rbl[r] = l;
    }
  };
  auto store = [&](int b) {
#pragma unroll
    for (int r = 0; r < L; r++) {
      const int e = t + r * kDT;
      const int i = TA ? e / kDBK : e % kDBM;
      const int kk = TA ? e % kDBK : e / kDBM;
      Ah[b][kk][i] = rah[r];
      if (ALO) Al[b][kk][i] = ral[r];
    }
#pragma unroll
    for (int r = 0; r < L; r++) {
      const int e = t + r * kDT;
      const int kk = e % kDBK, j = e / kDBK;
      Bh[b][kk][j] = rbh[r];
      if (BLO) Bl[b][kk][j] = rbl[r];
    }
  };
  df64 tot[4][4];
#pragma unroll
  for (int i = 0; i < 4; i++)
#pragma unroll
    for (int j = 0; j < 4; j++) tot[i][j] = df_make(0.f, 0.f);
  const int nk = (K + kDBK - 1) / kDBK;
  if (nk > 0) {
    load(0);
    store(0);
    __syncthreads();
    int b = 0;
    for (int kt = 0; kt < nk; kt++) {
      if (kt + 1 < nk) load((kt + 1) * kDBK);
      float s[4][4], c[4][4];
#pragma unroll
      for (int i = 0; i < 4; i++)
#pragma unroll
        for (int j = 0; j < 4; j++) s[i][j] = c[i][j] = 0.f;
#pragma unroll
      for (int kk = 0; kk < kDBK; kk++) {
        const float4 ah = *reinterpret_cast<const float4*>(&Ah[b][kk][ty * 4]);
        const float4 bh = *reinterpret_cast<const float4*>(&Bh[b][kk][tx * 4]);
        float4 al = make_float4(0.f, 0.f, 0.f, 0.f), bl = make_float4(0.f, 0.f, 0.f, 0.f);
        if (ALO) al = *reinterpret_cast<const float4*>(&Al[b][kk][ty * 4]);
        if (BLO) bl = *reinterpret_cast<const float4*>(&Bl[b][kk][tx * 4]);
        const float a_h[4] = {ah.x, ah.y, ah.z, ah.w}, a_l[4] = {al.x, al.y, al.z, al.w};
        const float b_h[4] = {bh.x, bh.y, bh.z, bh.w}, b_l[4] = {bl.x, bl.y, bl.z, bl.w};
#pragma unroll
        for (int i = 0; i < 4; i++)
#pragma unroll
          for (int j = 0; j < 4; j++) {
            const float p = a_h[i] * b_h[j];
            float e = fmaf(a_h[i], b_h[j], -p);
            if (BLO) e = fmaf(a_h[i], b_l[j], e);
            if (ALO) e = fmaf(a_l[i], b_h[j], e);
            float sn, err;
            two_sum(s[i][j], p, sn, err);
            s[i][j] = sn;
            c[i][j] += err + e;
          }
      }
#pragma unroll
      for (int i = 0; i < 4; i++)
#pragma unroll
        for (int j = 0; j < 4; j++) {
          df64 slab;
          quick_two_sum(s[i][j], c[i][j], slab.hi, slab.lo);
          tot[i][j] = df_add(tot[i][j], slab);
        }
      if (kt + 1 < nk) store(b ^ 1);
      __syncthreads();
      b ^= 1;
    }
  }
#pragma unroll
  for (int i = 0; i < 4; i++) {
    const int r = row0 + ty * 4 + i;
    if (r >= m) continue;
#pragma unroll
    for (int j = 0; j < 4; j++) {
      const int cc = col0 + tx * 4 + j;
      if (cc >= n || (g.lower && r < cc)) continue;
      const long long idx = (long long)r + (long long)cc * g.ldc;
      g.Chi[idx] = tot[i][j].hi;
      g.Clo[idx] = tot[i][j].lo;
    }
  }
}
}  // namespace

cudaError_t dfgemm_launch(const DfGemmDesc& g, bool ta, cudaStream_t st) {
  if (g.m <= 0 || g.n <= 0) return cudaSuccess;
  const int tiles = ((g.m + kDBM - 1) / kDBM) * ((g.n + kDBN - 1) / kDBN);
  const bool alo = g.Alo != nullptr, blo = g.Blo != nullptr;
  const int code = (ta ? 4 : 0) | (alo ? 2 : 0) | (blo ? 1 : 0);
  switch (code) {
    case 0: k_dfgemm<false, false, false><<<tiles, kDT, 0, st>>>(g); break;
    case 1: k_dfgemm<false, false, true><<<tiles, kDT, 0, st>>>(g); break;
    case 2: k_dfgemm<false, true, false><<<tiles, kDT, 0, st>>>(g); break;
    case 3: k_dfgemm<false, true, true><<<tiles, kDT, 0, st>>>(g); break;
    case 4: k_dfgemm<true, false, false><<<tiles, kDT, 0, st>>>(g); break;
    case 5: k_dfgemm<true, false, true><<<tiles, kDT, 0, st>>>(g); break;
    case 6: k_dfgemm<true, true, false><<<tiles, kDT, 0, st>>>(g); break;
    default: k_dfgemm<true, true, true><<<tiles, kDT, 0, st>>>(g); break;
  }
  return cudaGetLastError();
}

}  // namespace gla
