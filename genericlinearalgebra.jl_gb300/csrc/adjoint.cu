// Adjoint (reverse-mode derivative) of the batched symmetric
// eigen-decomposition, one CTA per matrix. No counterpart in
// GenericLinearAlgebra.jl: it is the kernel behind an rrule for eigen.
//
// For A = V diag(w) V' and cotangents wbar (of w) and Vbar (of V), the
// gradient with respect to the symmetric A is
//
//   Abar = V (diag(wbar) + sym(F o (V' Vbar))) V',   sym(X) = (X + X')/2,
//   F_ij = 1 / (w_j - w_i) for |w_j - w_i| > gap_rel * max|w|, else 0
//
// (the eigenvector term of the standard first-order perturbation result;
// masking near-degenerate pairs keeps it finite, as only their joint
// eigenspace is defined). Because F is antisymmetric, sym(F o G) equals
// F o skew(G): the part of V'Vbar that would change the eigenvectors' norms
// drops out.
//
// The three products V'Vbar, V M and (V M) V' (symmetric: upper tiles) run
// in double-float arithmetic on the FP32 pipe (df64.cuh), the gaps and F in
// FP64.
#include "gla_adjoint.h"
#include "tile_gemm.cuh"

namespace gla {

size_t adjoint_workspace_bytes(int64_t a_elems) { return 4 * sizeof(df64) * (size_t)a_elems + 1024; }

__global__ void __launch_bounds__(kRT) k_adjoint(const SmallDesc* __restrict__ descs, const int* __restrict__ perm,
                                                 const double* __restrict__ w, const double* __restrict__ V,
                                                 const double* __restrict__ wbar, const double* __restrict__ Vbar,
                                                 double* __restrict__ Abar, df64* __restrict__ ws, int64_t a_elems,
                                                 double gap_rel) {
  __shared__ df64 As[16 * kTP];
  __shared__ df64 Bs[16 * kTP];
  __shared__ double lam[kSmallMaxN], lbar[kSmallMaxN];
  __shared__ double red[kRT / 32];
  const int mid = perm[blockIdx.x];
  const SmallDesc dsc = descs[mid];
  const int n = dsc.n, tid = threadIdx.x;
  const size_t ao = dsc.a_off;
  df64* V2 = ws + ao;
  df64* B2 = ws + a_elems + ao;
  df64* M = ws + 2 * a_elems + ao;
  df64* T = ws + 3 * a_elems + ao;
  double amax = 0;
  for (int i = tid; i < n; i += kRT) {
    lam[i] = w[dsc.w_off + i];
    lbar[i] = wbar[dsc.w_off + i];
    amax = fmax(amax, fabs(lam[i]));
  }
  for (int idx = tid; idx < n * n; idx += kRT) {
    V2[idx] = df_from(V[ao + idx]);
    B2[idx] = df_from(Vbar[ao + idx]);
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) amax = fmax(amax, __shfl_xor_sync(0xffffffffu, amax, o));
  if ((tid & 31) == 0) red[tid >> 5] = amax;
  __syncthreads();
  amax = 0;
  for (int i = 0; i < kRT / 32; i++) amax = fmax(amax, red[i]);
  const double gap_min = gap_rel * amax;
  const df64 zero = df_make(0.f, 0.f);
  auto zinit = [&](int, int) { return zero; };
  // G = V' Vbar (into M)
  tile_gemm_df<df64>(
      n, [&](int i, int k) { return V2[(size_t)i * n + k]; }, [&](int k, int j) { return B2[(size_t)j * n + k]; },
      zinit, [&](int i, int j, df64 v) { M[(size_t)j * n + i] = v; }, As, Bs, false);
  // M = diag(wbar) + sym(F o G), pairs (i, j) and (j, i) by one thread
  for (int idx = tid; idx < n * n; idx += kRT) {
    const int i = idx % n, j = idx / n;
    if (i > j) continue;
    if (i == j) {
      M[idx] = df_from(lbar[i]);
      continue;
    }
    const double gap = lam[j] - lam[i];
    const df64 gij = M[(size_t)j * n + i], gji = M[(size_t)i * n + j];
    df64 m = zero;
    if (fabs(gap) > gap_min) {
      // 0.5 F_ij (G_ij - G_ji), F_ij = 1/(lam_j - lam_i)
      const df64 diff = df_add(gij, df_neg(gji));
      m = df_mul(diff, df_from(0.5 / gap));
    }
    M[(size_t)j * n + i] = m;
    M[(size_t)i * n + j] = m;
  }
  __syncthreads();
  // T = V M
  tile_gemm_df<df64>(
      n, [&](int i, int k) { return V2[(size_t)k * n + i]; }, [&](int k, int j) { return M[(size_t)j * n + k]; },
      zinit, [&](int i, int j, df64 v) { T[(size_t)j * n + i] = v; }, As, Bs, false);
  // Abar = T V' (symmetric: upper tiles, mirrored)
  double* Ab = Abar + ao;
  tile_gemm_df<df64>(
      n, [&](int i, int k) { return T[(size_t)k * n + i]; }, [&](int k, int j) { return V2[(size_t)k * n + j]; },
      zinit,
      [&](int i, int j, df64 v) {
        const double x = df_to(v);
        Ab[(size_t)j * n + i] = x;
        Ab[(size_t)i * n + j] = x;
      },
      As, Bs, true);
}

cudaError_t launch_adjoint(int nblocks, cudaStream_t st, const SmallDesc* descs, const int* perm, const double* w,
                           const double* V, const double* wbar, const double* Vbar, double* Abar, df64* ws,
                           int64_t a_elems, double gap_rel) {
  if (nblocks <= 0) return cudaSuccess;
  k_adjoint<<<nblocks, kRT, 0, st>>>(descs, perm, w, V, wbar, Vbar, Abar, ws, a_elems, gap_rel);
  return cudaGetLastError();
}

}  // namespace gla
