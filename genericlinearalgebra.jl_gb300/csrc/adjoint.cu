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
// to double-float accuracy on the tcgen05 tensor cores (tc_small.cuh, the
// Ozaki scheme of the refinement's products; TC) or in double-float
// arithmetic on the FP32 pipe (df64.cuh); the gaps and F in FP64.
#include "gla_adjoint.h"
#include "tc_small.cuh"
#include "tile_gemm.cuh"

namespace gla {

size_t adjoint_workspace_bytes(int64_t a_elems) { return 4 * sizeof(df64) * (size_t)a_elems + 1024; }

template <bool TC>
__global__ void __launch_bounds__(kRT) k_adjoint(const SmallDesc* __restrict__ descs, const int* __restrict__ perm,
                                                 const double* __restrict__ w, const double* __restrict__ V,
                                                 const double* __restrict__ wbar, const double* __restrict__ Vbar,
                                                 double* __restrict__ Abar, df64* __restrict__ ws, int64_t a_elems,
                                                 double gap_rel, int* __restrict__ err) {
  __shared__ df64 As[TC ? 1 : 16 * kTP];
  __shared__ df64 Bs[TC ? 1 : 16 * kTP];
  __shared__ double lam[kSmallMaxN], lbar[kSmallMaxN];
  __shared__ double red[kRT / 32];
  __shared__ int e1[TC ? kSmallMaxN : 1], e2[TC ? kSmallMaxN : 1];
  extern __shared__ __align__(128) unsigned char asm_raw[];
  __shared__ tcs::Shared tsh;
  tcs::Ctx tcx;
  if (TC) tcs::setup(tcx, &tsh, asm_raw, err);
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
  __syncthreads();  // V2, B2 complete
  if (TC) {
    tcs::col_exps(n, V2, e1);  // rows of V' = columns of V
    tcs::col_exps(n, B2, e2);
    tcs::gemm(
        tcx, n, e1, e2, [&](int i, int k) { return V2[(size_t)i * n + k]; },
        [&](int k, int j) { return B2[(size_t)j * n + k]; }, [&](int i, int j, df64 v) { M[(size_t)j * n + i] = v; },
        false);
  } else {
    tile_gemm_df<df64>(
        n, [&](int i, int k) { return V2[(size_t)i * n + k]; }, [&](int k, int j) { return B2[(size_t)j * n + k]; },
        zinit, [&](int i, int j, df64 v) { M[(size_t)j * n + i] = v; }, As, Bs, false);
  }
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
  double* Ab = Abar + ao;
  auto store_ab = [&](int i, int j, df64 v) {
    const double x = df_to(v);
    Ab[(size_t)j * n + i] = x;
    Ab[(size_t)i * n + j] = x;
  };
  if (TC) {
    tcs::row_exps(n, V2, e1);
    tcs::col_exps(n, M, e2);
    tcs::gemm(
        tcx, n, e1, e2, [&](int i, int k) { return V2[(size_t)k * n + i]; },
        [&](int k, int j) { return M[(size_t)j * n + k]; }, [&](int i, int j, df64 v) { T[(size_t)j * n + i] = v; },
        false);
    // Abar = T V' (symmetric: upper triangle, mirrored); columns of V' = rows of V (e1)
    tcs::row_exps(n, T, e2);
    tcs::gemm(
        tcx, n, e2, e1, [&](int i, int k) { return T[(size_t)k * n + i]; },
        [&](int k, int j) { return V2[(size_t)k * n + j]; }, store_ab, true);
    if (!tcs::ok(tcx))  // a tensor-core wait ran out: no gradient for this matrix
      for (int idx = tid; idx < n * n; idx += kRT) Ab[idx] = NAN;
    tcs::teardown(tcx);
  } else {
    tile_gemm_df<df64>(
        n, [&](int i, int k) { return V2[(size_t)k * n + i]; }, [&](int k, int j) { return M[(size_t)j * n + k]; },
        zinit, [&](int i, int j, df64 v) { T[(size_t)j * n + i] = v; }, As, Bs, false);
    // Abar = T V' (symmetric: upper tiles, mirrored)
    tile_gemm_df<df64>(
        n, [&](int i, int k) { return T[(size_t)k * n + i]; }, [&](int k, int j) { return V2[(size_t)k * n + j]; },
        zinit, store_ab, As, Bs, true);
  }
}

// Dynamic shared memory of k_adjoint: the product slabs, padded so that no
// more than two CTAs share an SM (each holds 256 of its 512 TMEM columns).
constexpr int kAdjSmem = 80 * 1024;
static_assert(kAdjSmem >= tcs::kSmem, "the product slabs");

cudaError_t adjoint_kernels_init() {
  return cudaFuncSetAttribute(k_adjoint<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, kAdjSmem);
}

cudaError_t launch_adjoint(int nblocks, cudaStream_t st, const SmallDesc* descs, const int* perm, const double* w,
                           const double* V, const double* wbar, const double* Vbar, double* Abar, df64* ws,
                           int64_t a_elems, double gap_rel) {
  if (nblocks <= 0) return cudaSuccess;
  // the tensor-core error word: the workspace's 1024-byte tail, cleared per call
  int* err = reinterpret_cast<int*>(ws + 4 * a_elems);
  cudaError_t e = cudaMemsetAsync(err, 0, sizeof(int), st);
  if (e != cudaSuccess) return e;
  k_adjoint<true><<<nblocks, kRT, kAdjSmem, st>>>(descs, perm, w, V, wbar, Vbar, Abar, ws, a_elems, gap_rel, err);
  return cudaGetLastError();
}

}  // namespace gla
