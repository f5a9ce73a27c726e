// FP32 tridiagonal eigensolver of the FP32 + refinement path (n <= 128),
// run by the CTA that has just tridiagonalised the matrix and formed Q in
// shared memory. No counterpart in GenericLinearAlgebra.jl: the reference's
// eigQL! (src/eigenSelfAdjoint.jl:221-288) is one serial chase per matrix;
// here every eigenpair is found by its own thread, so the critical path is
// O(n) dependent steps per eigenvalue instead of O(n^2) rotations per matrix.
//
//   1. Eigenvalues: bisection on Sturm counts (the inertia recurrence of
//      numnegevals, src/tridiag.jl:20-36, with LAPACK's pivmin guard), three
//      interleaved probes per step (quadsection, 2 bits per step), to an
//      absolute width of eps32 * ||T|| (Gershgorin bound).
//   2. Eigenvectors: the twisted factorisation T - lam I = N_r D_r N_r'
//      (K. V. Fernando 1997; B. N. Parlett, I. S. Dhillon, "Fernando's
//      solution to Wilkinson's problem", LAA 267 (1997)): stationary
//      forward and progressive backward LDL' pivots, the twist index r
//      minimising |gamma_r|, and z with z_r = 1 from the two bidiagonal
//      recurrences; one pass, no iteration.
//   3. Eigenvalues closer than 1e-3 ||T|| (LAPACK dstein's cluster bound)
//      have their vectors re-orthogonalised by modified Gram-Schmidt, one
//      warp per cluster.
//   4. X = Q Y, the eigenvectors of the dense matrix (columns ascending).
//
// A matrix whose eigenvalues come within kTightGap ||T|| of each other
// (there FP32 bisection no longer separates them), or whose vectors
// degenerate, is left to the QL chase:
// the CTA then writes Q as the plain path does and the chase and
// rotation-replay kernels finish it. The refinement that follows restores
// FP64 accuracy for both.
#pragma once
#include "gla_small.cuh"

namespace gla {

constexpr float kLooseGap = 1e-3f;  // cluster bound (re-orthogonalise inside)
// At or below kTightGap ||T|| (8 ulps of ||T||) leave the matrix to the QL
// chase. Above it the FP32 vectors of a close pair are each off by up to
// ~eps ||T|| / gap inside the pair's invariant subspace, which the
// Gram-Schmidt step and the refinement's Ritz rotation remove; a pair whose
// vectors come out nearly parallel fails the Gram-Schmidt norm test and
// goes to the chase as well.
constexpr float kTightGap = 1e-6f;

// 1/x from the MUFU seed (one rounding; the recurrences tolerate it: a
// relative perturbation of the pivots of a few ulps).
GLA_DEV float rcp_seed(float x) {
  float y;
  asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}

// Guarded pivot (LAPACK dlaebz / dstebz): a pivot smaller than pivmin in
// magnitude is replaced by -pivmin.
GLA_DEV float guard_piv(float q, float pivmin) { return fabsf(q) < pivmin ? -pivmin : q; }

// Numbers of eigenvalues of T below x0, x1, x2 (three interleaved Sturm
// sequences). d: diagonal, e2: squared off-diagonal (shared memory, read
// by every thread at the same index: broadcast).
GLA_DEV void sturm3(int n, const float* __restrict__ d, const float* __restrict__ e2, float x0, float x1, float x2,
                    float pivmin, int& c0, int& c1, int& c2) {
  float q0 = guard_piv(d[0] - x0, pivmin), q1 = guard_piv(d[0] - x1, pivmin), q2 = guard_piv(d[0] - x2, pivmin);
  int a0 = q0 < 0.f, a1 = q1 < 0.f, a2 = q2 < 0.f;
  for (int i = 1; i < n; i++) {
    const float di = d[i], ei = e2[i - 1];
    q0 = guard_piv(fmaf(-ei, rcp_seed(q0), di - x0), pivmin);
    q1 = guard_piv(fmaf(-ei, rcp_seed(q1), di - x1), pivmin);
    q2 = guard_piv(fmaf(-ei, rcp_seed(q2), di - x2), pivmin);
    a0 += q0 < 0.f;
    a1 += q1 < 0.f;
    a2 += q2 < 0.f;
  }
  c0 = a0;
  c1 = a1;
  c2 = a2;
}

// The k-th smallest eigenvalue (0-based) in [lo, hi] by quadsection.
GLA_DEV float eig_bisect(int n, const float* d, const float* e2, int k, float lo, float hi, float atol,
                         float pivmin) {
  for (int it = 0; it < 40 && hi - lo > atol; it++) {
    const float w = hi - lo;
    const float x0 = fmaf(0.25f, w, lo), x1 = fmaf(0.5f, w, lo), x2 = fmaf(0.75f, w, lo);
    int c0, c1, c2;
    sturm3(n, d, e2, x0, x1, x2, pivmin, c0, c1, c2);
    // count(x) > k  <=>  lambda_k < x
    if (c0 > k) {
      hi = x0;
    } else if (c1 > k) {
      lo = x0;
      hi = x1;
    } else if (c2 > k) {
      lo = x1;
      hi = x2;
    } else {
      lo = x2;
    }
  }
  return 0.5f * (lo + hi);
}

// Eigenvector of eigenvalue lam by the twisted factorisation, written to
// column k of Y (Y[i * ldy + k], row i). Returns false when the vector is
// not finite. e: off-diagonal, e2 = e^2.
GLA_DEV bool twisted_vector(int n, const float* __restrict__ d, const float* __restrict__ e,
                            const float* __restrict__ e2, float lam, float pivmin, float* __restrict__ Y, int ldy,
                            int k) {
  float* Yk = Y + k;
  // stationary forward pivots D+_i (stored in Y)
  float dp = guard_piv(d[0] - lam, pivmin);
  Yk[0] = dp;
  for (int i = 0; i + 1 < n; i++) {
    dp = guard_piv(fmaf(-e2[i], rcp_seed(dp), d[i + 1] - lam), pivmin);
    Yk[(size_t)(i + 1) * ldy] = dp;
  }
  // progressive backward pivots D-_i and gamma_i = D+_i + D-_i - (d_i - lam)
  float dm = guard_piv(d[n - 1] - lam, pivmin);
  int r = n - 1;
  float gmin = fabsf(Yk[(size_t)(n - 1) * ldy]);
  for (int i = n - 1; i >= 1; i--) {
    if (i < n - 1) {
      const float g = fabsf(Yk[(size_t)i * ldy] + dm - (d[i] - lam));
      if (g < gmin) {
        gmin = g;
        r = i;
      }
    }
    dm = guard_piv(fmaf(-e2[i - 1], rcp_seed(dm), d[i - 1] - lam), pivmin);
  }
  if (n > 1 && fabsf(dm) < gmin) r = 0;  // gamma_0 = D-_0
  // D-_i for i > r again, stored over D+_i (no longer needed there)
  dm = guard_piv(d[n - 1] - lam, pivmin);
  for (int i = n - 1; i > r; i--) {
    Yk[(size_t)i * ldy] = dm;
    dm = guard_piv(fmaf(-e2[i - 1], rcp_seed(dm), d[i - 1] - lam), pivmin);
  }
  // z_r = 1; z_i = -(e_i / D+_i) z_{i+1} above r, z_{i+1} = -(e_i / D-_{i+1}) z_i below
  Yk[(size_t)r * ldy] = 1.f;
  float z = 1.f, zmax = 1.f;
  for (int i = r - 1; i >= 0; i--) {
    z = -(e[i] * rcp_seed(Yk[(size_t)i * ldy])) * z;
    Yk[(size_t)i * ldy] = z;
    zmax = fmaxf(zmax, fabsf(z));
  }
  z = 1.f;
  for (int i = r; i + 1 < n; i++) {
    z = -(e[i] * rcp_seed(Yk[(size_t)(i + 1) * ldy])) * z;
    Yk[(size_t)(i + 1) * ldy] = z;
    zmax = fmaxf(zmax, fabsf(z));
  }
  if (!(zmax <= 1e30f)) return false;  // also catches NaN
  const float sc = 1.f / zmax;
  float s2 = 0.f;
  for (int i = 0; i < n; i++) {
    const float v = Yk[(size_t)i * ldy] * sc;
    s2 = fmaf(v, v, s2);
  }
  const float nrm = sc * rsqrtf(s2);
  for (int i = 0; i < n; i++) Yk[(size_t)i * ldy] *= nrm;
  return true;
}

// Modified Gram-Schmidt of the columns [c0, c1) of Y (ascending eigenvalue
// order) by one warp; false when a column loses its independence.
GLA_DEV bool mgs_cluster(int n, float* Y, int ldy, int c0, int c1) {
  const int lane = threadIdx.x & 31;
  bool ok = true;
  for (int k = c0 + 1; k < c1; k++) {
    for (int m = c0; m < k; m++) {
      float dot = 0.f;
      for (int i = lane; i < n; i += 32) dot = fmaf(Y[(size_t)i * ldy + m], Y[(size_t)i * ldy + k], dot);
      dot = warp_sum(dot);
      for (int i = lane; i < n; i += 32)
        Y[(size_t)i * ldy + k] = fmaf(-dot, Y[(size_t)i * ldy + m], Y[(size_t)i * ldy + k]);
      __syncwarp();
    }
    float s2 = 0.f;
    for (int i = lane; i < n; i += 32) s2 = fmaf(Y[(size_t)i * ldy + k], Y[(size_t)i * ldy + k], s2);
    s2 = warp_sum(s2);
    if (!(s2 > 0.01f)) ok = false;  // norm below 0.1 after removing the earlier columns
    const float sc = ok ? rsqrtf(s2) : 0.f;
    for (int i = lane; i < n; i += 32) Y[(size_t)i * ldy + k] *= sc;
    __syncwarp();
  }
  return ok;
}

// The whole solver for one matrix, run by every thread of the CTA (blockDim
// >= n): dd, ee the diagonal and off-diagonal, e2s, lams (n floats each),
// Ys (n x ldy), misc (n + 8 ints) and fscr (96 floats) shared scratch.
// Returns (uniformly) true with the ascending eigenvalues in lams and the
// orthonormal eigenvectors in the columns of Ys, or false when the matrix is
// left to the QL chase.
GLA_DEV bool stein_solve(int n, const float* __restrict__ dd, const float* __restrict__ ee, float* __restrict__ e2s,
                         float* __restrict__ lams, float* __restrict__ Ys, int ldy, int* __restrict__ misc,
                         float* __restrict__ fscr) {
  const int tid = threadIdx.x, NT = blockDim.x;
  // Gershgorin interval, ||T|| bound, pivmin (LAPACK dstebz's safeguards)
  float glo = 3.0e38f, ghi = -3.0e38f, e2max = 0.f;
  for (int i = tid; i < n; i += NT) {
    const float ai = (i > 0 ? fabsf(ee[i - 1]) : 0.f) + (i + 1 < n ? fabsf(ee[i]) : 0.f);
    glo = fminf(glo, dd[i] - ai);
    ghi = fmaxf(ghi, dd[i] + ai);
    const float e2 = (i + 1 < n) ? ee[i] * ee[i] : 0.f;
    e2s[i] = e2;
    e2max = fmaxf(e2max, e2);
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    glo = fminf(glo, __shfl_xor_sync(0xffffffffu, glo, o));
    ghi = fmaxf(ghi, __shfl_xor_sync(0xffffffffu, ghi, o));
    e2max = fmaxf(e2max, __shfl_xor_sync(0xffffffffu, e2max, o));
  }
  if ((tid & 31) == 0) {
    fscr[tid >> 5] = glo;
    fscr[32 + (tid >> 5)] = ghi;
    fscr[64 + (tid >> 5)] = e2max;
  }
  if (tid == 0) misc[0] = 0;
  __syncthreads();
  for (int w = 0; w < (NT >> 5); w++) {
    glo = fminf(glo, fscr[w]);
    ghi = fmaxf(ghi, fscr[32 + w]);
    e2max = fmaxf(e2max, fscr[64 + w]);
  }
  const float tnorm = fmaxf(fabsf(glo), fabsf(ghi));
  const float pivmin = 0x1p-100f * fmaxf(1.f, e2max);
  const float widen = 2.f * (float)n * prec<float>::eps * tnorm + 2.f * pivmin;
  glo -= widen;
  ghi += widen;
  const float atol = 2.f * prec<float>::eps * tnorm + 4.f * pivmin;
  if (tid < n) lams[tid] = eig_bisect(n, dd, e2s, tid, glo, ghi, atol, pivmin);
  __syncthreads();
  // strict: a zero gap is tight even when ||T|| = 0
  if (tid + 1 < n && !(lams[tid + 1] - lams[tid] > kTightGap * tnorm)) misc[0] = 1;
  __syncthreads();
  if (misc[0] != 0) return false;
  if (tid < n && !twisted_vector(n, dd, ee, e2s, lams[tid], pivmin, Ys, ldy, tid)) misc[0] = 1;
  if (tid == 0) {  // clusters of two or more eigenvalues within kLooseGap ||T||
    int nc = 0, s0 = 0;
    for (int k = 1; k <= n; k++) {
      if (k == n || lams[k] - lams[k - 1] > kLooseGap * tnorm) {
        if (k - s0 >= 2) {
          misc[2 + 2 * nc] = s0;
          misc[3 + 2 * nc] = k;
          nc++;
        }
        s0 = k;
      }
    }
    misc[1] = nc;
  }
  __syncthreads();
  const int nc = misc[1];
  for (int c = tid >> 5; c < nc; c += NT >> 5)
    if (!mgs_cluster(n, Ys, ldy, misc[2 + 2 * c], misc[3 + 2 * c]) && (tid & 31) == 0) misc[0] = 1;
  __syncthreads();
  return misc[0] == 0;
}

// Shared-memory words the solver needs beyond the tridiagonalisation's own
// arrays: Y (n x ldy floats), e^2 and the eigenvalues (n floats each), and
// n + 8 ints (flags, cluster count, cluster bounds).
__host__ __device__ inline int stein_ldy(int n) { return ((n + 3) & ~3) + 4; }
__host__ __device__ inline size_t stein_extra_words(int n) { return (size_t)n * stein_ldy(n) + 3 * (size_t)n + 8; }

}  // namespace gla
