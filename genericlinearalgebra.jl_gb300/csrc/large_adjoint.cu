// Adjoint of one eigen-decomposition of order above the one-CTA bound:
//
//   Abar = V (diag(wbar) + sym(F o (V' Vbar))) V',   sym(X) = (X + X') / 2,
//   F_ij = 1 / (w_j - w_i) when |w_j - w_i| > gap_rel max|w|, else 0,
//
// the same formula as the batched one-CTA adjoint, as three products on the
// tcgen05 tensor cores (the refinement's Ozaki GEMM, ozaki.cuh: double-float
// accuracy, ~2^-47 relative to the row and column maxima) -- M = V' Vbar,
// Y = V S, Abar = Y V' -- around one FP64 elementwise kernel that turns M
// into S in place. V and Vbar are split into float pairs (hi = x rounded to
// float, lo = x - hi rounded), with a transposed copy of V for the last
// product's right operand. Since F_ji = -F_ij, the symmetric middle factor
// is S_ij = S_ji = F_ij (M_ij - M_ji) / 2 off the diagonal and S_ii =
// wbar_i; one thread owns each pair (i, j), i > j, so the in-place update
// reads M_ij and M_ji before writing either. A bounded wait that ran out in
// a product leaves Abar NaN.
#include <algorithm>
#include <new>

#include "gla_large.h"

namespace gla {

namespace {
// *wmax = max_i |w_i| (one CTA)
__global__ void __launch_bounds__(256) k_adj_wmax(int n, const double* __restrict__ w, double* wmax) {
  __shared__ double red[8];
  double m = 0.0;
  for (int i = threadIdx.x; i < n; i += 256) m = fmax(m, fabs(w[i]));
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) m = fmax(m, __shfl_xor_sync(0xffffffffu, m, o));
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = m;
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int q = 1; q < 8; q++) m = fmax(m, red[q]);
    *wmax = fmax(m, red[0]);
  }
}

__global__ void __launch_bounds__(256) k_adj_middle(int n, const double* __restrict__ w,
                                                    const double* __restrict__ wbar, double* M,
                                                    const double* __restrict__ wmax, double gap_rel) {
  const double thr = gap_rel * *wmax;
  const long long npairs = (long long)n * (n - 1) / 2;
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < npairs + n; t += stride) {
    if (t >= npairs) {  // diagonal
      const int i = (int)(t - npairs);
      M[(long long)i * (n + 1)] = wbar[i];
      continue;
    }
    // pair index t -> (i, j), i > j: row i holds pairs i (i - 1) / 2 .. + i - 1
    int i = (int)((1.0 + sqrt(1.0 + 8.0 * (double)t)) * 0.5);
    while ((long long)i * (i - 1) / 2 > t) i--;
    while ((long long)(i + 1) * i / 2 <= t) i++;
    const int j = (int)(t - (long long)i * (i - 1) / 2);
    const long long ij = (long long)i + (long long)j * n, ji = (long long)j + (long long)i * n;
    const double gap = w[j] - w[i];
    const double f = fabs(gap) > thr ? 1.0 / gap : 0.0;
    const double s = 0.5 * f * (M[ij] - M[ji]);
    M[ij] = s;
    M[ji] = s;
  }
}

// float pair of x: hi = x rounded, lo = (x - hi) rounded (hi + lo = x to ~2^-48)
__global__ void __launch_bounds__(256) k_adj_split(int n, const double* __restrict__ X, long long ldx,
                                                   float* __restrict__ hi, float* __restrict__ lo,
                                                   float* __restrict__ thi, float* __restrict__ tlo) {
  __shared__ float th[32][33], tl[32][33];
  const int i0 = blockIdx.x * 32, j0 = blockIdx.y * 32;
  const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;  // 256 threads: 8 rows of the tile per pass
  for (int jj = ty; jj < 32; jj += 8) {
    const int i = i0 + tx, j = j0 + jj;
    float h = 0.f, l = 0.f;
    if (i < n && j < n) {
      const double x = X[i + (long long)j * ldx];
      h = (float)x;
      l = (float)(x - (double)h);
      hi[i + (long long)j * n] = h;
      lo[i + (long long)j * n] = l;
    }
    th[jj][tx] = h;
    tl[jj][tx] = l;
  }
  if (!thi) return;  // (uniform)
  __syncthreads();
  for (int ii = ty; ii < 32; ii += 8) {  // transposed: element (i, j) to (j, i)
    const int j = j0 + tx, i = i0 + ii;
    if (i < n && j < n) {
      thi[j + (long long)i * n] = th[tx][ii];
      tlo[j + (long long)i * n] = tl[tx][ii];
    }
  }
}

// Out[i, j] = hi + lo (double). sym: only i >= j of the pair is valid and
// is written to (i, j) and (j, i); NaN when a product's bounded wait ran out.
__global__ void __launch_bounds__(256) k_adj_join(int n, const float* __restrict__ hi, const float* __restrict__ lo,
                                                  double* __restrict__ out, long long ldo, bool sym,
                                                  const int* __restrict__ err) {
  const bool bad = err && *err;
  const long long nn = (long long)n * n;
  for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < nn; t += (long long)gridDim.x * blockDim.x) {
    const int i = (int)(t % n), j = (int)(t / n);
    if (sym && i < j) continue;
    const double x = bad ? NAN : (double)hi[t] + (double)lo[t];
    out[i + (long long)j * ldo] = x;
    if (sym) out[j + (long long)i * ldo] = x;
  }
}
}  // namespace

struct LargeAdjoint {
  int nmax = 0;
  OzWork* oz = nullptr;
  float* planes = nullptr;  // Vh Vl Vth Vtl Xh Xl Ch Cl, n^2 floats each
  double* M = nullptr;      // n^2 doubles, then max|w|
};

int large_adjoint_create(LargeAdjoint** out, int nmax) {
  *out = nullptr;
  LargeAdjoint* a = new (std::nothrow) LargeAdjoint();
  if (!a) return -1000 - (int)cudaErrorMemoryAllocation;
  a->nmax = nmax;
  const size_t nn = (size_t)nmax * nmax;
  int rc = oz_create(&a->oz, nmax, nmax, nmax);
  cudaError_t e = rc ? cudaErrorMemoryAllocation : cudaMalloc((void**)&a->planes, 8 * nn * sizeof(float));
  if (e == cudaSuccess) e = cudaMalloc((void**)&a->M, (nn + 1) * sizeof(double));
  if (rc || e != cudaSuccess) {
    large_adjoint_destroy(a);
    return rc ? rc : -1000 - (int)e;
  }
  *out = a;
  return 0;
}

void large_adjoint_destroy(LargeAdjoint* a) {
  if (!a) return;
  oz_destroy(a->oz);
  cudaFree(a->planes);
  cudaFree(a->M);
  delete a;
}

cudaError_t large_adjoint(LargeAdjoint* a, int n, const double* w, const double* V, long long ldv,
                          const double* wbar, const double* Vbar, long long ldvb, double* Abar, long long lda,
                          double gap_rel, cudaStream_t st) {
  if (n <= 0) return cudaSuccess;
  if (n > a->nmax) return cudaErrorInvalidValue;
  const size_t nn = (size_t)n * n;
  float* Vh = a->planes;
  float* Vl = Vh + nn;
  float* Vth = Vl + nn;
  float* Vtl = Vth + nn;
  float* Xh = Vtl + nn;
  float* Xl = Xh + nn;
  float* Ch = Xl + nn;
  float* Cl = Ch + nn;
  double* M = a->M;
  constexpr int S = 7;
  const dim3 tiles((n + 31) / 32, (n + 31) / 32);
  k_adj_split<<<tiles, 256, 0, st>>>(n, V, ldv, Vh, Vl, Vth, Vtl);
  k_adj_split<<<tiles, 256, 0, st>>>(n, Vbar, ldvb, Xh, Xl, nullptr, nullptr);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  // M = V' Vbar: the left operand's rows are V's columns
  if ((e = oz_slice(a->oz, true, Vh, Vl, n, n, n, S, st)) != cudaSuccess) return e;
  if ((e = oz_slice(a->oz, false, Xh, Xl, n, n, n, S, st)) != cudaSuccess) return e;
  if ((e = oz_gemm(a->oz, n, n, n, Ch, Cl, n, false, st)) != cudaSuccess) return e;
  const int jb = (int)std::min<long long>(((long long)nn + 255) / 256, 152 * 8);
  k_adj_join<<<jb, 256, 0, st>>>(n, Ch, Cl, M, n, false, nullptr);
  double* wmax = M + nn;
  k_adj_wmax<<<1, 256, 0, st>>>(n, w, wmax);
  const long long work = (long long)n * (n + 1) / 2;
  const int blocks = (int)std::min<long long>((work + 255) / 256, 152 * 8);
  k_adj_middle<<<blocks, 256, 0, st>>>(n, w, wbar, M, wmax, gap_rel);
  k_adj_split<<<tiles, 256, 0, st>>>(n, M, n, Xh, Xl, nullptr, nullptr);
  if ((e = cudaGetLastError()) != cudaSuccess) return e;
  // Y = V S: the left operand's rows are V's rows
  if ((e = oz_slice_rows(a->oz, Vh, Vl, n, n, n, S, st)) != cudaSuccess) return e;
  if ((e = oz_slice(a->oz, false, Xh, Xl, n, n, n, S, st)) != cudaSuccess) return e;
  if ((e = oz_gemm(a->oz, n, n, n, Ch, Cl, n, false, st)) != cudaSuccess) return e;
  // Abar = Y V' (symmetric: the lower triangle, mirrored): the right
  // operand's columns are V's rows (the transposed copy)
  if ((e = oz_slice_rows(a->oz, Ch, Cl, n, n, n, S, st)) != cudaSuccess) return e;
  if ((e = oz_slice(a->oz, false, Vth, Vtl, n, n, n, S, st)) != cudaSuccess) return e;
  if ((e = oz_gemm(a->oz, n, n, n, Xh, Xl, n, true, st)) != cudaSuccess) return e;
  k_adj_join<<<jb, 256, 0, st>>>(n, Xh, Xl, Abar, lda, true, oz_error_word(a->oz));
  return cudaGetLastError();
}

}  // namespace gla
