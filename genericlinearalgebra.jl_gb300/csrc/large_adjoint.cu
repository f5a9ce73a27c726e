// Adjoint of one eigen-decomposition of order above the one-CTA bound:
//
//   Abar = V (diag(wbar) + sym(F o (V' Vbar))) V',   sym(X) = (X + X') / 2,
//   F_ij = 1 / (w_j - w_i) when |w_j - w_i| > gap_rel max|w|, else 0,
//
// the same formula as the batched one-CTA adjoint, as three FP64 GEMMs on the
// SIMT GEMM (M = V' Vbar, Y = V S, Abar = Y V') around one elementwise
// kernel that turns M into S in place. Since F_ji = -F_ij, the symmetric
// middle factor is S_ij = S_ji = F_ij (M_ij - M_ji) / 2 off the diagonal and
// S_ii = wbar_i; one thread owns each pair (i, j), i > j, so the in-place
// update reads M_ij and M_ji before writing either.
#include <algorithm>

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
}  // namespace

size_t large_adjoint_workspace_elems(int n) { return 2 * (size_t)n * n + 1; }

cudaError_t large_adjoint(int n, const double* w, const double* V, long long ldv, const double* wbar,
                          const double* Vbar, long long ldvb, double* Abar, long long lda, double gap_rel,
                          double* ws, cudaStream_t st) {
  if (n <= 0) return cudaSuccess;
  double* M = ws;
  double* Y = ws + (size_t)n * n;
  GemmDesc g{};
  g.m = g.n = g.k = n;
  g.alpha = 1.0;
  g.beta = 0.0;
  // M = V' Vbar
  g.A = V;
  g.lda = ldv;
  g.B = Vbar;
  g.ldb = ldvb;
  g.C = M;
  g.ldc = n;
  cudaError_t e = gemm_launch(true, true, false, false, g, 1, st);
  if (e != cudaSuccess) return e;
  double* wmax = ws + 2 * (size_t)n * n;
  k_adj_wmax<<<1, 256, 0, st>>>(n, w, wmax);
  const long long work = (long long)n * (n + 1) / 2;
  const int blocks = (int)std::min<long long>((work + 255) / 256, 152 * 8);
  k_adj_middle<<<blocks, 256, 0, st>>>(n, w, wbar, M, wmax, gap_rel);
  if ((e = cudaGetLastError()) != cudaSuccess) return e;
  // Y = V S
  g.A = V;
  g.lda = ldv;
  g.B = M;
  g.ldb = n;
  g.C = Y;
  g.ldc = n;
  if ((e = gemm_launch(true, false, false, false, g, 1, st)) != cudaSuccess) return e;
  // Abar = Y V'
  g.A = Y;
  g.lda = n;
  g.B = V;
  g.ldb = ldv;
  g.C = Abar;
  g.ldc = lda;
  return gemm_launch(true, false, true, false, g, 1, st);
}

}  // namespace gla
