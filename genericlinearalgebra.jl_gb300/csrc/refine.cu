// Ogita-Aishima refinement (T. Ogita, K. Aishima, "Iterative refinement for
// symmetric eigenvalue decomposition", Japan J. Indust. Appl. Math. 35
// (2018), Algorithm 1) of the FP32 eigenvectors, one CTA per matrix:
//
//   R = I - X'X,  S = X'AX,  lam_i = s_ii / (1 - r_ii),
//   delta = 2 (||S - diag(lam)|| + ||A|| ||R||)          (Frobenius bounds)
//   E_ij = (s_ij + lam_j r_ij) / (lam_j - lam_i)  if |lam_i - lam_j| > delta
//        = r_ij / 2                               otherwise (and on i == j)
//   X <- X + X E
//
// repeated until max|E| < 2^-30 (the last correction is then below FP64
// rounding of the result) or kMaxRefineIters. Products are FP64. The result
// is sorted ascending (sorteig!, as the reference returns it).
// No counterpart in GenericLinearAlgebra.jl.
#include "gla_refine.h"

namespace gla {

constexpr int kMaxRefineIters = 6;
constexpr int kRT = 256;  // threads per CTA

size_t refine_workspace_bytes(int64_t a_elems, int64_t, int64_t) { return 4 * sizeof(double) * (size_t)a_elems + 1024; }

void refine_carve(RefineWork* rw, char* base, int64_t a_elems, int64_t, int64_t) {
  double* p = reinterpret_cast<double*>(base);
  rw->X = p;
  rw->Y = p + a_elems;
  rw->S = p + 2 * a_elems;
  rw->R = p + 3 * a_elems;
}

// C(i, j) = sum_k la(i, k) * lb(k, j) over 64 x 64 output tiles; 256 threads,
// 4 x 4 outputs per thread; `upper` skips tiles strictly below the diagonal.
template <class LA, class LB, class ST>
GLA_DEV void tile_gemm(int n, const LA& la, const LB& lb, const ST& store, double* As, double* Bs, bool upper) {
  const int tid = threadIdx.x, tx = tid & 15, ty = tid >> 4;
  for (int i0 = 0; i0 < n; i0 += 64) {
    for (int j0 = 0; j0 < n; j0 += 64) {
      if (upper && j0 + 63 < i0) continue;
      double acc[4][4];
#pragma unroll
      for (int u = 0; u < 4; u++)
#pragma unroll
        for (int v = 0; v < 4; v++) acc[u][v] = 0;
      for (int k0 = 0; k0 < n; k0 += 16) {
        __syncthreads();
        for (int t = tid; t < 16 * 64; t += kRT) {
          const int kk = t & 15, ii = t >> 4;
          const int i = i0 + ii, k = k0 + kk;
          As[kk * 64 + ii] = (i < n && k < n) ? la(i, k) : 0.0;
          const int j = j0 + ii;
          Bs[kk * 64 + ii] = (j < n && k < n) ? lb(k, j) : 0.0;
        }
        __syncthreads();
#pragma unroll 4
        for (int kk = 0; kk < 16; kk++) {
          double a[4], b[4];
#pragma unroll
          for (int u = 0; u < 4; u++) a[u] = As[kk * 64 + tx + 16 * u];
#pragma unroll
          for (int v = 0; v < 4; v++) b[v] = Bs[kk * 64 + ty + 16 * v];
#pragma unroll
          for (int u = 0; u < 4; u++)
#pragma unroll
            for (int v = 0; v < 4; v++) acc[u][v] = fma(a[u], b[v], acc[u][v]);
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

GLA_DEV double block_sum_d(double v, double* red) {
  v = warp_sum(v);
  __syncthreads();
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
  __syncthreads();
  double s = 0;
  for (int i = 0; i < kRT / 32; i++) s += red[i];
  return s;
}

GLA_DEV double block_max_d(double v, double* red) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
  __syncthreads();
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
  __syncthreads();
  double s = 0;
  for (int i = 0; i < kRT / 32; i++) s = fmax(s, red[i]);
  return s;
}

__global__ void __launch_bounds__(kRT) k_refine(const SmallDesc* __restrict__ descs, const int* __restrict__ perm,
                                                const double* __restrict__ A, int lower,
                                                const float* __restrict__ X32, const float* __restrict__ w32,
                                                double* __restrict__ Vout, double* __restrict__ wout,
                                                const int* __restrict__ info, RefineWork rw,
                                                unsigned long long* __restrict__ stats) {
  __shared__ double As[16 * 64], Bs[16 * 64];
  __shared__ double lam[kSmallMaxN];
  __shared__ double red[kRT / 32];
  __shared__ unsigned long long keys[kSmallMaxN];
  __shared__ int rank[kSmallMaxN];
  const int mid = perm[blockIdx.x];
  const SmallDesc dsc = descs[mid];
  const int n = dsc.n, tid = threadIdx.x;
  const size_t ao = dsc.a_off;
  const double* Ag = A + ao;
  double* V = Vout ? Vout + ao : nullptr;
  if (info[mid] == -1) {
    for (int idx = tid; idx < n * n; idx += kRT)
      if (V) V[idx] = NAN;
    for (int i = tid; i < n; i += kRT) wout[dsc.w_off + i] = NAN;
    return;
  }
  double* X = rw.X + ao;
  double* Y = rw.Y + ao;
  double* S = rw.S + ao;
  double* R = rw.R + ao;
  for (int idx = tid; idx < n * n; idx += kRT) X[idx] = (double)X32[ao + idx];
  double anorm2 = 0;
  for (int idx = tid; idx < n * n; idx += kRT) {
    const int i = idx % n, k = idx / n;
    const double a = (lower ? (i >= k) : (i <= k)) ? Ag[idx] : Ag[(size_t)i * n + k];
    anorm2 = fma(a, a, anorm2);
  }
  const double anorm = sqrt(block_sum_d(anorm2, red));
  auto Asym = [&](int i, int k) -> double {
    return (lower ? (i >= k) : (i <= k)) ? Ag[(size_t)k * n + i] : Ag[(size_t)i * n + k];
  };
  __syncthreads();
  for (int it = 0; it < kMaxRefineIters; it++) {
    // Y = A X
    tile_gemm(
        n, Asym, [&](int k, int j) { return X[(size_t)j * n + k]; },
        [&](int i, int j, double v) { Y[(size_t)j * n + i] = v; }, As, Bs, false);
    // S = X'Y, R = I - X'X (upper triangles, mirrored)
    tile_gemm(
        n, [&](int i, int k) { return X[(size_t)i * n + k]; }, [&](int k, int j) { return Y[(size_t)j * n + k]; },
        [&](int i, int j, double v) {
          S[(size_t)j * n + i] = v;
          S[(size_t)i * n + j] = v;
        },
        As, Bs, true);
    tile_gemm(
        n, [&](int i, int k) { return X[(size_t)i * n + k]; }, [&](int k, int j) { return X[(size_t)j * n + k]; },
        [&](int i, int j, double v) {
          const double r = (i == j ? 1.0 : 0.0) - v;
          R[(size_t)j * n + i] = r;
          R[(size_t)i * n + j] = r;
        },
        As, Bs, true);
    for (int i = tid; i < n; i += kRT) lam[i] = S[(size_t)i * n + i] / (1.0 - R[(size_t)i * n + i]);
    __syncthreads();
    double sd2 = 0, r2 = 0;
    for (int idx = tid; idx < n * n; idx += kRT) {
      const int i = idx % n, j = idx / n;
      const double sv = S[idx] - (i == j ? lam[i] : 0.0);
      sd2 = fma(sv, sv, sd2);
      r2 = fma(R[idx], R[idx], r2);
    }
    const double sdn = sqrt(block_sum_d(sd2, red));
    const double rn = sqrt(block_sum_d(r2, red));
    const double delta = 2.0 * (sdn + anorm * rn);
    double emax = 0;
    for (int idx = tid; idx < n * n; idx += kRT) {
      const int i = idx % n, j = idx / n;
      const double dl = lam[j] - lam[i];
      double e;
      if (i != j && fabs(dl) > delta) e = (S[idx] + lam[j] * R[idx]) / dl;
      else e = 0.5 * R[idx];
      emax = fmax(emax, fabs(e));
      S[idx] = e;  // E replaces S
    }
    emax = block_max_d(emax, red);
    // X <- X + X E
    tile_gemm(
        n, [&](int i, int k) { return X[(size_t)k * n + i]; }, [&](int k, int j) { return S[(size_t)j * n + k]; },
        [&](int i, int j, double v) { Y[(size_t)j * n + i] = X[(size_t)j * n + i] + v; }, As, Bs, false);
    double* t = X;
    X = Y;
    Y = t;
    if (tid == 0) atomicAdd(&stats[3], (unsigned long long)n * n * n);
    if (emax < 0x1p-30) break;
  }
  // sorteig!: ascending eigenvalues, columns permuted to match
  for (int i = tid; i < n; i += kRT) keys[i] = sort_key(lam[i]);
  __syncthreads();
  for (int i = tid; i < n; i += kRT) {
    const unsigned long long ki = keys[i];
    int rk = 0;
    for (int j = 0; j < n; j++) rk += (keys[j] < ki) || (keys[j] == ki && j < i);
    rank[i] = rk;
    wout[dsc.w_off + rk] = lam[i];
  }
  __syncthreads();
  if (V)
    for (int j = 0; j < n; j++) {
      const int dst = rank[j];
      for (int i = tid; i < n; i += kRT) V[(size_t)dst * n + i] = X[(size_t)j * n + i];
    }
}

cudaError_t refine_kernels_init() { return cudaSuccess; }

cudaError_t launch_refine(const RefineWork* rw, int nblocks, int nmax, cudaStream_t st, const SmallDesc* descs,
                          const int* perm, const double* A, int lower, const float* X32, const float* w32,
                          double* V, double* w, const int* info, unsigned long long* stats) {
  (void)nmax;
  if (nblocks <= 0) return cudaSuccess;
  k_refine<<<nblocks, kRT, 0, st>>>(descs, perm, A, lower, X32, w32, V, w, info, *rw, stats);
  return cudaGetLastError();
}

}  // namespace gla
