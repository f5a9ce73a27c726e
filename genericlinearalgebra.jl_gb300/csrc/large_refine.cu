// Ogita-Aishima refinement of FP32 eigenpairs of one large matrix back to
// FP64-class accuracy (no counterpart in GenericLinearAlgebra.jl; the
// reference computes in the input precision throughout).
//
// Iteration on X (double-float columns, ascending lam), with A scaled by an
// exact power of two:
//   P    = A X                              tcgen05 Ozaki GEMM (ozaki.cuh)
//   lam  = diag(X'P) / diag(X'X)            double-float column dots
//   Rres = P - X diag(lam)                  double-float, rounded to FP32
//   T    = X_hi' Rres                       FP32-accuracy tensor-core GEMM
// With R = I - X'X and S = X'AX = (I - R) diag(lam) + T, the Ogita-Aishima
// numerator s_ij + lam_j r_ij equals t_ij for i != j, so
//   E_ij = t_ij / (lam_j - lam_i)          separated pairs
//   E_ii = (1 - (X'X)_ii) / 2
//   E_ij = -(X'X)_ij / 2                   pairs inside one cluster
//   X   <- X + X_hi E                       FP32-accuracy tensor-core GEMM,
//                                           added in double-float
// (T. Ogita, K. Aishima, JJIAM 35 (2018) Alg. 1, rewritten on the residual;
// t_ij - t_ji = r_ij (lam_j - lam_i) carries the orthogonality correction of
// separated pairs, so X'X is only formed when clusters need it and in the
// final polishing iteration, by the same tensor-core GEMM).
// Clusters are runs of the sorted lam joined wherever a gap is below ten
// times the residual norms of its two columns, some pair (i, j) with
// |i - j| <= kWin has |t_ij| > kTheta |lam_j - lam_i| (the first-order update
// would not be small), or the gap is at rounding level. Each cluster J is
// rotated to the Ritz vectors of its projected matrix, which to first order is
//   C_J = diag(lam_J - mu) + (T_JJ + T_JJ') / 2     (mu the cluster mean)
// (JJIAM 36 (2019)); C_J is solved in FP32 by this library's own solvers
// (batched small path up to 128, large path above) and X_J <- X_J W_J in
// double-float, which keeps the span of X_J exact (columns are re-sorted
// afterwards when an update moved an eigenvalue past a neighbour); a cluster whose C_J is
// already diagonal to 1e-15 ||A|| is not rotated (an FP32 rotation would
// bring back 1e-7 non-orthogonality). When nothing was rotated and the
// corrections are below 2e-7 (or at their rounding floor), one last
// "polishing" iteration forms the full double-float Gram matrix and uses the
// symmetric form E = R/2 + sym(T)/(lam_j - lam_i): the residual form
// recovers r_ij only to ~u ||A|| / gap_ij, the symmetric form to u. The
// polish forms X E in double-float on the tensor cores and skips rotations
// that are rounding noise at tight gaps; when the orthogonality defect it
// started from exceeded 1e-7 (tight clusters rotated shortly before), one
// more symmetric step X <- X (I + R/2) squares the remaining ~d^2 away.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <map>
#include <new>
#include <vector>

#include "../../include/glagpu.h"
#include "df64.cuh"
#include "gla_large.h"
#include "gla_launch.h"

namespace gla {

constexpr int kRefMaxIters = 10;
constexpr int kWin = 32;
constexpr int kOzRotateMin = 64;  // cluster rotations of at least this many columns on the tensor cores
constexpr float kTheta = 0.05f;
constexpr double kResTheta = 0.1;

struct RefineLarge {
  int n = 0;
  float *Ahi = nullptr, *Alo = nullptr, *Xhi = nullptr, *Xlo = nullptr, *Phi = nullptr, *Plo = nullptr;
  float *Rres = nullptr, *T = nullptr, *E = nullptr, *XE = nullptr, *Ghi = nullptr, *Glo = nullptr;
  float* Cbuf = nullptr;   // cluster matrices, packed
  float* Wbuf = nullptr;   // their eigenvectors
  float* nubuf = nullptr;  // their eigenvalues
  double* lam = nullptr;
  double* gdiag = nullptr;
  int* couple = nullptr;   // per consecutive pair: joined into one cluster
  int* cid = nullptr;      // per column: cluster id (or -1)
  float* scal = nullptr;   // [0] max |E| outside clusters, [1] orthogonality defect entering the
                           // polish, [2] max column norm of Rres (float bits)
  float* offmax = nullptr; // per cluster: max |off-diagonal| of C_J
  float* rn = nullptr;     // per column: residual norm
  unsigned long long* amax = nullptr;
  int* flags = nullptr;    // [0] non-finite, [1] scale exponent
  int* cinfo = nullptr;
  std::map<int, LargeCtx*> big;  // FP32 solvers for clusters above the small limit
  OzWork* oz = nullptr;          // tcgen05 double-float GEMM: A slices (A operand), X slices (B operand)
  OzWork* ozx = nullptr;         // X slices as the A operand (the Gram matrix X'X)
  OzWork* oz32 = nullptr;        // tcgen05 FP32-accuracy GEMM: T = X_hi' Rres and X_hi E
  std::vector<double> h_lam;
  std::vector<int> h_couple;
  int iters = 0;
  int rotated = 0;  // cluster rotations of the last run
  int reorders = 0;
  int ortho_steps = 0;  // extra orthogonalisation steps after the polish
};

namespace {

__global__ void k_ref_maxabs(const double* __restrict__ A, long long lda, int n, bool lower,
                             unsigned long long* amax, int* nonfinite) {
  unsigned long long m = 0;
  int bad = 0;
  const int j = blockIdx.y;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    if (lower ? i < j : i > j) continue;
    const double x = A[i + (long long)j * lda];
    if (!isfinite(x)) bad = 1;
    else m = max(m, (unsigned long long)__double_as_longlong(fabs(x)));
  }
#pragma unroll
  for (int s = 16; s > 0; s >>= 1) {
    m = max(m, __shfl_xor_sync(0xffffffffu, m, s));
    bad |= __shfl_xor_sync(0xffffffffu, bad, s);
  }
  if ((threadIdx.x & 31) == 0) {
    if (m) atomicMax(amax, m);
    if (bad) atomicExch(nonfinite, 1);
  }
}

// Full symmetric A * 2^-e as (hi, lo) floats; X from the FP32 solve; lam scaled.
__global__ void k_ref_load(const double* __restrict__ A, long long lda, int n, bool lower,
                           const unsigned long long* amax, int* flags, float* __restrict__ Ahi,
                           float* __restrict__ Alo, const float* __restrict__ X32, long long ldx,
                           float* __restrict__ Xhi, float* __restrict__ Xlo, const float* __restrict__ w32,
                           double* __restrict__ lam) {
  const double am = __longlong_as_double((long long)*amax);
  const int ex = am > 0.0 ? ilogb(am) : 0;
  if (blockIdx.x == 0 && blockIdx.y == 0 && threadIdx.x == 0) flags[1] = ex;
  const double sc = ldexp(1.0, -ex);
  const int j = blockIdx.y;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const bool in = lower ? i >= j : i <= j;
    const double a = (in ? A[i + (long long)j * lda] : A[j + (long long)i * lda]) * sc;
    const float h = (float)a;
    const long long idx = i + (long long)j * n;
    Ahi[idx] = h;
    Alo[idx] = (float)(a - (double)h);
    Xhi[idx] = X32[i + (long long)j * ldx];
    Xlo[idx] = 0.f;
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) lam[j] = (double)w32[j] * sc;
}

// Column statistics (one warp per column): x'x and x'p in double-float.
__global__ void k_ref_colstats(const float* __restrict__ Xhi, const float* __restrict__ Xlo,
                               const float* __restrict__ Phi, const float* __restrict__ Plo, int n,
                               double* __restrict__ lam, double* __restrict__ gdiag) {
  const int j = blockIdx.x * (blockDim.x / 32) + (threadIdx.x >> 5), lane = threadIdx.x & 31;
  if (j >= n) return;
  df64 g = df_make(0.f, 0.f), s = df_make(0.f, 0.f);
  const long long o = (long long)j * n;
  for (int r = lane; r < n; r += 32) {
    const df64 x = df_make(Xhi[o + r], Xlo[o + r]);
    const df64 p = df_make(Phi[o + r], Plo[o + r]);
    g = df_mac(g, x, x);
    s = df_mac(s, x, p);
  }
  double gd = df_to(g), sd = df_to(s);
#pragma unroll
  for (int k = 16; k > 0; k >>= 1) {
    gd += __shfl_xor_sync(0xffffffffu, gd, k);
    sd += __shfl_xor_sync(0xffffffffu, sd, k);
  }
  if (lane == 0) {
    lam[j] = sd / gd;
    gdiag[j] = gd;
  }
}

// Rres = P - X diag(lam), double-float, rounded to FP32; column norms into
// rn[j] (residual norms) and their maximum into *rmax.
__global__ void k_ref_rres(const float* __restrict__ Xhi, const float* __restrict__ Xlo,
                           const float* __restrict__ Phi, const float* __restrict__ Plo,
                           const double* __restrict__ lam, int n, float* __restrict__ R, float* __restrict__ rn,
                           float* rmax) {
  const int j = blockIdx.x;
  const df64 l = df_from(-lam[j]);
  float ss = 0.f;
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    const long long idx = i + (long long)j * n;
    const df64 r = df_mac(df_make(Phi[idx], Plo[idx]), df_make(Xhi[idx], Xlo[idx]), l);
    const float v = r.hi + r.lo;
    R[idx] = v;
    ss = fmaf(v, v, ss);
  }
  __shared__ float red[8];
#pragma unroll
  for (int s = 16; s > 0; s >>= 1) ss += __shfl_xor_sync(0xffffffffu, ss, s);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = ss;
  __syncthreads();
  if (threadIdx.x == 0) {
    float t = 0.f;
    for (int w = 0; w < (int)(blockDim.x / 32); w++) t += red[w];
    rn[j] = sqrtf(t);
    atomicMax(reinterpret_cast<int*>(rmax), __float_as_int(sqrtf(t)));
  }
}

// couple[p] = 1 joins sorted columns p and p+1 into one cluster: the gap is
// below kResTheta^-1 times their residual norms (an eigenvector error bound
// of the Davis-Kahan kind would then not be small), some pair (i, j) across
// p with |i - j| <= kWin has |t_ij| > kTheta |lam_j - lam_i|, or the gap is
// at rounding level.
__global__ void k_ref_couple(const float* __restrict__ T, const double* __restrict__ lam,
                             const float* __restrict__ rn, int n, int* __restrict__ couple) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= n - 1) return;
  const double lmax = fmax(fabs(lam[0]), fabs(lam[n - 1]));
  const double gp = fabs(lam[p + 1] - lam[p]);
  int c = gp <= 64.0 * 0x1p-52 * lmax || gp * kResTheta <= (double)fmaxf(rn[p], rn[p + 1]);
  for (int i = max(0, p - kWin + 1); i <= p && !c; i++)
    for (int j = p + 1; j <= min(n - 1, i + kWin) && !c; j++) {
      const float gap = (float)fabs(lam[j] - lam[i]);
      const float t = fmaxf(fabsf(T[i + (long long)j * n]), fabsf(T[j + (long long)i * n]));
      c = t > kTheta * gap;
    }
  couple[p] = c;
}

// dst[:, j] = src[:, perm[j]] (n x n, leading dimension n).
__global__ void k_ref_gather(const float* __restrict__ src, float* __restrict__ dst, const int* __restrict__ perm,
                             int n) {
  const int j = blockIdx.y;
  const long long s0 = (long long)perm[j] * n, d0 = (long long)j * n;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) dst[d0 + i] = src[s0 + i];
}

__device__ __forceinline__ void atomic_max_pos(float* a, float v) {
  atomicMax(reinterpret_cast<int*>(a), __float_as_int(v));  // v >= 0
}

// The correction E (FP32); max |E_ij| over separated pairs into scal[0].
// polish: the full Gram matrix X'X (lower triangle in G) is available and
// separated pairs take the symmetric Ogita-Aishima form
// E_ij = r_ij / 2 + (t_ij + t_ji) / (2 (lam_j - lam_i)), r = I - X'X, whose
// E + E' = R holds whatever the rounding of T.
__global__ void k_ref_e(const float* __restrict__ T, const float* __restrict__ Ghi, const float* __restrict__ Glo,
                        const double* __restrict__ lam, const double* __restrict__ gdiag,
                        const int* __restrict__ cid, int n, int polish, double tfloor, float* __restrict__ E,
                        float* scal) {
  const int j = blockIdx.y;
  float em = 0.f, od = 0.f;
  const double lj = lam[j];
  const int cj = cid[j];
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const long long idx = i + (long long)j * n;
    const long long g = i > j ? idx : j + (long long)i * n;  // lower triangle of the Gram matrix
    float e;
    if (polish) od = fmaxf(od, i == j ? (float)fabs(1.0 - gdiag[j]) : fabsf(Ghi[g]));
    if (i == j) {
      e = (float)(0.5 * (1.0 - gdiag[j]));
    } else if (cj >= 0 && cid[i] == cj) {
      e = -0.5f * (Ghi[g] + Glo[g]);
    } else {
      const double gap = lj - lam[i];
      float sep;
      if (polish) {
        // polishing iteration: a pair at a tight gap whose coupling is at
        // the rounding floor of T is not rotated: the rotation would be
        // noise of size u ||A|| / gap (its square shows in the
        // orthogonality) and leaving it changes the residual by less than
        // tfloor; rotations below 1e-8 cost nothing in orthogonality and are
        // kept (they carry the residual's last bits)
        const double t = 0.5 * ((double)T[idx] + (double)T[j + (long long)i * n]);
        const double rot = t / gap;
        sep = (fabs(t) <= tfloor && fabs(rot) > 1e-8) ? 0.f : (float)rot;
      } else {
        sep = (float)((double)T[idx] / gap);
      }
      em = fmaxf(em, fabsf(sep));
      e = polish ? sep - 0.5f * (Ghi[g] + Glo[g]) : sep;
    }
    E[idx] = e;
  }
#pragma unroll
  for (int s = 16; s > 0; s >>= 1) {
    em = fmaxf(em, __shfl_xor_sync(0xffffffffu, em, s));
    od = fmaxf(od, __shfl_xor_sync(0xffffffffu, od, s));
  }
  if ((threadIdx.x & 31) == 0) {
    atomic_max_pos(scal, em);
    if (polish) atomic_max_pos(scal + 1, od);
  }
}

// Symmetric orthogonalisation step X <- X (I + R/2), R = I - X'X (one
// Newton-Schulz step towards the orthonormal polar factor): E from the
// lower triangle of the Gram matrix.
__global__ void k_ref_ortho_e(const float* __restrict__ Ghi, const float* __restrict__ Glo, int n,
                              float* __restrict__ E) {
  const int j = blockIdx.y;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const long long idx = i + (long long)j * n;
    const long long g = i >= j ? idx : j + (long long)i * n;
    const double gv = (double)Ghi[g] + (double)Glo[g];
    E[idx] = (float)(i == j ? 0.5 * (1.0 - gv) : -0.5 * gv);
  }
}

// X <- X + XE in double-float.
__global__ void k_ref_update(float* __restrict__ Xhi, float* __restrict__ Xlo, const float* __restrict__ XE,
                             long long count) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < count;
       i += (long long)gridDim.x * blockDim.x) {
    const df64 x = df_add(df_make(Xhi[i], Xlo[i]), df_make(XE[i], 0.f));
    Xhi[i] = x.hi;
    Xlo[i] = x.lo;
  }
}

// X <- X + (XE as a float pair) in double-float.
__global__ void k_ref_update_df(float* __restrict__ Xhi, float* __restrict__ Xlo, const float* __restrict__ Phi,
                                const float* __restrict__ Plo, long long count) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < count;
       i += (long long)gridDim.x * blockDim.x) {
    const df64 x = df_add(df_make(Xhi[i], Xlo[i]), df_make(Phi[i], Plo[i]));
    Xhi[i] = x.hi;
    Xlo[i] = x.lo;
  }
}

// Cluster matrix C_J (c x c, packed at off): diag(lam - mu) + sym(T_JJ);
// max |off-diagonal| into *offmax.
__global__ void k_ref_cmat(const float* __restrict__ T, const double* __restrict__ lam, int n, int j0, int c,
                           double mu, float* __restrict__ C, float* offmax) {
  float om = 0.f;
  for (int idx = blockIdx.x * blockDim.x + threadIdx.x; idx < c * c; idx += gridDim.x * blockDim.x) {
    const int a = idx % c, b = idx / c;
    const int i = j0 + a, j = j0 + b;
    float v = 0.5f * (T[i + (long long)j * n] + T[j + (long long)i * n]);
    if (a == b)
      v += (float)(lam[i] - mu);
    else
      om = fmaxf(om, fabsf(v));
    C[idx] = v;
  }
#pragma unroll
  for (int s = 16; s > 0; s >>= 1) om = fmaxf(om, __shfl_xor_sync(0xffffffffu, om, s));
  if ((threadIdx.x & 31) == 0) atomic_max_pos(offmax, om);
}

__global__ void k_ref_setlam(double* __restrict__ lam, int j0, int c, double mu, const float* __restrict__ nu) {
  const int a = blockIdx.x * blockDim.x + threadIdx.x;
  if (a < c) lam[j0 + a] = mu + (double)nu[a];
}

// Outputs: V (FP64) and w (unscaled); NaN for non-finite input.
__global__ void k_ref_store(const float* __restrict__ Xhi, const float* __restrict__ Xlo,
                            const double* __restrict__ lam, const int* __restrict__ perm, int n,
                            const int* __restrict__ flags, double* __restrict__ w, double* __restrict__ V,
                            long long ldv) {
  const int j = blockIdx.y;
  const int src = perm ? perm[j] : j;
  const bool bad = flags[0] != 0;
  if (blockIdx.x == 0 && threadIdx.x == 0) w[j] = bad ? NAN : ldexp(lam[src], flags[1]);
  if (!V) return;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const long long s = i + (long long)src * n;
    V[i + (long long)j * ldv] = bad ? NAN : (double)Xhi[s] + (double)Xlo[s];
  }
}

#define RF_CUDA(x)                                   \
  do {                                               \
    cudaError_t e_ = (x);                            \
    if (e_ != cudaSuccess) return -1000 - (int)e_;   \
  } while (0)

}  // namespace

int refine_large_create(RefineLarge** out, int n) {
  *out = nullptr;
  RefineLarge* r = new (std::nothrow) RefineLarge();
  if (!r) return -1000 - (int)cudaErrorMemoryAllocation;
  r->n = n;
  const size_t nn = (size_t)n * n;
  cudaError_t err = cudaSuccess;
  auto alloc = [&](void** p, size_t bytes) {
    if (err == cudaSuccess) err = cudaMalloc(p, std::max<size_t>(bytes, 16));
  };
  float** bufs[] = {&r->Ahi, &r->Alo, &r->Xhi, &r->Xlo, &r->Phi, &r->Plo, &r->Rres, &r->T, &r->E, &r->XE, &r->Ghi,
                    &r->Glo, &r->Cbuf, &r->Wbuf};
  for (float** b : bufs) alloc((void**)b, sizeof(float) * nn);
  alloc((void**)&r->nubuf, sizeof(float) * n);
  alloc((void**)&r->lam, sizeof(double) * n);
  alloc((void**)&r->gdiag, sizeof(double) * n);
  alloc((void**)&r->couple, sizeof(int) * n);
  alloc((void**)&r->cid, sizeof(int) * n);
  alloc((void**)&r->scal, sizeof(float) * 4);
  alloc((void**)&r->offmax, sizeof(float) * n);
  alloc((void**)&r->rn, sizeof(float) * n);
  alloc((void**)&r->amax, sizeof(unsigned long long));
  alloc((void**)&r->flags, sizeof(int) * 4);
  alloc((void**)&r->cinfo, sizeof(int) * n);
  if (err != cudaSuccess) {
    refine_large_destroy(r);
    return -1000 - (int)err;
  }
  int orc = oz_create(&r->oz, n, n, n);
  if (!orc) orc = oz_create(&r->ozx, n, 0, n);
  if (!orc) orc = oz_create_f32(&r->oz32, n, n, n);
  if (orc) {
    refine_large_destroy(r);
    return orc;
  }
  r->h_lam.resize(n);
  r->h_couple.resize(n);
  *out = r;
  return 0;
}

void refine_large_destroy(RefineLarge* r) {
  if (!r) return;
  float* bufs[] = {r->Ahi, r->Alo, r->Xhi, r->Xlo, r->Phi, r->Plo, r->Rres, r->T, r->E, r->XE, r->Ghi, r->Glo,
                   r->Cbuf, r->Wbuf};
  for (float* b : bufs) cudaFree(b);
  cudaFree(r->nubuf);
  cudaFree(r->lam);
  cudaFree(r->gdiag);
  cudaFree(r->couple);
  cudaFree(r->cid);
  cudaFree(r->scal);
  cudaFree(r->offmax);
  cudaFree(r->rn);
  cudaFree(r->amax);
  cudaFree(r->flags);
  cudaFree(r->cinfo);
  for (auto& kv : r->big) large_destroy(kv.second);
  oz_destroy(r->oz);
  oz_destroy(r->ozx);
  oz_destroy(r->oz32);
  delete r;
}

int refine_large_iters(const RefineLarge* r) { return r->iters; }
int refine_large_rotations(const RefineLarge* r) { return r->rotated; }
float* refine_large_xbuf(RefineLarge* r) { return r->Xhi; }
float* refine_large_wbuf(RefineLarge* r) { return r->nubuf; }

// Eigen-decompositions of the cluster matrices (FP32): small ones in one
// batched plan, large ones one at a time.
static int solve_clusters(RefineLarge* r, const std::vector<int>& cs, const std::vector<int>& cc,
                          const std::vector<long long>& coff, cudaStream_t st) {
  std::vector<int64_t> small_n;
  std::vector<int> small_idx;
  for (size_t k = 0; k < cs.size(); k++) {
    if (cc[k] <= GLA_MAX_SMALL_N) {
      small_n.push_back(cc[k]);
      small_idx.push_back((int)k);
    }
  }
  if (!small_n.empty()) {
    // the packed buffers already follow the plan's arena layout when the
    // small clusters come first in coff order; copy them into a contiguous
    // arena otherwise
    gla_plan_t p = nullptr;
    int rc = gla_plan_create(&p, GLA_PREC_F32, 'V', 'L', (int64_t)small_n.size(), small_n.data(), 0.0,
                             GLA_FLAG_F32_BISECT);
    if (rc) return rc;
    long long aoff = 0, woff = 0;
    float* arena = r->Glo;   // free at this point (Gram blocks consumed)
    float* varena = r->Ghi;  // idem
    float* warena = r->Rres; // idem
    for (size_t q = 0; q < small_idx.size(); q++) {
      const int k = small_idx[q];
      RF_CUDA(cudaMemcpyAsync(arena + aoff, r->Cbuf + coff[k], sizeof(float) * cc[k] * cc[k],
                              cudaMemcpyDeviceToDevice, st));
      aoff += (long long)cc[k] * cc[k];
      woff += cc[k];
    }
    rc = gla_plan_execute(p, arena, warena, varena, r->cinfo, st);
    if (rc) {
      gla_plan_destroy(p);
      return rc;
    }
    aoff = 0;
    woff = 0;
    for (size_t q = 0; q < small_idx.size(); q++) {
      const int k = small_idx[q];
      RF_CUDA(cudaMemcpyAsync(r->Wbuf + coff[k], varena + aoff, sizeof(float) * cc[k] * cc[k],
                              cudaMemcpyDeviceToDevice, st));
      RF_CUDA(cudaMemcpyAsync(r->nubuf + cs[k], warena + woff, sizeof(float) * cc[k], cudaMemcpyDeviceToDevice,
                              st));
      aoff += (long long)cc[k] * cc[k];
      woff += cc[k];
    }
    RF_CUDA(cudaStreamSynchronize(st));
    gla_plan_destroy(p);
  }
  for (size_t k = 0; k < cs.size(); k++) {
    if (cc[k] <= GLA_MAX_SMALL_N) continue;
    LargeCtx* lc = nullptr;
    auto it = r->big.find(cc[k]);
    if (it != r->big.end()) {
      lc = it->second;
    } else {
      int rc = large_create(&lc, cc[k], false, true);
      if (rc) return rc;
      r->big[cc[k]] = lc;
    }
    int inf = 0;
    int rc = large_syev(lc, kF32, true, true, r->Cbuf + coff[k], cc[k], r->nubuf + cs[k], r->Wbuf + coff[k], cc[k],
                        &inf, st);
    if (rc) return rc;
  }
  return 0;
}

int refine_large_run(RefineLarge* r, const double* A, long long lda, bool lower, const float* X32, long long ldx,
                     const float* w32, double* w, double* V, long long ldv, cudaStream_t st) {
  const int n = r->n;
  const long long nn = (long long)n * n;
  const dim3 g2((n + 255) / 256, n);
  RF_CUDA(cudaMemsetAsync(r->amax, 0, sizeof(unsigned long long), st));
  RF_CUDA(cudaMemsetAsync(r->flags, 0, sizeof(int) * 4, st));
  k_ref_maxabs<<<g2, 256, 0, st>>>(A, lda, n, lower, r->amax, r->flags);
  RF_CUDA(cudaGetLastError());
  k_ref_load<<<g2, 256, 0, st>>>(A, lda, n, lower, r->amax, r->flags, r->Ahi, r->Alo, X32, ldx, r->Xhi, r->Xlo, w32,
                                 r->lam);
  RF_CUDA(cudaGetLastError());
  // A is symmetric: its rows are the columns of the (hi, lo) storage
  RF_CUDA(oz_slice(r->oz, true, r->Ahi, r->Alo, n, n, n, 7, st));
  RF_CUDA(cudaMemsetAsync(oz_error_word(r->oz), 0, sizeof(int), st));
  int hflags[2] = {0, 0};
  RF_CUDA(cudaMemcpyAsync(hflags, r->flags, sizeof(hflags), cudaMemcpyDeviceToHost, st));
  RF_CUDA(cudaStreamSynchronize(st));
  r->iters = 0;
  r->rotated = 0;
  r->reorders = 0;
  r->ortho_steps = 0;
  if (hflags[0] == 0) {
    bool polish = false;
    double emax_prev = 1e300;
    for (int it = 0; it < kRefMaxIters; it++) {
      r->iters = it + 1;
      if (it == kRefMaxIters - 1) polish = true;
      // P = A X on the tensor cores (Ozaki slices; the FP32 eigenvectors of
      // the first iteration are exact floats, X_lo = 0)
      RF_CUDA(oz_slice(r->oz, false, r->Xhi, it == 0 ? nullptr : r->Xlo, n, n, n, 7, st));
      RF_CUDA(oz_gemm(r->oz, n, n, n, r->Phi, r->Plo, n, false, st));
      k_ref_colstats<<<(n + 7) / 8, 256, 0, st>>>(r->Xhi, r->Xlo, r->Phi, r->Plo, n, r->lam, r->gdiag);
      RF_CUDA(cudaGetLastError());
      RF_CUDA(cudaMemsetAsync(r->scal, 0, sizeof(float) * 4, st));
      k_ref_rres<<<n, 256, 0, st>>>(r->Xhi, r->Xlo, r->Phi, r->Plo, r->lam, n, r->Rres, r->rn, r->scal + 2);
      RF_CUDA(cudaGetLastError());
      // T = X_hi' Rres to FP32 accuracy on the tensor cores (A operand: the
      // columns of X_hi; B operand: the columns of Rres)
      RF_CUDA(oz_slice(r->oz32, true, r->Xhi, nullptr, n, n, n, 4, st));
      RF_CUDA(oz_slice(r->oz32, false, r->Rres, nullptr, n, n, n, 4, st));
      RF_CUDA(oz_gemm(r->oz32, n, n, n, r->T, nullptr, n, false, st));
      k_ref_couple<<<(n + 255) / 256, 256, 0, st>>>(r->T, r->lam, r->rn, n, r->couple);
      RF_CUDA(cudaGetLastError());
      RF_CUDA(cudaMemcpyAsync(r->h_lam.data(), r->lam, sizeof(double) * n, cudaMemcpyDeviceToHost, st));
      RF_CUDA(cudaMemcpyAsync(r->h_couple.data(), r->couple, sizeof(int) * (n - 1), cudaMemcpyDeviceToHost, st));
      RF_CUDA(cudaStreamSynchronize(st));
      // clusters (runs of joined neighbours), the smallest separated gap
      std::vector<int> cs, cc, hcid(n, -1);
      std::vector<long long> coff;
      double gmin = 1e300;
      const double lmax = std::max(std::fabs(r->h_lam[0]), std::fabs(r->h_lam[n - 1]));
      long long off = 0;
      for (int p = 0; p < n;) {
        int q = p;
        while (q < n - 1 && r->h_couple[q]) q++;
        if (q > p) {
          cs.push_back(p);
          cc.push_back(q - p + 1);
          coff.push_back(off);
          off += (long long)(q - p + 1) * (q - p + 1);
          for (int i = p; i <= q; i++) hcid[i] = (int)cs.size() - 1;
        }
        if (q + 1 < n) gmin = std::min(gmin, std::fabs(r->h_lam[q + 1] - r->h_lam[q]));
        p = q + 1;
      }
      RF_CUDA(cudaMemcpyAsync(r->cid, hcid.data(), sizeof(int) * n, cudaMemcpyHostToDevice, st));
      // the Gram matrix X'X (lower triangle, before the update) when some
      // pair needs it: the polishing iteration, or clusters (pairs inside a
      // cluster take E_ij = -(X'X)_ij / 2). One tensor-core GEMM; X's
      // B-operand slices are current.
      if (polish || !cs.empty()) {
        RF_CUDA(oz_slice(r->ozx, true, r->Xhi, r->Xlo, n, n, n, 7, st));
        RF_CUDA(cudaMemsetAsync(oz_error_word(r->ozx), 0, sizeof(int), st));
        RF_CUDA(oz_gemm2(r->ozx, r->oz, n, n, n, r->Ghi, r->Glo, n, true, st));
      }
      k_ref_e<<<g2, 256, 0, st>>>(r->T, r->Ghi, r->Glo, r->lam, r->gdiag, r->cid, n, polish ? 1 : 0, 1e-14 * lmax,
                                  r->E, r->scal);
      RF_CUDA(cudaGetLastError());
      // X <- X + X E: FP32 product of X_hi and E while E is a correction
      // that the next iteration refines (its rounding, 2^-24 |X E|, is a
      // perturbation removed quadratically); the polishing iteration, the
      // last, forms X E in double-float on the tensor cores (A operand: the
      // rows of X; B operand: E, in the slot of X's slices, unused from here)
      // unless the corrections of the iteration before were below 1e-8: the
      // polish's then are smaller still, and the FP32-accuracy product's
      // rounding, ~6e-8 |E|, stays below 1e-15
      if (polish && !(emax_prev < 1e-8)) {
        RF_CUDA(oz_slice_rows(r->ozx, r->Xhi, r->Xlo, n, n, n, 7, st));
        RF_CUDA(oz_slice(r->oz, false, r->E, nullptr, n, n, n, 7, st));
        RF_CUDA(oz_gemm2(r->ozx, r->oz, n, n, n, r->Phi, r->Plo, n, false, st));
        k_ref_update_df<<<2048, 256, 0, st>>>(r->Xhi, r->Xlo, r->Phi, r->Plo, nn);
      } else {
        RF_CUDA(oz_slice_rows(r->oz32, r->Xhi, nullptr, n, n, n, 4, st));
        RF_CUDA(oz_slice(r->oz32, false, r->E, nullptr, n, n, n, 4, st));
        RF_CUDA(oz_gemm(r->oz32, n, n, n, r->XE, nullptr, n, false, st));
        k_ref_update<<<2048, 256, 0, st>>>(r->Xhi, r->Xlo, r->XE, nn);
      }
      RF_CUDA(cudaGetLastError());
      // Rayleigh-Ritz inside the clusters whose projected matrix is still
      // coupled (a resolved cluster only gets the Gram correction above: an
      // FP32 rotation would bring back 1e-7 non-orthogonality)
      std::vector<double> mus(cs.size());
      if (!cs.empty()) RF_CUDA(cudaMemsetAsync(r->offmax, 0, sizeof(float) * cs.size(), st));
      for (size_t k = 0; k < cs.size(); k++) {
        double mu = 0;
        for (int a = 0; a < cc[k]; a++) mu += r->h_lam[cs[k] + a];
        mus[k] = mu / cc[k];
        k_ref_cmat<<<std::min(1024, (cc[k] * cc[k] + 255) / 256), 256, 0, st>>>(r->T, r->lam, n, cs[k], cc[k], mus[k],
                                                                                 r->Cbuf + coff[k], r->offmax + k);
        RF_CUDA(cudaGetLastError());
      }
      std::vector<float> hoff(cs.size());
      float hs[4] = {0.f, 0.f, 0.f, 0.f};
      if (!cs.empty())
        RF_CUDA(cudaMemcpyAsync(hoff.data(), r->offmax, sizeof(float) * cs.size(), cudaMemcpyDeviceToHost, st));
      RF_CUDA(cudaMemcpyAsync(hs, r->scal, sizeof(hs), cudaMemcpyDeviceToHost, st));
      int oz_err[3] = {0, 0, 0};
      RF_CUDA(cudaMemcpyAsync(&oz_err[0], oz_error_word(r->oz), sizeof(int), cudaMemcpyDeviceToHost, st));
      RF_CUDA(cudaMemcpyAsync(&oz_err[1], oz_error_word(r->ozx), sizeof(int), cudaMemcpyDeviceToHost, st));
      RF_CUDA(cudaMemcpyAsync(&oz_err[2], oz_error_word(r->oz32), sizeof(int), cudaMemcpyDeviceToHost, st));
      RF_CUDA(cudaStreamSynchronize(st));
      if (oz_err[0] || oz_err[1] || oz_err[2])
        return -1000 - (int)cudaErrorLaunchTimeout;  // a bounded wait of the tensor-core GEMM ran out
      std::vector<int> rs, rcnt;
      std::vector<long long> roff;
      std::vector<double> rmu;
      for (size_t k = 0; k < cs.size() && !polish; k++)  // the polishing iteration never rotates
        if ((double)hoff[k] > 1e-15 * lmax) {
          rs.push_back(cs[k]);
          rcnt.push_back(cc[k]);
          roff.push_back(coff[k]);
          rmu.push_back(mus[k]);
        }
      if (!rs.empty()) {
        int rc = solve_clusters(r, rs, rcnt, roff, st);
        if (rc) return rc;
        for (size_t k = 0; k < rs.size(); k++) {
          if (rcnt[k] >= kOzRotateMin) {
            // X_J W on the tensor cores in double-float (A operand: the rows
            // of X_J in the Gram's slot, B operand: W in X's slot; both are
            // free once E is formed, and X is sliced anew next iteration)
            RF_CUDA(oz_slice_rows(r->ozx, r->Xhi + (long long)rs[k] * n, r->Xlo + (long long)rs[k] * n, n, n,
                                  rcnt[k], 7, st));
            RF_CUDA(oz_slice(r->oz, false, r->Wbuf + roff[k], nullptr, rcnt[k], rcnt[k], rcnt[k], 7, st));
            RF_CUDA(oz_gemm2(r->ozx, r->oz, n, rcnt[k], rcnt[k], r->Phi + (long long)rs[k] * n,
                             r->Plo + (long long)rs[k] * n, n, false, st));
          } else {
          DfGemmDesc gr{};
          gr.m = n;
          gr.n = rcnt[k];
          gr.k = rcnt[k];
          gr.Ahi = r->Xhi + (long long)rs[k] * n;
          gr.Alo = r->Xlo + (long long)rs[k] * n;
          gr.lda = n;
          gr.Bhi = r->Wbuf + roff[k];
          gr.Blo = nullptr;
          gr.ldb = rcnt[k];
          gr.Chi = r->Phi + (long long)rs[k] * n;
          gr.Clo = r->Plo + (long long)rs[k] * n;
          gr.ldc = n;
          RF_CUDA(dfgemm_launch(gr, false, st));
          }
          RF_CUDA(cudaMemcpyAsync(r->Xhi + (long long)rs[k] * n, r->Phi + (long long)rs[k] * n,
                                  sizeof(float) * n * rcnt[k], cudaMemcpyDeviceToDevice, st));
          RF_CUDA(cudaMemcpyAsync(r->Xlo + (long long)rs[k] * n, r->Plo + (long long)rs[k] * n,
                                  sizeof(float) * n * rcnt[k], cudaMemcpyDeviceToDevice, st));
          k_ref_setlam<<<(rcnt[k] + 255) / 256, 256, 0, st>>>(r->lam, rs[k], rcnt[k], rmu[k], r->nubuf + rs[k]);
          RF_CUDA(cudaGetLastError());
        }
      }
      r->rotated += (int)rs.size();
      if (polish) {
        // the polish corrects the orthogonality defect d it started from to
        // first order, leaving ~3/4 d^2 (7.5e-15 at d = 1e-7, far inside the
        // 1e-13 target): above d = 1e-7 (tight clusters
        // rotated by FP32 Rayleigh-Ritz solutions shortly before) one more
        // symmetric step X <- X (I + R/2) squares it again; both products on
        // the tensor cores in double-float. The residual moves by
        // (lam_j - lam_i) r_ij / 2, negligible where the defect sits (pairs
        // at tight gaps).
        if (hs[1] > 1e-7f) {
          RF_CUDA(oz_slice(r->ozx, true, r->Xhi, r->Xlo, n, n, n, 7, st));
          RF_CUDA(oz_slice(r->oz, false, r->Xhi, r->Xlo, n, n, n, 7, st));
          RF_CUDA(oz_gemm2(r->ozx, r->oz, n, n, n, r->Ghi, r->Glo, n, true, st));
          k_ref_ortho_e<<<g2, 256, 0, st>>>(r->Ghi, r->Glo, n, r->E);
          RF_CUDA(cudaGetLastError());
          RF_CUDA(oz_slice_rows(r->ozx, r->Xhi, r->Xlo, n, n, n, 7, st));
          RF_CUDA(oz_slice(r->oz, false, r->E, nullptr, n, n, n, 7, st));
          RF_CUDA(oz_gemm2(r->ozx, r->oz, n, n, n, r->Phi, r->Plo, n, false, st));
          k_ref_update_df<<<2048, 256, 0, st>>>(r->Xhi, r->Xlo, r->Phi, r->Plo, nn);
          RF_CUDA(cudaGetLastError());
          int ozx_err = 0;
          RF_CUDA(cudaMemcpyAsync(&ozx_err, oz_error_word(r->ozx), sizeof(int), cudaMemcpyDeviceToHost, st));
          RF_CUDA(cudaStreamSynchronize(st));
          if (ozx_err) return -1000 - (int)cudaErrorLaunchTimeout;
          r->ortho_steps++;
        }
        break;
      }
      // the eigenvectors have (nearly) converged: nothing rotated, and the
      // corrections are below 2e-7 (the polishing iteration, quadratically
      // convergent, leaves ~emax^2 ||A|| = 4e-14 ||A|| in the residual, inside
      // the 1e-13 target) or have stopped
      // falling (the rounding floor of the residual form, u ||A|| / gap, at
      // the tightest gaps). One more iteration with the full Gram matrix then
      // restores orthogonality to working accuracy (the residual form
      // recovers r_ij only to ~u ||A|| / gap_ij).
      const double emax = hs[0];
      if (rs.empty() && (emax < 2e-7 || (emax < 1e-5 && emax > 0.25 * emax_prev))) polish = true;
      emax_prev = emax;
      // keep the columns in ascending order (cluster updates can move an
      // eigenvalue past a neighbour that was not in its cluster)
      RF_CUDA(cudaMemcpyAsync(r->h_lam.data(), r->lam, sizeof(double) * n, cudaMemcpyDeviceToHost, st));
      RF_CUDA(cudaStreamSynchronize(st));
      bool ordered = true;
      for (int i = 0; i + 1 < n; i++) ordered &= r->h_lam[i] <= r->h_lam[i + 1];
      if (!ordered) {
        std::vector<int> perm(n);
        for (int i = 0; i < n; i++) perm[i] = i;
        std::stable_sort(perm.begin(), perm.end(), [&](int a, int b) { return r->h_lam[a] < r->h_lam[b]; });
        std::vector<double> l2(n);
        for (int i = 0; i < n; i++) l2[i] = r->h_lam[perm[i]];
        RF_CUDA(cudaMemcpyAsync(r->cid, perm.data(), sizeof(int) * n, cudaMemcpyHostToDevice, st));
        k_ref_gather<<<g2, 256, 0, st>>>(r->Xhi, r->Phi, r->cid, n);
        k_ref_gather<<<g2, 256, 0, st>>>(r->Xlo, r->Plo, r->cid, n);
        RF_CUDA(cudaGetLastError());
        RF_CUDA(cudaMemcpyAsync(r->Xhi, r->Phi, sizeof(float) * nn, cudaMemcpyDeviceToDevice, st));
        RF_CUDA(cudaMemcpyAsync(r->Xlo, r->Plo, sizeof(float) * nn, cudaMemcpyDeviceToDevice, st));
        RF_CUDA(cudaMemcpyAsync(r->lam, l2.data(), sizeof(double) * n, cudaMemcpyHostToDevice, st));
        RF_CUDA(cudaStreamSynchronize(st));
        r->reorders++;
      }
    }
  }
  // final order (cluster updates keep it, but guard against swaps of
  // rounding-level neighbours)
  RF_CUDA(cudaMemcpyAsync(r->h_lam.data(), r->lam, sizeof(double) * n, cudaMemcpyDeviceToHost, st));
  RF_CUDA(cudaStreamSynchronize(st));
  bool sorted = true;
  for (int i = 0; i + 1 < n; i++) sorted &= r->h_lam[i] <= r->h_lam[i + 1];
  const int* dperm = nullptr;
  if (!sorted) {
    std::vector<int> perm(n);
    for (int i = 0; i < n; i++) perm[i] = i;
    std::stable_sort(perm.begin(), perm.end(), [&](int a, int b) { return r->h_lam[a] < r->h_lam[b]; });
    RF_CUDA(cudaMemcpyAsync(r->cid, perm.data(), sizeof(int) * n, cudaMemcpyHostToDevice, st));
    RF_CUDA(cudaStreamSynchronize(st));
    dperm = r->cid;
  }
  k_ref_store<<<g2, 256, 0, st>>>(r->Xhi, r->Xlo, r->lam, dperm, n, r->flags, w, V, ldv);
  RF_CUDA(cudaGetLastError());
  RF_CUDA(cudaStreamSynchronize(st));
  return hflags[0] ? -1 : 0;
}

}  // namespace gla
