// Batched Householder tridiagonalisation and explicit Q, one CTA per matrix,
// the whole matrix staged in shared memory (n <= 128).
//
// Replaces, per matrix:
//   symtriLower! (GenericLinearAlgebra.jl src/eigenSelfAdjoint.jl:450-504)
//   with LinearAlgebra.reflector! (called at :466) and BLAS symv (:477),
//   and Array(Q::EigenQ) = lmul!(Q, I) (:101, :23-41).
// uplo 'U' input is mirrored into the lower triangle on load, so both
// triangles run the 'L' reduction (the 'U' variant :507-564 reduces the
// mirrored matrix in reverse order and yields the same eigenpairs).
//
// Work split (FP64 on GB300 costs ~68 cycles per warp instruction no matter
// how many lanes are active, so every FP64 loop is spread over all lanes):
//   norm / dot products: one element per thread + block reduction,
//   SYMV: rows x (1, 2 or 4 column parts),
//   rank-2 update: flat index over the trailing lower triangle,
//   Q formation: dorg2l-style backward accumulation in place of the
//   reflectors (H_k applied only to the already-formed trailing block).
#include <algorithm>

#include "gla_launch.h"
#include "gla_small.cuh"
#include "small_stein.cuh"

namespace gla {

template <class T> struct AbsBits;
template <> struct AbsBits<double> {
  static GLA_DEV unsigned long long get(double x) { return (unsigned long long)__double_as_longlong(x) & 0x7fffffffffffffffull; }
  static GLA_DEV double from(unsigned long long b) { return __longlong_as_double((long long)b); }
};
template <> struct AbsBits<float> {
  static GLA_DEV unsigned long long get(float x) { return (unsigned long long)(__float_as_uint(x) & 0x7fffffffu); }
  static GLA_DEV float from(unsigned long long b) { return __uint_as_float((unsigned)b); }
};

// Sum and max (of non-negative bit patterns) over the block.
template <class T>
GLA_DEV void block_sum_max(T v, unsigned long long m, T* red, unsigned long long* redm, T& sum, unsigned long long& mx) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    v += __shfl_xor_sync(0xffffffffu, v, o);
    unsigned long long w = __shfl_xor_sync(0xffffffffu, m, o);
    m = w > m ? w : m;
  }
  __syncthreads();
  if (lane == 0) {
    red[wid] = v;
    redm[wid] = m;
  }
  __syncthreads();
  T s = red[0];
  unsigned long long x = redm[0];
  for (int i = 1; i < nw; i++) {
    s += red[i];
    x = redm[i] > x ? redm[i] : x;
  }
  sum = s;
  mx = x;
}

// Leading dimension of the staged matrix: odd, so that transposed accesses
// (stride ld across the lanes of a warp) spread over all shared-memory banks.
GLA_DEV int stage_ld(int n) { return (n + 1) | 1; }

size_t tridiag_smem_bytes(int n, int nt, int elem, bool) {
  // redm[32] u64 | red[32] (8-byte slots) | S[n*ld] | vv,uu,ww,taus [n] | part[8*nt]
  // (the FP32 tridiagonal solver reuses S and part once Q is in global memory)
  const size_t ld = (size_t)((n + 1) | 1);
  return 512 + (size_t)elem * ((size_t)n * ld + 4 * (size_t)n + 8 * (size_t)nt);
}

// X = Q Y (n x n, Q column-major with leading dimension ld, Y row-major in
// Ys with leading dimension ldy), stored column-major to Xg. Thread tiles of
// 8 x 8 outputs with rows and columns strided by ceil(n/8), so that the
// threads of a warp read consecutive (or identical) words.
GLA_DEV void small_gemm_qy(int n, const float* __restrict__ S, int ld, const float* __restrict__ Ys, int ldy,
                           float* __restrict__ Xg) {
  const int nt8 = (n + 7) >> 3;
  for (int t = threadIdx.x; t < nt8 * nt8; t += blockDim.x) {
    const int ti = t % nt8, tk = t / nt8;
    float acc[8][8];
#pragma unroll
    for (int u = 0; u < 8; u++)
#pragma unroll
      for (int v = 0; v < 8; v++) acc[u][v] = 0.f;
    int iu[8], kv[8];
#pragma unroll
    for (int u = 0; u < 8; u++) {
      iu[u] = min(ti + nt8 * u, n - 1);  // clamped: rows/columns past n are computed and not stored
      kv[u] = min(tk + nt8 * u, n - 1);
    }
    for (int j = 0; j < n; j++) {
      float q[8], y[8];
#pragma unroll
      for (int u = 0; u < 8; u++) q[u] = S[(size_t)j * ld + iu[u]];
#pragma unroll
      for (int v = 0; v < 8; v++) y[v] = Ys[(size_t)j * ldy + kv[v]];
#pragma unroll
      for (int u = 0; u < 8; u++)
#pragma unroll
        for (int v = 0; v < 8; v++) acc[u][v] = fmaf(q[u], y[v], acc[u][v]);
    }
#pragma unroll
    for (int u = 0; u < 8; u++)
#pragma unroll
      for (int v = 0; v < 8; v++) {
        const int i = ti + nt8 * u, k = tk + nt8 * v;
        if (i < n && k < n) Xg[(size_t)k * n + i] = acc[u][v];
      }
  }
}

// STEIN (float only): after forming Q, solve the tridiagonal in the same CTA
// (small_stein.cuh) and write X = Q Y and the ascending eigenvalues (times
// 2^scale) to wout, marking the matrix done for the chase; a matrix the
// solver leaves to the QL chase gets Q as usual. Q goes to qtmp (an n x n
// float scratch per matrix, arena layout) first, so that the solver's
// arrays reuse the shared memory of the reduction.
template <class T, class Tin, bool WANTQ, bool STEIN>
__global__ void __launch_bounds__(256) k_tridiag(const SmallDesc* __restrict__ descs, const int* __restrict__ perm,
                                                 const Tin* __restrict__ A, int lower, T* __restrict__ dout,
                                                 T* __restrict__ eout, T* __restrict__ Qout, int* __restrict__ info,
                                                 ChaseState* __restrict__ cst, int* __restrict__ scale_exp,
                                                 T* __restrict__ wout, T* __restrict__ qtmp) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int mid = perm[blockIdx.x];
  const SmallDesc dsc = descs[mid];
  const int n = dsc.n;
  const int ld = stage_ld(n);
  const int tid = threadIdx.x, NT = blockDim.x;
  unsigned long long* redm = reinterpret_cast<unsigned long long*>(smem_raw);
  T* red = reinterpret_cast<T*>(smem_raw + 256);
  T* S = reinterpret_cast<T*>(smem_raw + 512);
  T* vv = S + (size_t)n * ld;
  T* uu = vv + n;
  T* ww = uu + n;
  T* taus = ww + n;
  T* part = taus + n;

  const Tin* Ag = A + dsc.a_off;
  // ---- load the referenced triangle (mirroring 'U' into 'L'), check finiteness
  int bad = 0;
  unsigned long long amax = 0;
  for (int j = 0; j < n; j++) {
    for (int i = tid; i < n; i += NT) {
      if (lower ? (i >= j) : (i <= j)) {
        Tin v = Ag[(size_t)j * n + i];
        bad |= !isfinite(v);
        unsigned long long b = AbsBits<Tin>::get(v);
        amax = b > amax ? b : amax;
      }
    }
  }
  bad = __syncthreads_or(bad);
  if (tid == 0) {
    ChaseState st;
    st.bs = 0;
    st.nsweeps = 0;
    st.nrot = 0;
    st.nhdr = 0;
    st.status = bad ? kChaseDone : kChaseRunning;
    st.applied = 0;
    cst[mid] = st;
    info[mid] = bad ? -1 : 0;
  }
  if (bad) return;
  // Reduced-precision runs scale the matrix by an exact power of two so that
  // its largest entry is near 1 (no overflow/underflow in the narrow type).
  int sexp = 0;
  if (sizeof(Tin) != sizeof(T)) {
    unsigned long long mx = amax;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      unsigned long long w = __shfl_xor_sync(0xffffffffu, mx, o);
      mx = w > mx ? w : mx;
    }
    if ((tid & 31) == 0) redm[tid >> 5] = mx;
    __syncthreads();
    mx = redm[0];
    for (int w = 1; w < (NT >> 5); w++) mx = redm[w] > mx ? redm[w] : mx;
    __syncthreads();
    if (mx != 0) {
      int e2;
      frexp(AbsBits<Tin>::from(mx), &e2);
      sexp = e2;  // max |A| * 2^-sexp in [0.5, 1)
    }
    if (tid == 0) scale_exp[mid] = sexp;
  }
  for (int j = 0; j < n; j++) {
    for (int i = tid; i < n; i += NT) {
      if (lower ? (i >= j) : (i <= j)) {
        Tin v = Ag[(size_t)j * n + i];
        T t = (sizeof(Tin) != sizeof(T)) ? (T)ldexp((double)v, -sexp) : (T)v;
        if (lower) S[j * ld + i] = t;
        else S[i * ld + j] = t;
      }
    }
  }
  __syncthreads();

  // ---- symtriLower!: k = 0 .. n-3
  for (int k = 0; k + 2 < n; k++) {
    const int m = n - k - 1;
    T* xc = S + (size_t)k * ld + (k + 1);
    const T xi = (tid < m) ? xc[tid] : T(0);
    const T x0 = xc[0];  // read before the reduction's barriers; thread 0 rewrites xc[0] below
    T sumsq;
    unsigned long long mb;
    block_sum_max<T>(xi * xi, (tid < m) ? AbsBits<T>::get(xi) : 0ull, red, redm, sumsq, mb);
    T tau = 0;
    if (mb != 0) {
      // LinearAlgebra.reflector!: norm (scaled only when maxabs^2 would
      // overflow or underflow), nu = copysign(norm, x1), x1 += nu,
      // x[2:] /= x1, tau = x1/nu, x[1] = -nu.
      const T maxabs = AbsBits<T>::from(mb);
      const T mm = maxabs * maxabs;
      T normu;
      if (isfinite((T)m * mm) && mm != 0) {
        normu = prec<T>::sqrt_ieee(sumsq);
      } else {
        const T r = (tid < m) ? xi / maxabs : T(0);
        T s2;
        unsigned long long dummy;
        block_sum_max<T>(r * r, 0ull, red, redm, s2, dummy);
        normu = maxabs * prec<T>::sqrt_ieee(s2);
      }
      const T nu = tcopysign(normu, x0);
      const T xi1 = x0 + nu;
      tau = prec<T>::div_ieee(xi1, nu);
      const T scl = prec<T>::tame(xi1) ? prec<T>::rcp(xi1) : prec<T>::div_ieee(T(1), xi1);
      if (tid < m) {
        const T v = (tid == 0) ? T(1) : xi * scl;
        vv[tid] = v;
        xc[tid] = (tid == 0) ? -nu : v;
      }
    }
    if (tid == 0) taus[k] = tau;
    __syncthreads();
    if (mb == 0) continue;  // zero column: H = I, nothing to update

    // ---- u = tau * A~ * v (lower-triangle SYMV); rows x P column parts
    T* At = S + (size_t)(k + 1) * ld + (k + 1);
    {
      const int R = (m + 31) & ~31;
      int P = NT / R;
      P = P > 8 ? 8 : P;
      const int p = tid / R, i = tid - p * R;
      if (p < P && i < m) {
        const int j0 = (p * m) / P, j1 = ((p + 1) * m) / P;
        T acc0 = 0, acc1 = 0;
        int j = j0;
        for (; j + 1 < j1; j += 2) {
          const int a0 = (j <= i) ? (j * ld + i) : (i * ld + j);
          const int a1 = (j + 1 <= i) ? ((j + 1) * ld + i) : (i * ld + j + 1);
          acc0 = fma(At[a0], vv[j], acc0);
          acc1 = fma(At[a1], vv[j + 1], acc1);
        }
        if (j < j1) acc0 = fma(At[(j <= i) ? (j * ld + i) : (i * ld + j)], vv[j], acc0);
        part[p * NT + i] = acc0 + acc1;
      }
      __syncthreads();
      T ui = 0;
      if (tid < m) {
        T s = part[tid];
        for (int q = 1; q < P; q++) s += part[q * NT + tid];
        ui = tau * s;
        uu[tid] = ui;
      }
      // xi = tau * (v' u)
      const T vi = (tid < m) ? vv[tid] : T(0);
      const T xsum = block_sum(vi * ui, red);
      const T xiv = tau * xsum;
      if (tid < m) ww[tid] = xiv * vi - ui;
      __syncthreads();
    }
    // ---- A~ += v w' - u v'   (== x(xi x)' - x u' - u x' of :484-491), lower triangle
    {
      const int total = m * (m + 1) / 2;
      int j = 0, cs = 0, ce = m;
      for (int f = tid; f < total; f += NT) {
        while (f >= ce) {
          j++;
          cs = ce;
          ce += m - j;
        }
        const int i = j + (f - cs);
        T a = At[j * ld + i];
        a = fma(vv[i], ww[j], a);
        a = fma(-uu[i], vv[j], a);
        At[j * ld + i] = a;
      }
    }
    __syncthreads();
  }

  // ---- diagonals
  T* dg = dout + dsc.w_off;
  T* eg = eout + dsc.w_off;
  for (int i = tid; i < n; i += NT) {
    const T di = S[(size_t)i * ld + i], ei = (i + 1 < n) ? S[(size_t)i * ld + i + 1] : T(0);
    dg[i] = di;
    eg[i] = ei;
    if (STEIN) {  // uu, ww are free after the reduction: d and e for the tridiagonal solver
      uu[i] = di;
      ww[i] = ei;
    }
  }
  if (!WANTQ) return;
  __syncthreads();

  // ---- Q = H_0 H_1 ... H_{n-3} (Array(EigenQ) of the reference), in place.
  // Q = diag(1, Qt); reflector kk lives in column kk (rows kk+2..), Qt's
  // column kk is global column kk+1, formed after H_kk is applied to the
  // trailing columns kk+2.. (rows kk+1..).
  for (int r = tid; r < n; r += NT) S[(size_t)(n - 1) * ld + r] = (r == n - 1) ? T(1) : T(0);
  __syncthreads();
  for (int kk = n - 3; kk >= 0; kk--) {
    const T tau = taus[kk];
    const int M = n - kk - 1;
    if (tid < M) vv[tid] = (tid == 0) ? T(1) : S[(size_t)kk * ld + kk + 1 + tid];
    __syncthreads();
    const int C = n - kk - 2;
    if (tau != T(0)) {
      // two lanes per column (row halves), partial dots combined by shuffle
      const int half = (M + 1) >> 1;
      for (int t2 = tid; t2 < 2 * ((C + 15) / 16) * 16; t2 += NT) {
        const int t = t2 >> 1, h = t2 & 1;
        const bool live = t < C;
        T* col = S + (size_t)(kk + 2 + (live ? t : 0)) * ld + (kk + 1);
        const int r0 = h * half, r1 = h ? M : half;
        T d0 = 0, d1 = 0;
        if (live) {
          int r = r0;
          for (; r + 1 < r1; r += 2) {
            d0 = fma(vv[r], col[r], d0);
            d1 = fma(vv[r + 1], col[r + 1], d1);
          }
          if (r < r1) d0 = fma(vv[r], col[r], d0);
        }
        T dot = d0 + d1;
        dot += __shfl_xor_sync(0xffffffffu, dot, 1);
        const T tmp = tau * dot;
        if (live)
          for (int r = r0; r < r1; r++) col[r] = fma(-vv[r], tmp, col[r]);
      }
    }
    __syncthreads();
    {
      T* col = S + (size_t)(kk + 1) * ld;
      for (int r = tid; r < n; r += NT)
        col[r] = (r <= kk) ? T(0) : ((r == kk + 1) ? T(1) - tau : -tau * vv[r - kk - 1]);
    }
    __syncthreads();
  }
  for (int r = tid; r < n; r += NT) S[r] = (r == 0) ? T(1) : T(0);
  __syncthreads();
  T* Qg = Qout + dsc.a_off;
  if constexpr (STEIN) {
    float* Qt = qtmp + dsc.a_off;
    for (int j = 0; j < n; j++)
      for (int i = tid; i < n; i += NT) Qt[(size_t)j * n + i] = S[(size_t)j * ld + i];
    __syncthreads();
    // Y over S (leading dimension ld), e^2, eigenvalues and flags over part
    // (8 NT >= 3 n + 8 words), d and e stay in uu and ww
    float* Ys = S;
    float* e2s = part;
    float* lams = e2s + n;
    int* misc = reinterpret_cast<int*>(lams + n);  // [0] give up, [1] clusters, [2 + 2c], [3 + 2c] bounds
    // red and redm (64 8-byte slots) are free here: the solver's reduction scratch
    const bool solved = stein_solve(n, uu, ww, e2s, lams, Ys, ld, misc, reinterpret_cast<float*>(redm));
    if (solved) {
      small_gemm_qy(n, Qt, n, Ys, ld, Qg);
      for (int k = tid; k < n; k += NT) wout[dsc.w_off + k] = sexp ? ldexpf(lams[k], sexp) : lams[k];
      if (tid == 0) {
        ChaseState st;
        st.bs = n;
        st.nsweeps = 0;
        st.nrot = 0;
        st.nhdr = 0;
        st.status = kChaseDone;
        st.applied = 1;
        cst[mid] = st;
      }
      return;
    }
    // left to the QL chase: Q, the chase state stays "running"
    for (int j = 0; j < n; j++)
      for (int i = tid; i < n; i += NT) Qg[(size_t)j * n + i] = Qt[(size_t)j * n + i];
    return;
  }
  for (int j = 0; j < n; j++)
    for (int i = tid; i < n; i += NT) Qg[(size_t)j * n + i] = S[(size_t)j * ld + i];
}


size_t stein_tri_smem_bytes(int n) { return 512 + 4 * (2 * (size_t)n + stein_extra_words(n)); }

// Tridiagonal input on the FP32 stage (the leaves of the divide and conquer
// of the FP32 + refinement path): the per-eigenvalue solver of
// small_stein.cuh on (d, e) as the chase would take them, one CTA per
// matrix (blockDim >= n). A solved matrix gets its ascending eigenvalues in
// wout and its eigenvectors in Q, and is marked done for the chase and the
// rotation replay; the others keep Q = I and their "running" chase state.
__global__ void __launch_bounds__(128) k_stein_tri(const SmallDesc* __restrict__ descs, const int* __restrict__ perm,
                                                   const float* __restrict__ dg_all, const float* __restrict__ eg_all,
                                                   float* __restrict__ Qout, float* __restrict__ wout,
                                                   ChaseState* __restrict__ cst, const int* __restrict__ info) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int mid = perm[blockIdx.x];
  const SmallDesc dsc = descs[mid];
  const int n = dsc.n, tid = threadIdx.x;
  if (n < 1 || info[mid] != 0 || cst[mid].status != kChaseRunning) return;
  float* fscr = reinterpret_cast<float*>(smem_raw);  // 128 floats
  float* dd = reinterpret_cast<float*>(smem_raw + 512);
  float* ee = dd + n;
  const int ldy = stein_ldy(n);
  float* Ys = ee + n;
  float* e2s = Ys + (size_t)n * ldy;
  float* lams = e2s + n;
  int* misc = reinterpret_cast<int*>(lams + n);
  for (int i = tid; i < n; i += blockDim.x) {
    dd[i] = dg_all[dsc.w_off + i];
    ee[i] = (i + 1 < n) ? eg_all[dsc.w_off + i] : 0.f;
  }
  __syncthreads();
  if (!stein_solve(n, dd, ee, e2s, lams, Ys, ldy, misc, fscr)) return;
  float* Qg = Qout + dsc.a_off;
  for (int j = 0; j < n; j++)
    for (int i = tid; i < n; i += blockDim.x) Qg[(size_t)j * n + i] = Ys[(size_t)i * ldy + j];
  for (int k = tid; k < n; k += blockDim.x) wout[dsc.w_off + k] = lams[k];
  if (tid == 0) {
    ChaseState st;
    st.bs = n;
    st.nsweeps = 0;
    st.nrot = 0;
    st.nhdr = 0;
    st.status = kChaseDone;
    st.applied = 1;
    cst[mid] = st;
  }
}

cudaError_t launch_stein_tri(int nblocks, int nmax, cudaStream_t st, const SmallDesc* descs, const int* perm,
                             const void* d, const void* e, void* Q, void* w, ChaseState* cst, const int* info) {
  if (nblocks <= 0) return cudaSuccess;
  const int nt = std::max(32, (nmax + 31) / 32 * 32);
  k_stein_tri<<<nblocks, nt, stein_tri_smem_bytes(nmax), st>>>(descs, perm, (const float*)d, (const float*)e,
                                                               (float*)Q, (float*)w, cst, info);
  return cudaGetLastError();
}

template <class T, class Tin, bool Q, bool ST = false> static void set_tri_attr() {
  cudaFuncSetAttribute(k_tridiag<T, Tin, Q, ST>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                       (int)tridiag_smem_bytes(kSmallMaxN, 256, sizeof(T), ST));
}

cudaError_t tridiag_kernels_init() {
  set_tri_attr<double, double, true>();
  set_tri_attr<double, double, false>();
  set_tri_attr<float, float, true>();
  set_tri_attr<float, float, false>();
  set_tri_attr<float, double, true>();
  set_tri_attr<float, double, false>();
  set_tri_attr<float, double, true, true>();
  set_tri_attr<float, float, true, true>();
  cudaFuncSetAttribute(k_stein_tri, cudaFuncAttributeMaxDynamicSharedMemorySize,
                       (int)stein_tri_smem_bytes(kSmallMaxN));
  return cudaGetLastError();
}

cudaError_t launch_tridiag(int tcode, bool wantq, int nblocks, int nt, size_t smem, cudaStream_t st,
                           const SmallDesc* descs, const int* perm, const void* A, int lower, void* d, void* e,
                           void* Q, int* info, ChaseState* cst, int* scale_exp, bool stein, void* w,
                           void* qtmp) {
  if (nblocks <= 0) return cudaSuccess;
#define GLA_TRI(T, Tin, WQ, ST)                                                                                 \
  k_tridiag<T, Tin, WQ, ST><<<nblocks, nt, smem, st>>>(descs, perm, (const Tin*)A, lower, (T*)d, (T*)e, (T*)Q, \
                                                       info, cst, scale_exp, (T*)w, (T*)qtmp)
  if (tcode == kF64) {
    if (wantq) GLA_TRI(double, double, true, false);
    else GLA_TRI(double, double, false, false);
  } else if (tcode == kF32) {
    if (wantq && stein) GLA_TRI(float, float, true, true);
    else if (wantq) GLA_TRI(float, float, true, false);
    else GLA_TRI(float, float, false, false);
  } else {
    if (wantq && stein) GLA_TRI(float, double, true, true);
    else if (wantq) GLA_TRI(float, double, true, false);
    else GLA_TRI(float, double, false, false);
  }
#undef GLA_TRI
  return cudaGetLastError();
}

}  // namespace gla
