// Device body of the batched Householder tridiagonalisation (one CTA per
// matrix, n <= 128), shared by its kernel (small_tridiag.cu) and by the
// persistent FP32 + refinement kernel (refine.cu). See small_tridiag.cu.
#pragma once
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
GLA_DEV void tridiag_body(int mid, unsigned char* smem_raw, const SmallDesc* __restrict__ descs,
                          const Tin* __restrict__ A, int lower, T* __restrict__ dout, T* __restrict__ eout,
                          T* __restrict__ Qout, int* __restrict__ info, ChaseState* __restrict__ cst,
                          int* __restrict__ scale_exp, T* __restrict__ wout, T* __restrict__ qtmp,
                          T* __restrict__ rows2 = nullptr) {
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
  // (flat over the n^2 entries, so that every thread has several
  // independent loads in flight; column j = idx / n by a float reciprocal,
  // exact for idx < 2^14: the quotient's fraction stays >= 1/(2n) from 1)
  int bad = 0;
  unsigned long long amax = 0;
  const float inv_n = 1.f / (float)n;
#pragma unroll 4
  for (int idx = tid; idx < n * n; idx += NT) {
    const int j = (int)(((float)idx + 0.5f) * inv_n), i = idx - j * n;
    if (lower ? (i >= j) : (i <= j)) {
      Tin v = Ag[idx];
      bad |= !isfinite(v);
      unsigned long long b = AbsBits<Tin>::get(v);
      amax = b > amax ? b : amax;
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
#pragma unroll 4
  for (int idx = tid; idx < n * n; idx += NT) {
    const int j = (int)(((float)idx + 0.5f) * inv_n), i = idx - j * n;
    if (lower ? (i >= j) : (i <= j)) {
      Tin v = Ag[idx];
      T t = (sizeof(Tin) != sizeof(T)) ? (T)ldexp((double)v, -sexp) : (T)v;
      if (lower) S[j * ld + i] = t;
      else S[i * ld + j] = t;
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
    // ---- A~ += v w' - u v'   (== x(xi x)' - x u' - u x' of :484-491), lower triangle:
    // a warp per column (columns dealt in snake order, w, 2 nw - 1 - w, 2 nw + w,
    // ..., which evens out their lengths), lanes over its rows
    {
      const int lane = tid & 31, wid = tid >> 5, nw = NT >> 5;
      for (int r = 0;; r++) {
        const int j = r * nw + ((r & 1) ? (nw - 1 - wid) : wid);
        if (j >= m) break;
        const T wj = ww[j], vj = vv[j];
        T* col = At + (size_t)j * ld;
        for (int i = j + lane; i < m; i += 32) {
          T a = col[i];
          a = fma(vv[i], wj, a);
          a = fma(-uu[i], vj, a);
          col[i] = a;
        }
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
  if (!WANTQ && rows2) {
    // eigen2! (src/eigenSelfAdjoint.jl:633-644): only rows 1 and n of Q,
    // [e_1'; e_n'] Q = rmul!(V, Q) (:62-80), in place of Array(Q): row 1 is
    // e_1' (Q = diag(1, Qt)); row n is e_n' H_0 H_1 ... H_{n-3}, one
    // reflector at a time (H_k on indices k+1.., v = [1; column k below its
    // subdiagonal], tau_k). Stored 2 x n column-major at 2 w_off.
    __syncthreads();
    T* r = vv;  // the row being formed (n entries); uu holds the dot-product partials
    for (int i = tid; i < n; i += NT) r[i] = (i == n - 1) ? T(1) : T(0);
    __syncthreads();
    for (int k = 0; k + 2 < n; k++) {
      const T tau = taus[k];
      if (tau == T(0)) continue;  // uniform: taus is shared
      T part = T(0);
      for (int i = k + 1 + tid; i < n; i += NT) part = fma(r[i], (i == k + 1) ? T(1) : S[(size_t)k * ld + i], part);
      const T dot = block_sum(part, red);
      const T f = tau * dot;
      for (int i = k + 1 + tid; i < n; i += NT) r[i] = fma(-f, (i == k + 1) ? T(1) : S[(size_t)k * ld + i], r[i]);
      __syncthreads();
    }
    T* R2 = rows2 + 2 * dsc.w_off;
    for (int i = tid; i < n; i += NT) {
      R2[2 * i] = (i == 0) ? T(1) : T(0);
      R2[2 * i + 1] = r[i];
    }
    return;
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

}  // namespace gla
