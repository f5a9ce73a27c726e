// Householder tridiagonalisation of one large symmetric matrix (lower
// triangle), blocked in panels of kSytrdNB columns: the LAPACK dsytrd/dlatrd
// organisation of the reference's symtriLower! (src/eigenSelfAdjoint.jl:450-504).
//
// Column j of a panel (c = j - k0 columns into it):
//   x  = A[j+1:, j] after the panel's earlier rank-2 terms
//   reflector H_j = I - tau v v' from x (reflector! convention: beta = -sign(x1)|x|,
//   v[j+1] = 1, v stored in A[j+2:, j] like the reference)
//   y  = A_t v - V (W' v) - W (V' v)     A_t = A[j+1:, j+1:] without this panel
//   w  = tau y - (tau^2 / 2)(y' v) v     (so A_t - v w' - w v' = H A_t H)
// and after the panel one rank-2k update A_t -= V W' + W V' (a GEMM over
// the lower tiles). Every panel is one cooperative launch over all SMs with
// two grid barriers per column:
//   phase 2 (all CTAs): reflector scalars from the norm partials, then the
//     SYMV in warp units of 32 columns x 256 rows of the trailing lower
//     triangle (each unit adds A_IJ v_J to its rows and A_IJ' v_I to its
//     columns, into deterministic partial buffers), the dot products V'v,
//     W'v and the quadratic form v'A_t v;
//   phase 3 (rows split over CTAs): y from the partials, w, the reflector
//     stored, and the next column updated with this column's terms plus its
//     norm partial.
// The barrier is a counter/generation pair in global memory whose waits are
// bounded: a wait that runs out sets the error word and every CTA leaves.
#include <cuda_runtime.h>

#include <algorithm>
#include <vector>

#include "gla_common.cuh"
#include "gla_large.h"

namespace gla {

constexpr int kTW = 32;        // SYMV unit width (columns)
constexpr int kRC = 256;       // SYMV unit height (rows): 8 rows per lane
constexpr int kDotRows = 1024; // rows per dot-product unit
constexpr int kPT = 256;       // threads per CTA
constexpr long long kSpinLimit = 1ll << 26;

template <class T>
struct SytrdArgs {
  T* A;
  long long ld;
  int n, k0, nbp;
  T* V;              // column c of the panel's V (n rows, leading dimension ldv)
  T* W;
  long long ldv;
  T* d;
  T* e;
  T* tau;
  T* P;              // row partials   [nTC][n]
  T* Qp;             // column partials [nCH][n]
  T* normp;          // [G]
  T* qfp;            // [G]
  T* dots;           // [2][kSytrdNB][nDCH]
  int nDCH;
  const int2* units; // (tile column, chunk), ordered by tile column
  const int* ustart; // first unit of each tile column; ustart[nTC] = total
  int nTC;
  unsigned* bar;     // [0] arrivals, [1] generation
  int* err;
};

// Returns the same verdict to every thread of the CTA (thread 0 decides and
// broadcasts it), so a CTA never splits at an early return.
GLA_DEV bool grid_sync(unsigned* bar, int* err) {
  __shared__ int s_ok;
  __syncthreads();
  if (threadIdx.x == 0) {
    volatile unsigned* vgen = bar + 1;
    volatile int* verr = err;
    const unsigned gen = *vgen;
    __threadfence();
    const unsigned arrived = atomicAdd(bar, 1u);
    if (arrived == gridDim.x - 1) {
      atomicExch(bar, 0u);
      __threadfence();
      atomicAdd(bar + 1, 1u);
    } else {
      long long it = 0;
      while (*vgen == gen) {
        if (*verr) break;
        if (++it > kSpinLimit) {
          atomicExch(err, 1);
          break;
        }
        __nanosleep(32);
      }
    }
    __threadfence();
    s_ok = *verr == 0;
  }
  __syncthreads();
  return s_ok != 0;
}

// Deterministic block sum (every CTA gets the same bits for the same inputs).
template <class T>
GLA_DEV T block_sum_all(T v, T* sred) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  __syncthreads();
  if ((threadIdx.x & 31) == 0) sred[threadIdx.x >> 5] = v;
  __syncthreads();
  T s = 0;
#pragma unroll
  for (int i = 0; i < kPT / 32; i++) s += sred[i];
  return s;
}

template <class T>
struct StepScalars {
  int j, s;
  T scale;  // v_i = A[i, j] * scale for i > s, v_s = 1
};

template <class T>
GLA_DEV T v_at(const T* __restrict__ A, long long ld, const StepScalars<T>& st, int i) {
  if (i == st.s) return T(1);
  if (i < st.s) return T(0);
  return A[i + (long long)st.j * ld] * st.scale;
}

// One warp: SYMV unit (tile column J, chunk ch). Adds rowacc to P[J][r] and
// the column sums to Qp[ch][c]; returns the unit's part of v'A_t v.
template <class T>
__device__ T symv_unit(const SytrdArgs<T>& a, const StepScalars<T>& st, int J, int ch, T* svcol) {
  const int lane = threadIdx.x & 31, n = a.n;
  const long long ld = a.ld;
  const T* __restrict__ A = a.A;
  const int c0 = J * kTW, r0 = c0 + ch * kRC;
  const int cc = c0 + lane;
  const T vc = cc < n ? v_at(A, ld, st, cc) : T(0);
  svcol[lane] = vc;
  __syncwarp();
  T vr[8], rowacc[8];
#pragma unroll
  for (int q = 0; q < 8; q++) {
    const int r = r0 + lane + 32 * q;
    vr[q] = r < n ? v_at(A, ld, st, r) : T(0);
    rowacc[q] = T(0);
  }
  const bool diag = ch == 0;
  T colacc[kTW];
#pragma unroll
  for (int ci = 0; ci < kTW; ci++) {
    const T vcv = svcol[ci];
    const bool cin = c0 + ci < n;
    const T* __restrict__ col = A + (long long)(c0 + ci) * ld;
    T ca = T(0);
#pragma unroll
    for (int q = 0; q < 8; q++) {
      const int r = r0 + lane + 32 * q;
      T x = (cin && r < n) ? col[r] : T(0);
      T xr = x, xc = x;
      if (q == 0 && diag) {  // diagonal tile: lower part only (row >= column)
        xr = lane >= ci ? x : T(0);
        xc = lane > ci ? x : T(0);
      }
      rowacc[q] = fma(xr, vcv, rowacc[q]);
      ca = fma(xc, vr[q], ca);
    }
    colacc[ci] = ca;
  }
  T qf = T(0);
#pragma unroll
  for (int q = 0; q < 8; q++) {
    const int r = r0 + lane + 32 * q;
    if (r < n) a.P[(long long)J * n + r] = rowacc[q];
    qf = fma(rowacc[q], vr[q], qf);
  }
  // reduce-scatter the 32 column sums across the warp: lane l keeps column l
#pragma unroll
  for (int half = 16; half >= 1; half >>= 1) {
    const bool up = (lane & half) != 0;
#pragma unroll
    for (int i = 0; i < half; i++) {
      const T send = up ? colacc[i] : colacc[i + half];
      const T keep = up ? colacc[i + half] : colacc[i];
      colacc[i] = keep + __shfl_xor_sync(0xffffffffu, send, half);
    }
  }
  if (cc < n) a.Qp[(long long)ch * n + cc] = colacc[0];
  qf = fma(colacc[0], vc, qf);
  __syncwarp();
  return qf;
}

// Rows of the trailing range [s, n) owned by CTA g.
GLA_DEV void own_rows(int s, int n, int& lo, int& hi) {
  const int m = n - s, G = gridDim.x;
  const int R = (m + G - 1) / G;
  lo = min(n, s + (int)blockIdx.x * R);
  hi = min(n, lo + R);
}

template <class T>
__global__ void __launch_bounds__(kPT, 1) k_sytrd_panel(const SytrdArgs<T> a) {
  const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
  const int n = a.n, G = gridDim.x, g = blockIdx.x;
  const long long ld = a.ld, ldv = a.ldv;
  T* __restrict__ A = a.A;
  __shared__ T sred[kPT / 32];
  __shared__ T svcol[kPT / 32][32];
  __shared__ T sdotV[kSytrdNB], sdotW[kSytrdNB], sVs[kSytrdNB + 1], sWs[kSytrdNB + 1];
  __shared__ T sys[2];

  // panel start: norm partial of column k0 below the subdiagonal
  {
    const int j = a.k0, s = j + 1;
    int lo, hi;
    own_rows(s, n, lo, hi);
    T part = T(0);
    for (int i = lo + tid; i < hi; i += kPT)
      if (i > s) {
        const T x = A[i + (long long)j * ld];
        part = fma(x, x, part);
      }
    part = block_sum_all(part, sred);
    if (tid == 0) a.normp[g] = part;
  }
  if (!grid_sync(a.bar, a.err)) return;

  for (int c = 0; c < a.nbp; c++) {
    const int j = a.k0 + c, s = j + 1, m = n - s;
    // ---------------- phase 2: reflector scalars (redundant per CTA), SYMV, dots
    T sigma = T(0);
    for (int i = tid; i < G; i += kPT) sigma += a.normp[i];
    sigma = block_sum_all(sigma, sred);
    const T alpha = A[s + (long long)j * ld];
    T beta, tau, scale;
    if (sigma == T(0)) {
      beta = alpha;
      tau = T(0);
      scale = T(0);
    } else {
      const T nrm2 = fma(alpha, alpha, sigma);
      const T nrm = nrm2 * prec<T>::rsqrt(nrm2);
      beta = -copysign(nrm, alpha);
      const T rb = prec<T>::rcp(beta);
      tau = (beta - alpha) * rb;
      scale = prec<T>::rcp(alpha - beta);
    }
    if (g == 0 && tid == 0) {
      a.d[j] = A[j + (long long)j * ld];
      a.e[j] = beta;
      a.tau[j] = tau;
    }
    StepScalars<T> st;
    st.j = j;
    st.s = s;
    st.scale = scale;
    const int J0 = s / kTW;
    const int usym0 = a.ustart[J0], nsym = a.ustart[a.nTC] - usym0;
    const int ndch = (m + kDotRows - 1) / kDotRows;
    const int ndot = 2 * c * ndch;
    T qf = T(0);
    for (int u = g * (kPT / 32) + wid; u < nsym + ndot; u += G * (kPT / 32)) {
      if (u < nsym) {
        const int2 jc = a.units[usym0 + u];
        qf += symv_unit(a, st, jc.x, jc.y, svcol[wid]);
      } else {
        const int du = u - nsym;
        const int which = du / (c * ndch), rem = du % (c * ndch);
        const int q = rem / ndch, chn = rem % ndch;
        const T* __restrict__ X = (which == 0 ? a.V : a.W) + (long long)q * ldv;
        const int r0 = s + chn * kDotRows, r1 = min(n, r0 + kDotRows);
        T acc = T(0);
        for (int r = r0 + lane; r < r1; r += 32) acc = fma(X[r], v_at(A, ld, st, r), acc);
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
        if (lane == 0) a.dots[((long long)which * kSytrdNB + q) * a.nDCH + chn] = acc;
      }
    }
    qf = block_sum_all(qf, sred);
    if (tid == 0) a.qfp[g] = qf;
    if (!grid_sync(a.bar, a.err)) return;

    // ---------------- phase 3: y, w, reflector store, next column
    for (int q = tid; q < c; q += kPT) {
      T sv = T(0), sw = T(0);
      for (int k = 0; k < ndch; k++) {
        sv += a.dots[((long long)0 * kSytrdNB + q) * a.nDCH + k];
        sw += a.dots[((long long)1 * kSytrdNB + q) * a.nDCH + k];
      }
      sdotV[q] = sv;
      sdotW[q] = sw;
      sVs[q] = a.V[s + (long long)q * ldv];
      sWs[q] = a.W[s + (long long)q * ldv];
    }
    T qsum = T(0);
    for (int i = tid; i < G; i += kPT) qsum += a.qfp[i];
    qsum = block_sum_all(qsum, sred);  // (its barriers also publish sdotV/sdotW)
    T pq = T(0);
    for (int q = tid; q < c; q += kPT) pq = fma(sdotV[q], sdotW[q], pq);
    pq = block_sum_all(pq, sred);
    const T ytv = qsum - T(2) * pq;
    const T hw = T(0.5) * tau * tau * ytv;  // w = tau y - hw v
    // y_s and w_s (every CTA; warp 0)
    if (wid == 0) {
      T ys = T(0);
      const int Js = s / kTW;
      const int nch = (n - Js * kTW + kRC - 1) / kRC;
      if (lane == 0) ys += a.P[(long long)Js * n + s];
      for (int k = lane; k < nch; k += 32) ys += a.Qp[(long long)k * n + s];
      for (int q = lane; q < c; q += 32) ys -= sVs[q] * sdotW[q] + sWs[q] * sdotV[q];
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) ys += __shfl_xor_sync(0xffffffffu, ys, o);
      if (lane == 0) sys[0] = tau * ys - hw;
    }
    __syncthreads();
    if (tid == 0) {
      sVs[c] = T(1);
      sWs[c] = sys[0];
    }
    __syncthreads();
    const bool last_in_panel = c + 1 == a.nbp;
    const bool update_next = !last_in_panel || s == n - 1;
    int lo, hi;
    own_rows(s, n, lo, hi);
    const int R = hi - lo;
    int tpr = 1;
    while (tpr < 32 && tpr * 2 * R <= kPT) tpr *= 2;
    const int sub = tid % tpr, rpp = kPT / tpr;
    T npart = T(0);
    for (int base = lo; base < hi; base += rpp) {
      const int i = base + tid / tpr;
      const bool act = i < hi;
      const int ii = act ? i : lo;
      // y_i from the partial buffers, minus the panel terms
      T y = T(0);
      const int Ji = ii / kTW;
      for (int Jx = J0 + sub; Jx <= Ji; Jx += tpr) y += a.P[(long long)Jx * n + ii];
      const int nch = (n - Ji * kTW + kRC - 1) / kRC;
      for (int k = sub; k < nch; k += tpr) y += a.Qp[(long long)k * n + ii];
      for (int q = sub; q < c; q += tpr)
        y -= a.V[ii + (long long)q * ldv] * sdotW[q] + a.W[ii + (long long)q * ldv] * sdotV[q];
      for (int o = tpr / 2; o > 0; o >>= 1) y += __shfl_xor_sync(0xffffffffu, y, o, tpr);
      const T vi = v_at(A, ld, st, ii);
      const T wi = tau * y - hw * vi;
      T xn = T(0);
      if (update_next) {
        for (int q = sub; q < c; q += tpr)
          xn += a.V[ii + (long long)q * ldv] * sWs[q] + a.W[ii + (long long)q * ldv] * sVs[q];
        for (int o = tpr / 2; o > 0; o >>= 1) xn += __shfl_xor_sync(0xffffffffu, xn, o, tpr);
        xn += vi * sWs[c] + wi * sVs[c];
      }
      // all reads of column j (v_at) are done by every thread of the group before the store
      __syncwarp();
      if (act && sub == 0) {
        a.V[ii + (long long)c * ldv] = vi;
        a.W[ii + (long long)c * ldv] = wi;
        if (ii > s) A[ii + (long long)j * ld] = vi;
        if (update_next) {
          const T x = A[ii + (long long)s * ld] - xn;
          A[ii + (long long)s * ld] = x;
          if (ii > s + 1) npart = fma(x, x, npart);
          if (s == n - 1) a.d[n - 1] = x;
        }
      }
    }
    npart = block_sum_all(npart, sred);
    if (tid == 0) a.normp[g] = npart;
    if (c + 1 < a.nbp)
      if (!grid_sync(a.bar, a.err)) return;
  }
}

// ---------------------------------------------------------------- host side

struct SytrdPlan {
  int n = 0, G = 0;
  int nTC = 0, nCH = 0, nDCH = 0;
  int2* units = nullptr;
  int* ustart = nullptr;
  void* P = nullptr;
  void* Qp = nullptr;
  void* normp = nullptr;
  void* qfp = nullptr;
  void* dots = nullptr;
  void* VW = nullptr;     // [V | W] panel buffer, n x 2 kSytrdNB
  int* bkidx = nullptr;   // SYR2K k remaps: [2 nb] for nbp = kSytrdNB, then for the last panel
  unsigned* bar = nullptr;
  int* err = nullptr;
  bool f64 = true;
};

}  // namespace gla

namespace {
using namespace gla;

template <class T>
cudaError_t sytrd_run(SytrdPlan& sp, T* A, long long lda, T* d, T* e, T* tau, cudaStream_t st) {
  const int n = sp.n;
  cudaError_t err;
  if ((err = cudaMemsetAsync(sp.bar, 0, 2 * sizeof(unsigned), st)) != cudaSuccess) return err;
  if ((err = cudaMemsetAsync(sp.err, 0, sizeof(int), st)) != cudaSuccess) return err;
  SytrdArgs<T> a;
  a.A = A;
  a.ld = lda;
  a.n = n;
  a.ldv = n;
  a.d = d;
  a.e = e;
  a.tau = tau;
  a.P = (T*)sp.P;
  a.Qp = (T*)sp.Qp;
  a.normp = (T*)sp.normp;
  a.qfp = (T*)sp.qfp;
  a.dots = (T*)sp.dots;
  a.nDCH = sp.nDCH;
  a.units = sp.units;
  a.ustart = sp.ustart;
  a.nTC = sp.nTC;
  a.bar = sp.bar;
  a.err = sp.err;
  T* VW = (T*)sp.VW;
  const int nsteps = n - 1;  // reflectors 0 .. n-2
  for (int k0 = 0; k0 < nsteps; k0 += kSytrdNB) {
    const int nbp = std::min(kSytrdNB, nsteps - k0);
    a.k0 = k0;
    a.nbp = nbp;
    a.V = VW;
    a.W = VW + (long long)nbp * n;
    void* args[] = {(void*)&a};
    err = cudaLaunchCooperativeKernel((const void*)k_sytrd_panel<T>, dim3(sp.G), dim3(kPT), args, 0, st);
    if (err != cudaSuccess) return err;
    const int t = k0 + nbp;
    if (t < n - 1) {  // trailing update A[t:, t:] -= V W' + W V' (lower tiles)
      GemmDesc g{};
      g.m = n - t;
      g.n = n - t;
      g.k = 2 * nbp;
      g.A = VW + t;
      g.lda = n;
      g.B = VW + t;
      g.ldb = n;
      g.C = A + t + (long long)t * lda;
      g.ldc = lda;
      g.b_kidx = sp.bkidx + (nbp == kSytrdNB ? 0 : 2 * kSytrdNB);
      g.alpha = -1.0;
      g.beta = 1.0;
      err = gemm_launch(sizeof(T) == 8, false, true, true, g, 1, st);
      if (err != cudaSuccess) return err;
    }
  }
  return cudaSuccess;
}

}  // namespace

namespace gla {

cudaError_t sytrd_plan_create(SytrdPlan** out, int n, bool f64) {
  *out = nullptr;
  SytrdPlan* sp = new SytrdPlan();
  sp->n = n;
  sp->f64 = f64;
  int dev = 0, nsm = 0, per = 0;
  cudaError_t err = cudaGetDevice(&dev);
  if (err == cudaSuccess) err = cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  if (err == cudaSuccess)
    err = cudaOccupancyMaxActiveBlocksPerMultiprocessor(
        &per, f64 ? (const void*)k_sytrd_panel<double> : (const void*)k_sytrd_panel<float>, kPT, 0);
  if (err == cudaSuccess && per < 1) err = cudaErrorCooperativeLaunchTooLarge;
  if (err != cudaSuccess) {
    delete sp;
    return err;
  }
  sp->G = nsm;  // one CTA per SM (co-residency of a cooperative launch)
  sp->nTC = (n + kTW - 1) / kTW;
  sp->nCH = (n + kRC - 1) / kRC;
  sp->nDCH = (n + kDotRows - 1) / kDotRows;
  std::vector<int2> units;
  std::vector<int> ustart(sp->nTC + 1);
  for (int J = 0; J < sp->nTC; J++) {
    ustart[J] = (int)units.size();
    const int nch = (n - J * kTW + kRC - 1) / kRC;
    for (int ch = 0; ch < nch; ch++) units.push_back(make_int2(J, ch));
  }
  ustart[sp->nTC] = (int)units.size();
  std::vector<int> bk(4 * kSytrdNB);
  const int last = (n - 1) % kSytrdNB == 0 ? kSytrdNB : (n - 1) % kSytrdNB;
  for (int kk = 0; kk < 2 * kSytrdNB; kk++) bk[kk] = kk < kSytrdNB ? kSytrdNB + kk : kk - kSytrdNB;
  for (int kk = 0; kk < 2 * last; kk++) bk[2 * kSytrdNB + kk] = kk < last ? last + kk : kk - last;
  const size_t el = f64 ? 8 : 4;
  auto alloc = [&](void** p, size_t bytes) {
    if (err == cudaSuccess) err = cudaMalloc(p, std::max<size_t>(bytes, 16));
  };
  alloc((void**)&sp->units, sizeof(int2) * units.size());
  alloc((void**)&sp->ustart, sizeof(int) * ustart.size());
  alloc(&sp->P, el * (size_t)sp->nTC * n);
  alloc(&sp->Qp, el * (size_t)sp->nCH * n);
  alloc(&sp->normp, el * sp->G);
  alloc(&sp->qfp, el * sp->G);
  alloc(&sp->dots, el * 2 * kSytrdNB * sp->nDCH);
  alloc(&sp->VW, el * (size_t)n * 2 * kSytrdNB);
  alloc((void**)&sp->bkidx, sizeof(int) * bk.size());
  alloc((void**)&sp->bar, 2 * sizeof(unsigned));
  alloc((void**)&sp->err, sizeof(int));
  if (err == cudaSuccess)
    err = cudaMemcpy(sp->units, units.data(), sizeof(int2) * units.size(), cudaMemcpyHostToDevice);
  if (err == cudaSuccess)
    err = cudaMemcpy(sp->ustart, ustart.data(), sizeof(int) * ustart.size(), cudaMemcpyHostToDevice);
  if (err == cudaSuccess) err = cudaMemcpy(sp->bkidx, bk.data(), sizeof(int) * bk.size(), cudaMemcpyHostToDevice);
  if (err == cudaSuccess) err = cudaMemset(sp->VW, 0, el * (size_t)n * 2 * kSytrdNB);
  if (err != cudaSuccess) {
    sytrd_plan_destroy(sp);
    return err;
  }
  *out = sp;
  return cudaSuccess;
}

void sytrd_plan_destroy(SytrdPlan* sp) {
  if (!sp) return;
  cudaFree(sp->units);
  cudaFree(sp->ustart);
  cudaFree(sp->P);
  cudaFree(sp->Qp);
  cudaFree(sp->normp);
  cudaFree(sp->qfp);
  cudaFree(sp->dots);
  cudaFree(sp->VW);
  cudaFree(sp->bkidx);
  cudaFree(sp->bar);
  cudaFree(sp->err);
  delete sp;
}

cudaError_t sytrd_enqueue(SytrdPlan* sp, void* A, long long lda, void* d, void* e, void* tau, cudaStream_t st) {
  if (sp->f64) return sytrd_run<double>(*sp, (double*)A, lda, (double*)d, (double*)e, (double*)tau, st);
  return sytrd_run<float>(*sp, (float*)A, lda, (float*)d, (float*)e, (float*)tau, st);
}

int* sytrd_error_word(SytrdPlan* sp) { return sp->err; }

}  // namespace gla
