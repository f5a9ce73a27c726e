// Householder tridiagonalisation of one large symmetric matrix (lower
// triangle), blocked in panels of kSytrdNB columns: the LAPACK dsytrd/dlatrd
// organisation of the reference's symtriLower! (src/eigenSelfAdjoint.jl:450-504).
//
// Column j of a panel (c = j - k0 columns into it), s = j + 1:
//   x  = A[s:, j] after the panel's earlier rank-2 terms
//   reflector H_j = I - tau v v' from x (reflector! convention: beta = -sign(x1)|x|,
//   v[s] = 1, v stored in A[s+1:, j] like the reference)
//   y  = A_t v - V (W' v) - W (V' v)     A_t = A[s:, s:] without this panel
//   w  = tau y - (tau^2 / 2)(y' v) v     (so A_t - v w' - w v' = H A_t H)
// and after the panel one rank-2k update A_t -= V W' + W V' (a GEMM over
// the lower tiles). Every panel is one cooperative launch over all SMs with
// two grid barriers per column:
//   phase A (all CTAs): the SYMV of A_t with the raw column a (a_i = x_i
//     below row s, so it needs no reflector scalars and starts at once), in
//     warp units of 32 columns x 64 rows of the lower triangle (each unit
//     adds A_IJ a_J to its rows and A_IJ' a_I to its columns, into
//     deterministic partial buffers), the dot products V'a, W'a,
//     a'A[:, s] and the quadratic form a'A_t a;
//   phase B (rows split over CTAs): the reflector scalars from the norm
//     partials, v = scale a + e_s applied to the phase A results by
//     linearity, y, w, the reflector stored, and the next column updated
//     with this column's terms plus its norm partial.
// Each phase issues all of its global loads before its first reduction:
// on GB300 an L2 round trip costs about a microsecond and is the unit of
// cost at the small trailing orders. Phase B's rows are split over the CTAs
// once per panel (rows k0 + 1 .. n - 1; a row above the current column's s
// is idle), so each CTA computes V and W for the same rows in every column
// of the panel and keeps them in shared memory for the rank-2 corrections
// of the later columns, instead of reading them back from L2.
#include <cuda_runtime.h>

#include <algorithm>
#include <vector>

#include "gla_common.cuh"
#include "gla_large.h"
#include "tc_gemm.cuh"

namespace gla {

constexpr int kTW = 32;        // SYMV unit width (columns)
constexpr int kRC = 64;        // SYMV unit height (rows): 2 rows per lane
constexpr int kMaxTC = 16384 / kTW;  // tile columns at the largest order
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
  T* dots;           // [3][kSytrdNB][nDCH]
  int nDCH;
  const int* ustart; // first SYMV unit of each tile column; ustart[nTC] = total
  int nTC;
  unsigned* bar;     // arrival counter (monotonic over the launches of one tridiagonalisation)
  unsigned bar_base; // counter value when this launch starts
  int* err;
};

// Grid barrier on a monotonic arrival counter: barrier number k of a launch
// completes when the counter reaches (k + 1) * gridDim.x. Thread 0 of each
// CTA arrives with a release add and polls with acquire loads; the wait is
// bounded (kSpinLimit polls) and a timeout sets the error word, which every
// waiting CTA also watches. The verdict is broadcast through shared memory
// so that all threads of a CTA return the same value.
GLA_DEV bool grid_sync(unsigned* bar, int* err, unsigned& target) {
  __shared__ int s_ok;
  target += gridDim.x;
  __syncthreads();
  if (threadIdx.x == 0) {
    __threadfence();
    asm volatile("red.release.gpu.global.add.u32 [%0], 1;" ::"l"(bar) : "memory");
    volatile int* verr = err;
    long long it = 0;
    for (;;) {
      unsigned v;
      asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(bar) : "memory");
      if ((int)(v - target) >= 0) break;
      if (*verr) break;
      if (++it > kSpinLimit) {
        atomicExch(err, 1);
        break;
      }
    }
    s_ok = *verr == 0;
  }
  __syncthreads();
  return s_ok != 0;
}

// Deterministic block sum of up to 4 values (every CTA gets the same bits
// for the same inputs). `buf` alternates between two shared slots so that
// consecutive calls need a single __syncthreads each.
template <class T, int K>
GLA_DEV void block_sum(T (&v)[K], T (*sred)[kPT / 32][4], int& buf) {
#pragma unroll
  for (int k = 0; k < K; k++)
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v[k] += __shfl_xor_sync(0xffffffffu, v[k], o);
  if ((threadIdx.x & 31) == 0)
#pragma unroll
    for (int k = 0; k < K; k++) sred[buf][threadIdx.x >> 5][k] = v[k];
  __syncthreads();
#pragma unroll
  for (int k = 0; k < K; k++) {
    T s = T(0);
#pragma unroll
    for (int i = 0; i < kPT / 32; i++) s += sred[buf][i][k];
    v[k] = s;
  }
  buf ^= 1;
}

// a_i = A[i, j] below row s (the raw reflector column), 0 elsewhere. The
// SYMV runs on a (no reflector scalars needed yet); phase B restores
// v = scale a + e_s by linearity.
template <class T>
GLA_DEV T a_at(const T* __restrict__ A, long long ld, int j, int s, int i) {
  return i > s ? A[i + (long long)j * ld] : T(0);
}

// One warp: SYMV unit (tile column J, chunk ch) of the trailing lower
// triangle on the raw column a, row by row (lane l holds row r0 + l + 32 q);
// all loads of the unit are issued before its FMAs. Adds the row sums to
// P[J][r] and the column sums to Qp[ch][c]; returns the unit's part of a'A_t a.
template <class T>
__device__ T symv_unit(const SytrdArgs<T>& a, int j, int s, int J, int ch, T* svcol) {
  constexpr int NQ = kRC / 32;
  const int lane = threadIdx.x & 31, n = a.n;
  const long long ld = a.ld;
  const T* __restrict__ A = a.A;
  const int c0 = J * kTW, r0 = c0 + ch * kRC;
  const int cc = c0 + lane;
  const T vc = cc < n ? a_at(A, ld, j, s, cc) : T(0);
  const T* __restrict__ base = A + (long long)c0 * ld + r0 + lane;
  const int ncol = min(kTW, n - c0);
  T x[NQ][kTW], vr[NQ];
#pragma unroll
  for (int q = 0; q < NQ; q++) {
    const int r = r0 + lane + 32 * q;
    const bool rin = r < n;
    const T* rowp = base + 32 * q;
#pragma unroll
    for (int ci = 0; ci < kTW; ci++) x[q][ci] = (rin && ci < ncol) ? rowp[(long long)ci * ld] : T(0);
    vr[q] = rin ? a_at(A, ld, j, s, r) : T(0);
  }
  svcol[lane] = vc;
  __syncwarp();
  T colacc[kTW];
#pragma unroll
  for (int ci = 0; ci < kTW; ci++) colacc[ci] = T(0);
  T qf = T(0);
#pragma unroll
  for (int q = 0; q < NQ; q++) {
    if (r0 + 32 * q >= n) break;  // warp-uniform
    const bool diag = ch == 0 && q == 0;  // diagonal tile: lower part only (row >= column)
    T rowacc = T(0);
#pragma unroll
    for (int ci = 0; ci < kTW; ci++) {
      const T xr = (diag && lane < ci) ? T(0) : x[q][ci];
      const T xc = (diag && lane <= ci) ? T(0) : x[q][ci];
      rowacc = fma(xr, svcol[ci], rowacc);
      colacc[ci] = fma(xc, vr[q], colacc[ci]);
    }
    const int r = r0 + lane + 32 * q;
    if (r < n) a.P[(long long)J * n + r] = rowacc;
    qf = fma(rowacc, vr[q], qf);
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

// Rows per CTA of phase B in the panel starting at column k0 (the split of
// rows k0 + 1 .. n - 1, fixed for the panel).
GLA_DEV __host__ int panel_rows(int k0, int n, int G) { return (n - k0 - 1 + G - 1) / G; }

// Dot-product unit kinds, in work-list order after the SYMV units.
constexpr int kDotA = 0;  // sum_r a_r A[r, s]        (cross term of v'A_t v)
constexpr int kDotV = 1;  // sum_r a_r V[r, q], q < c
constexpr int kDotW = 2;  // sum_r a_r W[r, q]

template <class T>
__global__ void __launch_bounds__(kPT, 1) k_sytrd_panel(const SytrdArgs<T> a) {
  const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
  const int n = a.n, G = gridDim.x, g = blockIdx.x;
  const long long ld = a.ld, ldv = a.ldv;
  T* __restrict__ A = a.A;
  __shared__ T sred[2][kPT / 32][4];
  __shared__ T svcol[kPT / 32][32];
  __shared__ T sdotV[kSytrdNB], sdotW[kSytrdNB], sVs[kSytrdNB], sWs[kSytrdNB];
  __shared__ int sust[kMaxTC + 1];
  __shared__ T sscal[4];
  // this CTA's V and W rows of the panel (rows lo0 .. lo0 + R0 - 1, columns
  // 0 .. nbp - 1), dynamic shared memory
  extern __shared__ __align__(16) unsigned char vw_raw[];
  T* sVr = reinterpret_cast<T*>(vw_raw);
  const int R0 = panel_rows(a.k0, n, G);
  T* sWr = sVr + (size_t)R0 * kSytrdNB;
  const int lo0 = min(n, a.k0 + 1 + g * R0), hi0 = min(n, lo0 + R0);
  for (int i = tid; i < 2 * R0 * kSytrdNB; i += kPT) sVr[i] = T(0);
  int rb = 0;
  unsigned bar_target = a.bar_base;
  for (int i = tid; i <= a.nTC; i += kPT) sust[i] = a.ustart[i];

  // panel start: norm partial of column k0 below the subdiagonal
  {
    const int j = a.k0, s = j + 1;
    int lo, hi;
    own_rows(s, n, lo, hi);
    T part[1] = {T(0)};
    for (int i = lo + tid; i < hi; i += kPT)
      if (i > s) {
        const T x = A[i + (long long)j * ld];
        part[0] = fma(x, x, part[0]);
      }
    block_sum(part, sred, rb);
    if (tid == 0) a.normp[g] = part[0];
  }
  if (!grid_sync(a.bar, a.err, bar_target)) return;

  for (int c = 0; c < a.nbp; c++) {
    const int j = a.k0 + c, s = j + 1, m = n - s;
    const int J0 = s / kTW;
    // ---------------- phase A: SYMV and dot products on the raw column a
    {
      const int usym0 = sust[J0], nsym = sust[a.nTC] - usym0;
      const int ndch = (m + kDotRows - 1) / kDotRows;
      const int ndot = (2 * c + 1) * ndch;
      T qf[1] = {T(0)};
      // unit u goes to CTA u % G, so every CTA gets an even share
      for (int k = wid;; k += kPT / 32) {
        const int u = g + G * k;
        if (u >= nsym + ndot) break;
        if (u < nsym) {
          const int ug = usym0 + u;
          int lo = J0, hi = a.nTC - 1;  // tile column: last J with sust[J] <= ug
          while (lo < hi) {
            const int mid = (lo + hi + 1) >> 1;
            if (sust[mid] <= ug) lo = mid; else hi = mid - 1;
          }
          qf[0] += symv_unit(a, j, s, lo, ug - sust[lo], svcol[wid]);
        } else {
          const int du = u - nsym;
          const int kind = du < ndch ? kDotA : (du - ndch) / (c * ndch) + 1;
          const int rem = du < ndch ? du : (du - ndch) % (c * ndch);
          const int q = rem / ndch, chn = rem % ndch;
          const T* __restrict__ X = kind == kDotA ? A + (long long)s * ld
                                                  : (kind == kDotV ? a.V : a.W) + (long long)q * ldv;
          const int r0 = s + 1 + chn * kDotRows, r1 = min(n, r0 + kDotRows);
          T acc = T(0);
          for (int r = r0 + lane; r < r1; r += 32) acc = fma(X[r], A[r + (long long)j * ld], acc);
#pragma unroll
          for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
          if (lane == 0) a.dots[((long long)kind * kSytrdNB + q) * a.nDCH + chn] = acc;
        }
      }
      block_sum(qf, sred, rb);
      if (tid == 0) a.qfp[g] = qf[0];
    }
    if (!grid_sync(a.bar, a.err, bar_target)) return;

    // ---------------- phase B: reflector scalars, y, w, reflector store, next column
    const int ndch = (m + kDotRows - 1) / kDotRows;
    const int Js = s / kTW;
    const int nchs = (n - Js * kTW + kRC - 1) / kRC;
    const int R = R0;
    int tpr = 1;
    while (tpr < 32 && tpr * 2 * R <= kPT) tpr *= 2;
    const int sub = tid % tpr;
    const int rl = tid / tpr;  // this thread's row of the CTA's panel rows
    const int i = lo0 + rl;
    const bool act = i < hi0 && i >= s;
    const int ii = act ? i : s;  // idle threads read row s (always in range)
    const int rc = rl < R ? rl : R - 1;  // (idle threads: any cached row)
    // (1) every load of the phase, independent of the reductions
    T red[4] = {T(0), T(0), T(0), T(0)};  // sigma, a'A_t a, sum a_r A[r,s], y_s raw
    for (int t = tid; t < G; t += kPT) {
      red[0] += a.normp[t];
      red[1] += a.qfp[t];
    }
    for (int k = tid; k < ndch; k += kPT) red[2] += a.dots[((long long)kDotA * kSytrdNB) * a.nDCH + k];
    if (tid < c) {
      T sv = T(0), sw = T(0);
      for (int k = 0; k < ndch; k++) {
        sv += a.dots[((long long)kDotV * kSytrdNB + tid) * a.nDCH + k];
        sw += a.dots[((long long)kDotW * kSytrdNB + tid) * a.nDCH + k];
      }
      sdotV[tid] = sv;
      sdotW[tid] = sw;
      sVs[tid] = a.V[s + (long long)tid * ldv];
      sWs[tid] = a.W[s + (long long)tid * ldv];
    }
    for (int k = tid - 64; k >= 0 && k < nchs; k += kPT - 64) red[3] += a.Qp[(long long)k * n + s];
    if (tid == 63) red[3] += a.P[(long long)Js * n + s];
    const T alpha = A[s + (long long)j * ld];
    const T Ass = A[s + (long long)s * ld];
    T yraw = T(0);
    {
      const int Ji = ii / kTW;
      for (int Jx = J0 + sub; Jx <= Ji; Jx += tpr) yraw += a.P[(long long)Jx * n + ii];
      const int nch = (n - Ji * kTW + kRC - 1) / kRC;
      for (int k = sub; k < nch; k += tpr) yraw += a.Qp[(long long)k * n + ii];
    }
    const T ai = a_at(A, ld, j, s, ii);
    const T Ais = A[ii + (long long)s * ld];
    block_sum(red, sred, rb);  // also publishes sdotV/sdotW/sVs/sWs
    // (2) reflector scalars and the q-sums once, in warp 0 (lanes over q;
    // FP64 work repeated by every warp would queue on the FP64 pipe)
    if (wid == 0) {
      const T sigma = red[0];
      T beta, tau, scale;
      if (sigma == T(0)) {
        beta = alpha;
        tau = T(0);
        scale = T(0);
      } else {
        const T nrm2 = fma(alpha, alpha, sigma);
        const T nrm = nrm2 * prec<T>::rsqrt(nrm2);
        beta = -copysign(nrm, alpha);
        tau = (beta - alpha) * prec<T>::rcp(beta);
        scale = prec<T>::rcp(alpha - beta);
      }
      // p = V'v, q = W'v with v = scale a + e_s; y_s and v'A_t v by linearity
      T pq = T(0), corr = T(0);
      if (lane < c) {
        const T pv = fma(scale, sdotV[lane], sVs[lane]), qv = fma(scale, sdotW[lane], sWs[lane]);
        pq = pv * qv;
        corr = sVs[lane] * qv + sWs[lane] * pv;
      }
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) {
        pq += __shfl_xor_sync(0xffffffffu, pq, o);
        corr += __shfl_xor_sync(0xffffffffu, corr, o);
      }
      if (lane == 0) {
        const T vAv = scale * scale * red[1] + T(2) * scale * red[2] + Ass;
        const T hw = T(0.5) * tau * tau * (vAv - T(2) * pq);  // w = tau y - hw v
        const T y_s = scale * red[3] + Ass - corr;
        sscal[0] = tau;
        sscal[1] = scale;
        sscal[2] = hw;
        sscal[3] = tau * y_s - hw;  // w_s
        if (g == 0) {
          if (c == 0) a.d[j] = A[j + (long long)j * ld];  // later columns: written by the previous step
          a.e[j] = beta;
          a.tau[j] = tau;
        }
      }
    }
    __syncthreads();
    const T tau = sscal[0], scale = sscal[1], hw = sscal[2], w_s = sscal[3];
    const bool last_in_panel = c + 1 == a.nbp;
    const bool update_next = !last_in_panel || s == n - 1;
    // (3) own rows
    T y = T(0), xn = T(0);
    for (int q = sub; q < c; q += tpr) {
      const T vq = sVr[(size_t)rc * kSytrdNB + q], wq = sWr[(size_t)rc * kSytrdNB + q];
      const T pv = fma(scale, sdotV[q], sVs[q]), qv = fma(scale, sdotW[q], sWs[q]);
      y -= vq * qv + wq * pv;
      xn += vq * sWs[q] + wq * sVs[q];
    }
    if (sub == 0) y += scale * yraw + Ais;
    else y += scale * yraw;
    for (int o = tpr / 2; o > 0; o >>= 1) {
      y += __shfl_xor_sync(0xffffffffu, y, o, tpr);
      xn += __shfl_xor_sync(0xffffffffu, xn, o, tpr);
    }
    const T vi = ii == s ? T(1) : scale * ai;
    const T wi = tau * y - hw * vi;
    xn += vi * w_s + wi;  // the q = c term: v_s = 1, w_s
    T npart[1] = {T(0)};
    if (act && sub == 0) {
      a.V[ii + (long long)c * ldv] = vi;
      a.W[ii + (long long)c * ldv] = wi;
      sVr[(size_t)rl * kSytrdNB + c] = vi;
      sWr[(size_t)rl * kSytrdNB + c] = wi;
      if (ii > s) A[ii + (long long)j * ld] = vi;
      if (update_next) {
        // A[s, s] is read by every CTA in this phase: its new value goes to d[s]
        const T x = Ais - xn;
        if (ii == s)
          a.d[s] = x;
        else
          A[ii + (long long)s * ld] = x;
        if (ii > s + 1) npart[0] = x * x;
      }
    }
    block_sum(npart, sred, rb);
    if (tid == 0) a.normp[g] = npart[0];
    if (c + 1 < a.nbp)
      if (!grid_sync(a.bar, a.err, bar_target)) return;
  }
}

// ---------------------------------------------------------------- host side

struct SytrdPlan {
  int n = 0, G = 0;
  int nTC = 0, nCH = 0, nDCH = 0;
  int* ustart = nullptr;
  void* P = nullptr;
  void* Qp = nullptr;
  void* normp = nullptr;
  void* qfp = nullptr;
  void* dots = nullptr;
  void* VW = nullptr;     // [V | W] panel buffer, n x 2 kSytrdNB
  float* VWt = nullptr;   // FP32: [V | W] transposed (2 kSytrdNB x n), the tensor-core update's K-major operand
  int* bkidx = nullptr;   // SYR2K k remaps: [2 nb] for nbp = kSytrdNB, then for the last panel
  unsigned* bar = nullptr;
  int* err = nullptr;
  bool f64 = true;
};

// [V | W] of a panel with nbp reflectors (V at VW, W at VW + nbp n, rows
// t.. of interest) into VWt: row kk < 32 = V column kk, row 32 + kk = W
// column kk (zero for kk >= nbp), column i = row i.
__global__ void k_vw_transpose(const float* __restrict__ VW, int n, int nbp, int t, float* __restrict__ VWt) {
  __shared__ float tile[32][65];
  const int i0 = t + blockIdx.x * 32;
  for (int idx = threadIdx.x; idx < 32 * 64; idx += blockDim.x) {
    const int ii = idx % 32, kk = idx / 32;
    const int i = i0 + ii;
    const int c = kk < 32 ? kk : kk - 32;
    float v = 0.f;
    if (i < n && c < nbp) v = VW[i + (long long)(kk < 32 ? c : nbp + c) * n];
    tile[ii][kk] = v;
  }
  __syncthreads();
  for (int idx = threadIdx.x; idx < 32 * 64; idx += blockDim.x) {
    const int kk = idx % 64, ii = idx / 64;
    const int i = i0 + ii;
    if (i < n) VWt[kk + (long long)i * 64] = tile[ii][kk];
  }
}

}  // namespace gla

namespace {
using namespace gla;

// The trailing update A[t:, t:] -= V W' + W V' (lower tiles) as two K
// segments of the 3xTF32 tensor-core GEMM: A operand rows = V / W rows
// (K-major through VWt), B operand columns = W / V rows. False when the
// shapes do not allow the tensor maps (the SIMT GEMM then runs).
bool sytrd_update_tc(SytrdPlan& sp, float* A, long long lda, int n, int t, int nbp, cudaStream_t st,
                     cudaError_t* err) {
  *err = cudaSuccess;
  if (sp.VWt == nullptr || kSytrdNB != 32) return false;
  CUtensorMap m;
  if (!tc::tc_make_map(&m, sp.VWt, 64, n, 64, tc::kBM)) return false;
  k_vw_transpose<<<(n - t + 31) / 32, 256, 0, st>>>((const float*)sp.VW, n, nbp, t, sp.VWt);
  if ((*err = cudaGetLastError()) != cudaSuccess) return true;
  tc::TcArgs g{};
  g.M = g.N = n - t;
  g.nseg = 2;
  g.K[0] = g.K[1] = 32;
  g.a_x[0] = 0;   // V
  g.b_x[0] = 32;  // W
  g.a_x[1] = 32;  // W
  g.b_x[1] = 0;   // V
  g.a_y = g.b_y = t;
  g.D = A + t + (long long)t * lda;
  g.ldd = lda;
  g.alpha = -1.f;
  g.beta = 1.f;
  g.lower = 1;
  g.err = sp.err;
  *err = tc::tc_gemm_launch(m, m, g, 1, st);
  return true;
}

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
  a.ustart = sp.ustart;
  a.nTC = sp.nTC;
  a.bar = sp.bar;
  a.err = sp.err;
  T* VW = (T*)sp.VW;
  unsigned bar_base = 0;
  const int nsteps = n - 1;  // reflectors 0 .. n-2
  for (int k0 = 0; k0 < nsteps; k0 += kSytrdNB) {
    const int nbp = std::min(kSytrdNB, nsteps - k0);
    a.k0 = k0;
    a.nbp = nbp;
    a.V = VW;
    a.W = VW + (long long)nbp * n;
    a.bar_base = bar_base;
    bar_base += 2u * (unsigned)nbp * (unsigned)sp.G;  // barriers per launch: 1 + nbp + (nbp - 1)
    void* args[] = {(void*)&a};
    err = cudaLaunchCooperativeKernel((const void*)k_sytrd_panel<T>, dim3(sp.G), dim3(kPT), args,
                                      2 * (size_t)panel_rows(k0, n, sp.G) * kSytrdNB * sizeof(T), st);
    if (err != cudaSuccess) return err;
    const int t = k0 + nbp;
    if (t < n - 1) {  // trailing update A[t:, t:] -= V W' + W V' (lower tiles)
      if (sizeof(T) == 4 && sytrd_update_tc(sp, (float*)A, lda, n, t, nbp, st, &err)) {
        if (err != cudaSuccess) return err;
        continue;
      }
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

cudaError_t sytrd_plan_create(SytrdPlan** out, int n, bool f64, bool tc) {
  *out = nullptr;
  SytrdPlan* sp = new SytrdPlan();
  sp->n = n;
  sp->f64 = f64;
  int dev = 0, nsm = 0, per = 0;
  cudaError_t err = cudaGetDevice(&dev);
  if (err == cudaSuccess) err = cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  // phase B's V / W row cache: 2 rows-per-CTA x kSytrdNB values. The limit
  // is a property of the kernel, shared by every plan: always the largest
  // order's, so that a plan made later never lowers it below an earlier
  // plan's launches.
  const void* kfn = f64 ? (const void*)k_sytrd_panel<double> : (const void*)k_sytrd_panel<float>;
  const int vwbytes = 2 * panel_rows(0, kMaxTC * kTW, std::max(nsm, 1)) * kSytrdNB * (f64 ? 8 : 4);
  if (err == cudaSuccess) err = cudaFuncSetAttribute(kfn, cudaFuncAttributeMaxDynamicSharedMemorySize, vwbytes);
  if (err == cudaSuccess) err = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, kfn, kPT, vwbytes);
  if (err == cudaSuccess && per < 1) err = cudaErrorCooperativeLaunchTooLarge;
  if (err != cudaSuccess) {
    delete sp;
    return err;
  }
  sp->G = nsm;  // one CTA per SM (co-residency of a cooperative launch)
  sp->nTC = (n + kTW - 1) / kTW;
  sp->nCH = (n + kRC - 1) / kRC;
  sp->nDCH = (n + kDotRows - 1) / kDotRows;
  std::vector<int> ustart(sp->nTC + 1);
  int total = 0;
  for (int J = 0; J < sp->nTC; J++) {
    ustart[J] = total;
    total += (n - J * kTW + kRC - 1) / kRC;  // chunks of tile column J
  }
  ustart[sp->nTC] = total;
  std::vector<int> bk(4 * kSytrdNB);
  const int last = (n - 1) % kSytrdNB == 0 ? kSytrdNB : (n - 1) % kSytrdNB;
  for (int kk = 0; kk < 2 * kSytrdNB; kk++) bk[kk] = kk < kSytrdNB ? kSytrdNB + kk : kk - kSytrdNB;
  for (int kk = 0; kk < 2 * last; kk++) bk[2 * kSytrdNB + kk] = kk < last ? last + kk : kk - last;
  const size_t el = f64 ? 8 : 4;
  auto alloc = [&](void** p, size_t bytes) {
    if (err == cudaSuccess) err = cudaMalloc(p, std::max<size_t>(bytes, 16));
  };
  alloc((void**)&sp->ustart, sizeof(int) * ustart.size());
  alloc(&sp->P, el * (size_t)sp->nTC * n);
  alloc(&sp->Qp, el * (size_t)sp->nCH * n);
  alloc(&sp->normp, el * sp->G);
  alloc(&sp->qfp, el * sp->G);
  alloc(&sp->dots, el * 3 * kSytrdNB * sp->nDCH);
  alloc(&sp->VW, el * (size_t)n * 2 * kSytrdNB);
  alloc((void**)&sp->bkidx, sizeof(int) * bk.size());
  alloc((void**)&sp->bar, 2 * sizeof(unsigned));
  alloc((void**)&sp->err, sizeof(int));
  if (err == cudaSuccess)
    err = cudaMemcpy(sp->ustart, ustart.data(), sizeof(int) * ustart.size(), cudaMemcpyHostToDevice);
  if (err == cudaSuccess) err = cudaMemcpy(sp->bkidx, bk.data(), sizeof(int) * bk.size(), cudaMemcpyHostToDevice);
  if (err == cudaSuccess) err = cudaMemset(sp->VW, 0, el * (size_t)n * 2 * kSytrdNB);
  if (err == cudaSuccess && !f64 && tc && tc::tc_available()) alloc((void**)&sp->VWt, sizeof(float) * 64 * (size_t)n);
  if (err != cudaSuccess) {
    sytrd_plan_destroy(sp);
    return err;
  }
  *out = sp;
  return cudaSuccess;
}

void sytrd_plan_destroy(SytrdPlan* sp) {
  if (!sp) return;
  cudaFree(sp->ustart);
  cudaFree(sp->P);
  cudaFree(sp->Qp);
  cudaFree(sp->normp);
  cudaFree(sp->qfp);
  cudaFree(sp->dots);
  cudaFree(sp->VW);
  cudaFree(sp->VWt);
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
