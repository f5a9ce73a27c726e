// Divide-and-conquer eigensolver for one large symmetric tridiagonal matrix
// (the large-order replacement of the reference's eigQL! on the
// SymTridiagonal, src/eigenSelfAdjoint.jl:221-288, which costs ~6n^3 flops of
// rotations; the eigenvalues and eigenvectors are the same up to rounding and
// eigenvector signs).
//
// Cuppen's splitting: T = diag(T1, T2) + rho u u' with u = e_p + sign(beta)
// e_{p+1} at every split (beta = e[p], rho = |beta|, T1's last and T2's
// first diagonal entries reduced by rho). Leaves (orders <= kLeafMax) are
// solved by the batched small-matrix QL path. A merge of two solved halves
// Q1' T1 Q1 = D1, Q2' T2 Q2 = D2 is the rank-one problem D + rho z z' with
// z = [last row of Q1; sign(beta) first row of Q2] / sqrt(2), rho = 2|beta|:
//   1. sort D (merge of two ascending lists) and deflate: entries with
//      rho |z_i| <= tol keep (d_i, e_i); pairs of close entries are rotated
//      (Givens on the two columns of Q) until one z component vanishes;
//   2. the k remaining roots of the secular equation
//      f(l) = 1/rho + sum z_i^2 / (d_i - l) = 0, one per interval, each root
//      by one warp with a two-pole rational model step (Li's "middle way")
//      inside a bisection bracket, stored as an offset tau from its nearer pole;
//   3. Gu-Eisenstat: z is recomputed from the roots (zhat_i^2 =
//      prod_j (l_j - d_i) / (rho prod_{j!=i} (d_j - d_i))) so that the
//      eigenvectors u_j = (zhat_i / (d_i - l_j))_i / norm are orthogonal to
//      working precision;
//   4. Q := diag(Q1, Q2) [rotated columns] U by two GEMMs (rows of the top
//      half over top/mixed columns, rows of the bottom half over
//      bottom/mixed columns), written straight to the sorted output columns;
//      deflated columns are copied.
// All merges of one tree level run in the same launches; sizes that are
// only known on the device (k, the GEMM column lists) reach the GEMM through
// device-side descriptors, so the sequence needs no host synchronisation.
#include <cuda_runtime.h>

#include <algorithm>
#include <mutex>
#include <vector>

#include "gla_common.cuh"
#include "gla_large.h"
#include "gla_launch.h"
#include "gla_small.cuh"
#include "../../include/glagpu.h"

namespace gla {

constexpr int kLeafMax = 64;
constexpr int kPrepThreads = 1024;
constexpr int kPrepChunk = 1024;

template <class T>
struct dc_eps;
template <>
struct dc_eps<double> {
  static constexpr double u = 0x1p-53;
};
template <>
struct dc_eps<float> {
  static constexpr float u = 0x1p-24f;
};

struct MergeInfo {
  int o, m1, m2;
  int k, nf, nrot;
  int ktop, kbot;
  int fail;
  int pad;
};

template <class T>
struct DcArrays {
  T* dd;        // eigenvalues of the current blocks (ascending per block)
  const T* e;   // original off-diagonal
  T *sD, *sZ;   // sorted D and z
  int* ssrc;    // local source column of each sorted entry
  int* zdef;    // z-deflation flag of each sorted entry
  int* ctype;   // per local column: 0 top, 1 bottom, 2 mixed
  T *kd, *kz;   // kept entries
  int* ksrc;
  T* fd;        // deflated eigenvalues
  int* fsrc;
  T *rc, *rs;   // rotation list
  int *rp, *rt;
  int* org;     // secular roots: origin (kept index) and offset
  T* tau;
  T* zh;
  int *opos_k, *opos_f;  // absolute output column of kept / deflated entries
  int *gt_a, *gt_b, *gb_a, *gb_b;  // GEMM gather lists
  T* U;         // per-merge k x k eigenvector matrices
  long long u_stride;  // U offset of a merge = o * u_stride
  T *Zin, *Zout;
  long long ld;
  MergeInfo* info;
  GemmDesc* gdesc;
};

// ---------------------------------------------------------------- leaves

template <class T>
__global__ void k_dc_split(const T* __restrict__ d, const T* __restrict__ e, T* __restrict__ dm, T* __restrict__ em,
                           int n, const int* __restrict__ splits, int nsplit) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    T di = d[i];
    T ei = i + 1 < n ? e[i] : T(0);
    for (int s = 0; s < nsplit; s++) {
      const int p = splits[s];  // split between rows p-1 and p
      if (i == p - 1) {
        di -= fabs(e[p - 1]);
        ei = T(0);
      }
      if (i == p) di -= fabs(e[p - 1]);
    }
    dm[i] = di;
    em[i] = ei;
  }
}

// Leaf eigenvectors (packed L x L blocks) into the diagonal blocks of Z.
template <class T>
__global__ void k_dc_leaf_copy(const T* __restrict__ Qleaf, const int* __restrict__ leaf_o,
                               const int* __restrict__ leaf_m, const long long* __restrict__ leaf_a, T* __restrict__ Z,
                               long long ld) {
  const int b = blockIdx.x, o = leaf_o[b], m = leaf_m[b];
  const T* Q = Qleaf + leaf_a[b];
  for (int idx = threadIdx.x; idx < m * m; idx += blockDim.x) {
    const int i = idx % m, j = idx / m;
    Z[(o + i) + (long long)(o + j) * ld] = Q[idx];
  }
}

// ---------------------------------------------------------------- merge: deflation

template <class T>
__global__ void __launch_bounds__(kPrepThreads) k_dc_prep(DcArrays<T> a) {
  MergeInfo* mi = a.info + blockIdx.x;
  const int o = mi->o, m1 = mi->m1, m2 = mi->m2, m = m1 + m2;
  const int tid = threadIdx.x;
  const long long ld = a.ld;
  const T beta = a.e[o + m1 - 1];
  const T sgn = beta < T(0) ? T(-1) : T(1);
  const T rho = T(2) * fabs(beta);
  const T rs2 = T(0.70710678118654752440);
  __shared__ T sred[kPrepThreads / 32];
  // z, merged order, max |D|
  T dmax = T(0);
  for (int i = tid; i < m; i += kPrepThreads) {
    const T di = a.dd[o + i];
    T zi;
    int rank;
    if (i < m1) {
      zi = a.Zin[(o + m1 - 1) + (long long)(o + i) * ld] * rs2;
      int lo = 0, hi = m2;  // entries of the bottom half strictly below di
      while (lo < hi) {
        const int mid = (lo + hi) >> 1;
        if (a.dd[o + m1 + mid] < di) lo = mid + 1; else hi = mid;
      }
      rank = i + lo;
    } else {
      zi = sgn * a.Zin[(o + m1) + (long long)(o + i) * ld] * rs2;
      int lo = 0, hi = m1;  // entries of the top half at or below di
      while (lo < hi) {
        const int mid = (lo + hi) >> 1;
        if (a.dd[o + mid] <= di) lo = mid + 1; else hi = mid;
      }
      rank = (i - m1) + lo;
    }
    a.sD[o + rank] = di;
    a.sZ[o + rank] = zi;
    a.ssrc[o + rank] = i;
    a.ctype[o + i] = i < m1 ? 0 : 1;
    dmax = fmax(dmax, fabs(di));
  }
#pragma unroll
  for (int s = 16; s > 0; s >>= 1) dmax = fmax(dmax, __shfl_xor_sync(0xffffffffu, dmax, s));
  if ((tid & 31) == 0) sred[tid >> 5] = dmax;
  __syncthreads();
  dmax = T(0);
  for (int i = 0; i < kPrepThreads / 32; i++) dmax = fmax(dmax, sred[i]);
  const T tol = T(8) * dc_eps<T>::u * fmax(dmax, rho);
  for (int t = tid; t < m; t += kPrepThreads) a.zdef[o + t] = rho * fabs(a.sZ[o + t]) <= tol;
  __syncthreads();

  // sequential pair deflation by thread 0 over chunks staged in shared memory
  __shared__ T cD[kPrepChunk], cZ[kPrepChunk];
  __shared__ int cS[kPrepChunk], cF[kPrepChunk];
  int k = 0, nf = 0, nr = 0;
  T Dp = T(0), zp = T(0);
  int sp = -1;
  for (int c0 = 0; c0 < m; c0 += kPrepChunk) {
    const int cn = min(kPrepChunk, m - c0);
    __syncthreads();
    for (int t = tid; t < cn; t += kPrepThreads) {
      cD[t] = a.sD[o + c0 + t];
      cZ[t] = a.sZ[o + c0 + t];
      cS[t] = a.ssrc[o + c0 + t];
      cF[t] = a.zdef[o + c0 + t];
    }
    __syncthreads();
    if (tid == 0) {
      for (int t = 0; t < cn; t++) {
        const T Dt = cD[t], zt = cZ[t];
        const int st = cS[t];
        if (cF[t]) {
          a.fd[o + nf] = Dt;
          a.fsrc[o + nf] = st;
          nf++;
          continue;
        }
        if (sp < 0) {
          Dp = Dt;
          zp = zt;
          sp = st;
          continue;
        }
        const T r2 = zp * zp + zt * zt;
        if (fabs(Dt - Dp) * fabs(zp * zt) <= tol * r2) {
          const T r = sqrt(r2);
          const T cs = zt / r, sn = zp / r;
          a.rc[o + nr] = cs;
          a.rs[o + nr] = sn;
          a.rp[o + nr] = sp;
          a.rt[o + nr] = st;
          nr++;
          if (a.ctype[o + sp] != a.ctype[o + st]) {
            a.ctype[o + sp] = 2;
            a.ctype[o + st] = 2;
          }
          a.fd[o + nf] = cs * cs * Dp + sn * sn * Dt;
          a.fsrc[o + nf] = sp;
          nf++;
          Dp = sn * sn * Dp + cs * cs * Dt;
          zp = r;
          sp = st;
        } else {
          a.kd[o + k] = Dp;
          a.kz[o + k] = zp;
          a.ksrc[o + k] = sp;
          k++;
          Dp = Dt;
          zp = zt;
          sp = st;
        }
      }
    }
  }
  if (tid == 0) {
    if (sp >= 0) {
      a.kd[o + k] = Dp;
      a.kz[o + k] = zp;
      a.ksrc[o + k] = sp;
      k++;
    }
    mi->k = k;
    mi->nf = nf;
    mi->nrot = nr;
    mi->fail = 0;
  }
}

// Deflation rotations on the columns of Zin (rows of the merged block).
template <class T>
__global__ void k_dc_rot(DcArrays<T> a) {
  const MergeInfo mi = a.info[blockIdx.y];
  const int m = mi.m1 + mi.m2, o = mi.o;
  const int row = blockIdx.x * blockDim.x + threadIdx.x;
  if (mi.nrot == 0 || row >= m) return;
  T* Z = a.Zin + o + row;
  for (int r = 0; r < mi.nrot; r++) {
    const T c = a.rc[o + r], s = a.rs[o + r];
    T* pp = Z + (long long)(o + a.rp[o + r]) * a.ld;
    T* pt = Z + (long long)(o + a.rt[o + r]) * a.ld;
    const T qp = *pp, qt = *pt;
    *pp = c * qp - s * qt;
    *pt = s * qp + c * qt;
  }
}

// ---------------------------------------------------------------- merge: secular equation

template <class T>
__global__ void __launch_bounds__(256) k_dc_secular(DcArrays<T> a) {
  MergeInfo* mp = a.info + blockIdx.y;
  const int k = mp->k, o = mp->o;
  const int j = blockIdx.x * 8 + (threadIdx.x >> 5), lane = threadIdx.x & 31;
  if (j >= k) return;
  const T* __restrict__ D = a.kd + o;
  const T* __restrict__ Z = a.kz + o;
  const T rho = T(2) * fabs(a.e[o + mp->m1 - 1]);
  const T irho = T(1) / rho;
  const T eps = dc_eps<T>::u;
  if (k == 1) {
    if (lane == 0) {
      a.org[o] = 0;
      a.tau[o] = rho * Z[0] * Z[0];
    }
    return;
  }
  const bool last = j == k - 1;
  int og;
  T lo, hi;
  if (!last) {
    const T mid = T(0.5) * (D[j] + D[j + 1]);
    T f = T(0);
    for (int i = lane; i < k; i += 32) f += Z[i] * Z[i] / (D[i] - mid);
#pragma unroll
    for (int s = 16; s > 0; s >>= 1) f += __shfl_xor_sync(0xffffffffu, f, s);
    f += irho;
    if (f >= T(0)) {
      og = j;
      lo = T(0);
      hi = mid - D[j];
    } else {
      og = j + 1;
      lo = mid - D[j + 1];
      hi = T(0);
    }
  } else {
    og = j;
    T z2 = T(0);
    for (int i = lane; i < k; i += 32) z2 += Z[i] * Z[i];
#pragma unroll
    for (int s = 16; s > 0; s >>= 1) z2 += __shfl_xor_sync(0xffffffffu, z2, s);
    lo = T(0);
    hi = rho * z2 * (T(1) + T(4) * eps);
  }
  const T Dorg = D[og];
  const T dL = D[j] - Dorg;
  const T dR = last ? T(0) : D[j + 1] - Dorg;
  T tau = T(0.5) * (lo + hi);
  bool conv = false;
  for (int it = 0; it < 100; it++) {
    T psi = T(0), dpsi = T(0), phi = T(0), dphi = T(0);
    for (int i = lane; i < k; i += 32) {
      const T del = (D[i] - Dorg) - tau;
      const T t = Z[i] / del;
      const T term = Z[i] * t, der = t * t;
      if (i <= j) {
        psi += term;
        dpsi += der;
      } else {
        phi += term;
        dphi += der;
      }
    }
#pragma unroll
    for (int s = 16; s > 0; s >>= 1) {
      psi += __shfl_xor_sync(0xffffffffu, psi, s);
      dpsi += __shfl_xor_sync(0xffffffffu, dpsi, s);
      phi += __shfl_xor_sync(0xffffffffu, phi, s);
      dphi += __shfl_xor_sync(0xffffffffu, dphi, s);
    }
    const T g = irho + psi + phi;
    const T gtol = eps * (irho + (T(8) + T(k) / T(16)) * (fabs(psi) + fabs(phi)) + T(2) * fabs(tau) * (dpsi + dphi));
    if (fabs(g) <= gtol) {
      conv = true;
      break;
    }
    if (g < T(0)) lo = tau; else hi = tau;
    if (hi - lo <= T(4) * eps * fmax(fabs(lo), fabs(hi))) {
      conv = true;
      break;
    }
    const T DL = dL - tau;
    T eta;
    bool ok = false;
    if (!last) {
      const T DR = dR - tau;
      const T c = g - DL * dpsi - DR * dphi;
      const T qa = c * (DL + DR) + DL * DL * dpsi + DR * DR * dphi;
      const T qb = DL * DR * g;
      if (fabs(c) <= eps * fabs(qa)) {
        if (qa != T(0)) {
          eta = qb / qa;
          ok = true;
        }
      } else {
        T disc = qa * qa - T(4) * qb * c;
        disc = disc > T(0) ? sqrt(disc) : T(0);
        const T tq = qa >= T(0) ? T(0.5) * (qa + disc) : T(0.5) * (qa - disc);
        const T e1 = tq / c;
        const T e2 = tq != T(0) ? qb / tq : e1;
        const bool in1 = e1 > DL && e1 < DR, in2 = e2 > DL && e2 < DR;
        if (in1 != in2) {
          eta = in1 ? e1 : e2;
          ok = true;
        } else if (in1) {
          eta = fabs(e1) < fabs(e2) ? e1 : e2;
          ok = true;
        }
      }
    } else {
      const T c = g - DL * dpsi;
      if (c > T(0)) {
        eta = DL + DL * DL * dpsi / c;
        ok = true;
      }
    }
    T tn = ok ? tau + eta : T(0.5) * (lo + hi);
    if (!(tn > lo && tn < hi)) tn = T(0.5) * (lo + hi);
    const bool small_step = fabs(tn - tau) <= T(2) * eps * fabs(tau);
    tau = tn;
    if (small_step) {
      conv = true;
      break;
    }
  }
  if (lane == 0) {
    a.org[o + j] = og;
    a.tau[o + j] = tau;
    if (!conv) atomicExch(&mp->fail, 1);
  }
}

// zhat_i (one warp per i): product of ratios, each in (0, 1].
template <class T>
__global__ void __launch_bounds__(256) k_dc_zhat(DcArrays<T> a) {
  const MergeInfo mi = a.info[blockIdx.y];
  const int k = mi.k, o = mi.o;
  const int i = blockIdx.x * 8 + (threadIdx.x >> 5), lane = threadIdx.x & 31;
  if (i >= k) return;
  const T* __restrict__ D = a.kd + o;
  const T rho = T(2) * fabs(a.e[o + mi.m1 - 1]);
  const T Di = D[i];
  // lambda_j - D_i = tau_j - (D_i - D_org(j))
  T prod = T(1);
  for (int j = lane; j < k; j += 32) {
    const int og = a.org[o + j];
    const T num = a.tau[o + j] - (Di - D[og]);
    T den;
    if (j == k - 1)
      den = rho;
    else
      den = j < i ? D[j] - Di : D[j + 1] - Di;
    prod *= num / den;
  }
#pragma unroll
  for (int s = 16; s > 0; s >>= 1) prod *= __shfl_xor_sync(0xffffffffu, prod, s);
  if (lane == 0) {
    const T zi = a.kz[o + i];
    const T zh = sqrt(fabs(prod));
    a.zh[o + i] = zi < T(0) ? -zh : zh;
  }
}

// Column j of U: u_i = zhat_i / (D_i - lambda_j), normalised.
template <class T>
__global__ void __launch_bounds__(256) k_dc_vec(DcArrays<T> a) {
  const MergeInfo mi = a.info[blockIdx.y];
  const int k = mi.k, o = mi.o, j = blockIdx.x;
  if (j >= k) return;
  const T* __restrict__ D = a.kd + o;
  const int og = a.org[o + j];
  const T Dorg = D[og], tau = a.tau[o + j];
  T* U = a.U + (long long)o * a.u_stride + (long long)j * k;
  __shared__ T sred[8];
  T ss = T(0);
  for (int i = threadIdx.x; i < k; i += 256) {
    const T u = a.zh[o + i] / ((D[i] - Dorg) - tau);
    U[i] = u;
    ss = fma(u, u, ss);
  }
#pragma unroll
  for (int s = 16; s > 0; s >>= 1) ss += __shfl_xor_sync(0xffffffffu, ss, s);
  if ((threadIdx.x & 31) == 0) sred[threadIdx.x >> 5] = ss;
  __syncthreads();
  ss = T(0);
  for (int w = 0; w < 8; w++) ss += sred[w];
  const T inv = T(1) / sqrt(ss);
  for (int i = threadIdx.x; i < k; i += 256) U[i] *= inv;
}

// ---------------------------------------------------------------- merge: output order, GEMM lists

// Sorted order of the m eigenvalues of a merge (bitonic sort of packed keys
// in shared memory), output columns, the new dd, and the GEMM descriptors.
template <class T>
__global__ void __launch_bounds__(1024) k_dc_post(DcArrays<T> a, int mpow2) {
  MergeInfo* mp = a.info + blockIdx.x;
  const int o = mp->o, m1 = mp->m1, m = m1 + mp->m2, k = mp->k;
  const int tid = threadIdx.x;
  extern __shared__ unsigned char smraw[];
  unsigned long long* key = reinterpret_cast<unsigned long long*>(smraw);
  int* tag = reinterpret_cast<int*>(key + mpow2);
  // eigenvalue of entry t: kept roots first (t < k), then deflated
  for (int t = tid; t < mpow2; t += 1024) {
    if (t < m) {
      T v = t < k ? a.kd[o + a.org[o + t]] + a.tau[o + t] : a.fd[o + (t - k)];
      key[t] = sort_key(v);
      tag[t] = t;
    } else {
      key[t] = ~0ull;
      tag[t] = 0x7fffffff;
    }
  }
  __syncthreads();
  for (int size = 2; size <= mpow2; size <<= 1) {
    for (int stride = size >> 1; stride > 0; stride >>= 1) {
      for (int t = tid; t < mpow2 / 2; t += 1024) {
        const int lo = 2 * t - (t & (stride - 1));
        const int hi = lo + stride;
        const bool up = (lo & size) == 0;
        const unsigned long long kl = key[lo], kh = key[hi];
        const int tl = tag[lo], th = tag[hi];
        const bool gt = kl > kh || (kl == kh && tl > th);
        if (gt == up) {
          key[lo] = kh;
          key[hi] = kl;
          tag[lo] = th;
          tag[hi] = tl;
        }
      }
      __syncthreads();
    }
  }
  for (int pos = tid; pos < m; pos += 1024) {
    const int t = tag[pos];
    T v;
    if (t < k) {
      v = a.kd[o + a.org[o + t]] + a.tau[o + t];
      a.opos_k[o + t] = o + pos;
    } else {
      v = a.fd[o + (t - k)];
      a.opos_f[o + (t - k)] = o + pos;
    }
    a.dd[o + pos] = v;
  }
  // GEMM gather lists: ordered compaction of kept entries by column type
  __shared__ int cnt_t[1024], cnt_b[1024];
  const int per = (k + 1023) / 1024;
  const int b0 = min(k, tid * per), b1 = min(k, b0 + per);
  int ct = 0, cb = 0;
  for (int i = b0; i < b1; i++) {
    const int ty = a.ctype[o + a.ksrc[o + i]];
    ct += ty != 1;
    cb += ty != 0;
  }
  cnt_t[tid] = ct;
  cnt_b[tid] = cb;
  __syncthreads();
  if (tid == 0) {
    int st = 0, sb = 0;
    for (int i = 0; i < 1024; i++) {
      const int x = cnt_t[i], y = cnt_b[i];
      cnt_t[i] = st;
      cnt_b[i] = sb;
      st += x;
      sb += y;
    }
    mp->ktop = st;
    mp->kbot = sb;
  }
  __syncthreads();
  ct = cnt_t[tid];
  cb = cnt_b[tid];
  for (int i = b0; i < b1; i++) {
    const int src = a.ksrc[o + i];
    const int ty = a.ctype[o + src];
    if (ty != 1) {
      a.gt_a[o + ct] = o + src;
      a.gt_b[o + ct] = i;
      ct++;
    }
    if (ty != 0) {
      a.gb_a[o + cb] = o + src;
      a.gb_b[o + cb] = i;
      cb++;
    }
  }
  __syncthreads();
  if (tid == 0) {
    GemmDesc g{};
    g.m = m1;
    g.n = k;
    g.k = mp->ktop;
    g.A = a.Zin + o;
    g.lda = a.ld;
    g.B = a.U + (long long)o * a.u_stride;
    g.ldb = k > 0 ? k : 1;
    g.C = a.Zout + o;
    g.ldc = a.ld;
    g.a_kidx = a.gt_a + o;
    g.b_kidx = a.gt_b + o;
    g.c_nidx = a.opos_k + o;
    g.alpha = 1.0;
    g.beta = 0.0;
    a.gdesc[2 * blockIdx.x] = g;
    g.m = m - m1;
    g.k = mp->kbot;
    g.A = a.Zin + o + m1;
    g.C = a.Zout + o + m1;
    g.a_kidx = a.gb_a + o;
    g.b_kidx = a.gb_b + o;
    a.gdesc[2 * blockIdx.x + 1] = g;
  }
}

// Deflated columns: full column of the merged block copied to its output column.
template <class T>
__global__ void k_dc_copydefl(DcArrays<T> a) {
  const MergeInfo mi = a.info[blockIdx.y];
  const int p = blockIdx.x;
  if (p >= mi.nf) return;
  const int o = mi.o, m = mi.m1 + mi.m2;
  const T* src = a.Zin + o + (long long)(o + a.fsrc[o + p]) * a.ld;
  T* dst = a.Zout + o + (long long)a.opos_f[o + p] * a.ld;
  for (int i = threadIdx.x; i < m; i += blockDim.x) dst[i] = src[i];
}

template <class T>
__global__ void k_dc_fail(const MergeInfo* info, int nm, int* out) {
  int f = 0;
  for (int i = threadIdx.x; i < nm; i += blockDim.x) f |= info[i].fail;
  f = __syncthreads_or(f);
  if (threadIdx.x == 0 && f) *out = 1;
}

// ---------------------------------------------------------------- host side

struct DcLevel {
  int first;  // index of the level's first merge in the merge table
  int count;
  int mmax, m1max;
};

struct DcPlan {
  int n = 0;
  bool f64 = true;
  std::vector<DcLevel> levels;
  int nmerge = 0;
  int nleaf = 0;
  MergeInfo* d_info = nullptr;
  std::vector<MergeInfo> h_info;
  GemmDesc* d_gdesc = nullptr;
  int* d_splits = nullptr;
  int nsplit = 0;
  int *d_leaf_o = nullptr, *d_leaf_m = nullptr;
  long long* d_leaf_a = nullptr;
  gla_plan_s* leafplan = nullptr;
  void* arrays = nullptr;   // scalar arrays of n entries
  void* U = nullptr;
  void* Z1 = nullptr;       // second eigenvector buffer (n x n)
  void* Qleaf = nullptr;    // packed leaf eigenvectors
  void* dm = nullptr;       // split-modified d, e
  void* em = nullptr;
  int* d_fail = nullptr;
  long long u_stride = 0;
  DcArrays<double> a64{};
  DcArrays<float> a32{};
};

}  // namespace gla

extern "C" int gla_plan_create(gla_plan_s** plan_out, int precision, char jobz, char uplo, int64_t batch,
                               const int64_t* n, double tol, int flags);
extern "C" int gla_plan_destroy(gla_plan_s* p);

namespace gla {

namespace {

// Every leaf sits at depth `leaves_at` (sizes differ by at most one), so each
// tree level reads one eigenvector buffer and writes the other.
void build_tree(int o, int m, int depth, int leaves_at, std::vector<std::vector<MergeInfo>>& by_depth,
                std::vector<int>& leaf_o, std::vector<int>& leaf_m, std::vector<int>& splits) {
  if (depth == leaves_at) {
    leaf_o.push_back(o);
    leaf_m.push_back(m);
    return;
  }
  const int m1 = m / 2, m2 = m - m1;
  build_tree(o, m1, depth + 1, leaves_at, by_depth, leaf_o, leaf_m, splits);
  build_tree(o + m1, m2, depth + 1, leaves_at, by_depth, leaf_o, leaf_m, splits);
  if ((int)by_depth.size() <= depth) by_depth.resize(depth + 1);
  MergeInfo mi{};
  mi.o = o;
  mi.m1 = m1;
  mi.m2 = m2;
  by_depth[depth].push_back(mi);
  splits.push_back(o + m1);
}

template <class T>
void carve_arrays(DcPlan& p, DcArrays<T>& a, char* base, int n) {
  size_t off = 0;
  auto take = [&](size_t bytes) {
    char* q = base + off;
    off += (bytes + 255) / 256 * 256;
    return q;
  };
  a.sD = (T*)take(sizeof(T) * n);
  a.sZ = (T*)take(sizeof(T) * n);
  a.ssrc = (int*)take(sizeof(int) * n);
  a.zdef = (int*)take(sizeof(int) * n);
  a.ctype = (int*)take(sizeof(int) * n);
  a.kd = (T*)take(sizeof(T) * n);
  a.kz = (T*)take(sizeof(T) * n);
  a.ksrc = (int*)take(sizeof(int) * n);
  a.fd = (T*)take(sizeof(T) * n);
  a.fsrc = (int*)take(sizeof(int) * n);
  a.rc = (T*)take(sizeof(T) * n);
  a.rs = (T*)take(sizeof(T) * n);
  a.rp = (int*)take(sizeof(int) * n);
  a.rt = (int*)take(sizeof(int) * n);
  a.org = (int*)take(sizeof(int) * n);
  a.tau = (T*)take(sizeof(T) * n);
  a.zh = (T*)take(sizeof(T) * n);
  a.opos_k = (int*)take(sizeof(int) * n);
  a.opos_f = (int*)take(sizeof(int) * n);
  a.gt_a = (int*)take(sizeof(int) * n);
  a.gt_b = (int*)take(sizeof(int) * n);
  a.gb_a = (int*)take(sizeof(int) * n);
  a.gb_b = (int*)take(sizeof(int) * n);
  a.U = (T*)p.U;
  a.u_stride = p.u_stride;
  a.info = p.d_info;
  a.gdesc = p.d_gdesc;
}

size_t arrays_bytes(int n, size_t el) { return 32 * ((el * n + 255) / 256 * 256); }

template <class T>
int dc_run(DcPlan& p, T* d, const T* e, T* Z, int* info, cudaStream_t st) {
  const int n = p.n;
  const long long ldz = n;
  DcArrays<T>& a = *reinterpret_cast<DcArrays<T>*>(sizeof(T) == 8 ? (void*)&p.a64 : (void*)&p.a32);
  cudaError_t err;
#define DC_CUDA(x)                                \
  do {                                            \
    if ((err = (x)) != cudaSuccess) return -1000 - (int)err; \
  } while (0)
  DC_CUDA(cudaMemsetAsync(p.d_fail, 0, sizeof(int), st));
  // leaves
  k_dc_split<T><<<(n + 255) / 256, 256, 0, st>>>(d, e, (T*)p.dm, (T*)p.em, n, p.d_splits, p.nsplit);
  DC_CUDA(cudaGetLastError());
  const int tc = sizeof(T) == 8 ? kF64 : kF32;
  int rc = plan_stev_batched(p.leafplan, tc, p.dm, p.em, p.Qleaf, d, info, st);
  if (rc) return rc;
  // Z buffers: the ping-pong order is fixed so that the last level writes Z
  const int nlev = (int)p.levels.size();
  T* bufs[2] = {Z, (T*)p.Z1};
  T* zin = bufs[nlev % 2];
  // off-diagonal blocks of every merge must read as zero
  DC_CUDA(cudaMemsetAsync(Z, 0, sizeof(T) * (size_t)n * n, st));
  DC_CUDA(cudaMemsetAsync(p.Z1, 0, sizeof(T) * (size_t)n * n, st));
  k_dc_leaf_copy<T><<<p.nleaf, 256, 0, st>>>((const T*)p.Qleaf, p.d_leaf_o, p.d_leaf_m, p.d_leaf_a, zin, ldz);
  DC_CUDA(cudaGetLastError());
  a.dd = d;
  a.e = e;
  a.ld = ldz;
  for (int L = 0; L < nlev; L++) {
    const DcLevel& lv = p.levels[L];
    T* zout = (zin == bufs[0]) ? bufs[1] : bufs[0];
    DcArrays<T> al = a;
    al.Zin = zin;
    al.Zout = zout;
    al.info = p.d_info + lv.first;
    al.gdesc = p.d_gdesc + 2 * lv.first;
    k_dc_prep<T><<<lv.count, kPrepThreads, 0, st>>>(al);
    DC_CUDA(cudaGetLastError());
    k_dc_rot<T><<<dim3((lv.mmax + 255) / 256, lv.count), 256, 0, st>>>(al);
    DC_CUDA(cudaGetLastError());
    k_dc_secular<T><<<dim3((lv.mmax + 7) / 8, lv.count), 256, 0, st>>>(al);
    DC_CUDA(cudaGetLastError());
    k_dc_zhat<T><<<dim3((lv.mmax + 7) / 8, lv.count), 256, 0, st>>>(al);
    DC_CUDA(cudaGetLastError());
    k_dc_vec<T><<<dim3(lv.mmax, lv.count), 256, 0, st>>>(al);
    DC_CUDA(cudaGetLastError());
    int mp2 = 1;
    while (mp2 < lv.mmax) mp2 <<= 1;
    const size_t psm = (size_t)mp2 * (sizeof(unsigned long long) + sizeof(int));
    k_dc_post<T><<<lv.count, 1024, psm, st>>>(al, mp2);
    DC_CUDA(cudaGetLastError());
    DC_CUDA(gemm_launch_grouped(sizeof(T) == 8, al.gdesc, 2 * lv.count, lv.m1max + 1, lv.mmax, st));
    k_dc_copydefl<T><<<dim3(lv.mmax, lv.count), 256, 0, st>>>(al);
    DC_CUDA(cudaGetLastError());
    k_dc_fail<T><<<1, 256, 0, st>>>(al.info, lv.count, p.d_fail);
    DC_CUDA(cudaGetLastError());
    zin = zout;
  }
#undef DC_CUDA
  return 0;
}

}  // namespace

int dc_plan_create(DcPlan** out, int n, bool f64, bool bisect_leaves) {
  *out = nullptr;
  DcPlan* p = new DcPlan();
  p->n = n;
  p->f64 = f64;
  std::vector<std::vector<MergeInfo>> by_depth;
  std::vector<int> leaf_o, leaf_m, splits;
  int depth = 0;
  while ((n + (1 << depth) - 1) >> depth > kLeafMax) depth++;
  build_tree(0, n, 0, depth, by_depth, leaf_o, leaf_m, splits);
  // levels bottom-up (deepest merges first)
  for (int dpt = (int)by_depth.size() - 1; dpt >= 0; dpt--) {
    DcLevel lv;
    lv.first = (int)p->h_info.size();
    lv.count = (int)by_depth[dpt].size();
    lv.mmax = 0;
    lv.m1max = 0;
    for (const MergeInfo& mi : by_depth[dpt]) {
      p->h_info.push_back(mi);
      lv.mmax = std::max(lv.mmax, mi.m1 + mi.m2);
      lv.m1max = std::max(lv.m1max, std::max(mi.m1, mi.m2));
    }
    if (lv.count) p->levels.push_back(lv);
  }
  p->nmerge = (int)p->h_info.size();
  p->nleaf = (int)leaf_o.size();
  p->nsplit = (int)splits.size();
  const size_t el = f64 ? 8 : 4;
  int mmax_all = 0;
  for (const DcLevel& lv : p->levels) mmax_all = std::max(mmax_all, lv.mmax);
  p->u_stride = std::max(1, mmax_all);
  std::vector<int64_t> lsz(leaf_m.begin(), leaf_m.end());
  std::vector<long long> leaf_a(p->nleaf);
  long long aoff = 0;
  for (int b = 0; b < p->nleaf; b++) {
    leaf_a[b] = aoff;
    aoff += (long long)leaf_m[b] * leaf_m[b];
  }
  int rc = gla_plan_create(&p->leafplan, f64 ? GLA_PREC_F64 : GLA_PREC_F32, 'V', 'L', p->nleaf, lsz.data(), 0.0,
                           (!f64 && bisect_leaves) ? GLA_FLAG_F32_BISECT : 0);
  if (rc) {
    delete p;
    return rc;
  }
  cudaError_t err = cudaSuccess;
  auto alloc = [&](void** q, size_t bytes) {
    if (err == cudaSuccess) err = cudaMalloc(q, std::max<size_t>(bytes, 16));
  };
  alloc((void**)&p->d_info, sizeof(MergeInfo) * std::max(1, p->nmerge));
  alloc((void**)&p->d_gdesc, sizeof(GemmDesc) * 2 * std::max(1, p->nmerge));
  alloc((void**)&p->d_splits, sizeof(int) * std::max(1, p->nsplit));
  alloc((void**)&p->d_leaf_o, sizeof(int) * p->nleaf);
  alloc((void**)&p->d_leaf_m, sizeof(int) * p->nleaf);
  alloc((void**)&p->d_leaf_a, sizeof(long long) * p->nleaf);
  alloc(&p->arrays, arrays_bytes(n, 8));
  alloc(&p->U, el * (size_t)n * p->u_stride);
  alloc(&p->Z1, el * (size_t)n * n);
  alloc(&p->Qleaf, el * (size_t)std::max<long long>(aoff, 1));
  alloc(&p->dm, el * n);
  alloc(&p->em, el * n);
  alloc((void**)&p->d_fail, sizeof(int));
  if (err == cudaSuccess && p->nmerge)
    err = cudaMemcpy(p->d_info, p->h_info.data(), sizeof(MergeInfo) * p->nmerge, cudaMemcpyHostToDevice);
  if (err == cudaSuccess && p->nsplit)
    err = cudaMemcpy(p->d_splits, splits.data(), sizeof(int) * p->nsplit, cudaMemcpyHostToDevice);
  if (err == cudaSuccess) err = cudaMemcpy(p->d_leaf_o, leaf_o.data(), sizeof(int) * p->nleaf, cudaMemcpyHostToDevice);
  if (err == cudaSuccess) err = cudaMemcpy(p->d_leaf_m, leaf_m.data(), sizeof(int) * p->nleaf, cudaMemcpyHostToDevice);
  if (err == cudaSuccess)
    err = cudaMemcpy(p->d_leaf_a, leaf_a.data(), sizeof(long long) * p->nleaf, cudaMemcpyHostToDevice);
  if (err == cudaSuccess) {
    // the limit is per kernel, not per plan: only ever raise it
    static std::mutex mu;
    static size_t raised[2] = {0, 0};
    int mp2 = 1;
    while (mp2 < mmax_all) mp2 <<= 1;
    const size_t psm = (size_t)mp2 * (sizeof(unsigned long long) + sizeof(int));
    std::lock_guard<std::mutex> lk(mu);
    if (psm > raised[f64]) {
      err = cudaFuncSetAttribute(f64 ? (const void*)k_dc_post<double> : (const void*)k_dc_post<float>,
                                 cudaFuncAttributeMaxDynamicSharedMemorySize, (int)psm);
      if (err == cudaSuccess) raised[f64] = psm;
    }
  }
  if (err != cudaSuccess) {
    dc_plan_destroy(p);
    return -1000 - (int)err;
  }
  if (f64)
    carve_arrays<double>(*p, p->a64, (char*)p->arrays, n);
  else
    carve_arrays<float>(*p, p->a32, (char*)p->arrays, n);
  *out = p;
  return 0;
}

void dc_plan_destroy(DcPlan* p) {
  if (!p) return;
  if (p->leafplan) gla_plan_destroy(p->leafplan);
  cudaFree(p->d_info);
  cudaFree(p->d_gdesc);
  cudaFree(p->d_splits);
  cudaFree(p->d_leaf_o);
  cudaFree(p->d_leaf_m);
  cudaFree(p->d_leaf_a);
  cudaFree(p->arrays);
  cudaFree(p->U);
  cudaFree(p->Z1);
  cudaFree(p->Qleaf);
  cudaFree(p->dm);
  cudaFree(p->em);
  cudaFree(p->d_fail);
  delete p;
}

// Z has leading dimension n.
int dc_enqueue(DcPlan* p, void* d, const void* e, void* Z, int* info, cudaStream_t st) {
  if (p->f64) return dc_run<double>(*p, (double*)d, (const double*)e, (double*)Z, info, st);
  return dc_run<float>(*p, (float*)d, (const float*)e, (float*)Z, info, st);
}

int* dc_fail_word(DcPlan* p) { return p->d_fail; }
int dc_leaf_count(const DcPlan* p) { return p->nleaf; }
size_t dc_plan_bytes(const DcPlan* p) {
  const size_t el = p->f64 ? 8 : 4;
  return arrays_bytes(p->n, 8) + el * (size_t)p->n * (p->u_stride + p->n);
}

}  // namespace gla
