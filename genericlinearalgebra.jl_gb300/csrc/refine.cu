// Eigenpair refinement of the FP32 eigenvectors back to FP64-class accuracy,
// one CTA per matrix (n <= 128). No counterpart in GenericLinearAlgebra.jl.
//
// Ogita-Aishima iteration (T. Ogita, K. Aishima, "Iterative refinement for
// symmetric eigenvalue decomposition", JJIAM 35 (2018), Algorithm 1):
//
//   R = I - X'X,  S = X'AX,  lam_i = s_ii / (1 - r_ii),
//   delta = 2 (||S - diag(lam)||_F + ||A||_F ||R||_F)
//   E_ij = (s_ij + lam_j r_ij) / (lam_j - lam_i)   if |lam_j - lam_i| > delta
//        = r_ij / 2                                 otherwise (and i == j)
//   X <- X + X E
//
// Eigenvalues closer than delta form clusters (runs of the sorted lam);
// within each cluster the columns are additionally rotated to the Ritz
// vectors of the projected pencil, Z = eig((I + R_JJ/2) S_JJ (I + R_JJ/2)),
// as in the clustered-eigenvalue extension of the same authors (JJIAM 36,
// 2019). The small symmetric eigenproblem is solved by cyclic Jacobi in
// FP32 after shifting by the cluster mean (its accuracy only needs to be
// relative to the cluster's spread; the next iteration restores the rest).
//
// Arithmetic: the products AX, X'(AX) and X'X are evaluated to double-float
// accuracy, ~2^-47 relative, on the tcgen05 tensor cores (tc_small.cuh: the
// Ozaki scheme with seven bf16 slices per operand) or, with
// GLA_FLAG_REFINE_SIMT, in double-float arithmetic (df64.cuh) on the FP32
// pipe; X E in FP32 (below); lam and the gaps in FP64.
//
// The first iteration exploits that X0 (the FP32 eigenvectors) holds exact
// floats. The update X <- X + X E is evaluated in FP32: its rounding error
// (<= 2^-24 |X E| per entry, |E| <= 1e-3) is a perturbation of the next
// iterate that the next iteration removes quadratically; from the second
// iteration on |E| <= 1e-8 and the error is below 1e-15.
#include "df64.cuh"
#include "gla_launch.h"
#include "gla_refine.h"
#include "small_tridiag.cuh"
#include "tc_small.cuh"
#include "tile_gemm.cuh"

namespace gla {

constexpr int kMaxRefineIters = 8;
constexpr int kJacobiSweeps = 15;

size_t refine_workspace_bytes(int64_t a_elems, int64_t, int64_t) {
  return (7 * sizeof(df64) + 4 * sizeof(float)) * (size_t)a_elems + 4096;
}

size_t refine_pcache_bytes() { return (size_t)tcs::kPCacheBytes; }

void refine_carve(RefineWork* rw, char* base, int64_t a_elems, int64_t, int64_t) {
  df64* p = reinterpret_cast<df64*>(base);
  rw->A2 = p;
  rw->X2 = p + a_elems;
  rw->Y2 = p + 2 * a_elems;
  rw->S2 = p + 3 * a_elems;
  rw->R2 = p + 4 * a_elems;
  rw->S0 = p + 5 * a_elems;
  rw->R0 = p + 6 * a_elems;
  rw->E = reinterpret_cast<float*>(p + 7 * a_elems);
  rw->J = rw->E + a_elems;
  rw->T = rw->J + 2 * a_elems;
  rw->err = reinterpret_cast<int*>(rw->T + a_elems);  // in the 4096-byte tail
}

GLA_DEV float block_sum_f(float v, float* red) {
  v = warp_sum(v);
  __syncthreads();
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
  __syncthreads();
  float s = 0;
  for (int i = 0; i < kRT / 32; i++) s += red[i];
  return s;
}

GLA_DEV float block_max_f(float v, float* red) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = fmaxf(v, __shfl_xor_sync(0xffffffffu, v, o));
  __syncthreads();
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
  __syncthreads();
  float s = 0;
  for (int i = 0; i < kRT / 32; i++) s = fmaxf(s, red[i]);
  return s;
}

// Cyclic Jacobi on the k x k symmetric C (column-major, ld k) by one warp;
// Z receives the eigenvectors. Off-diagonal Frobenius norm driven below
// 1e-7 of the total, or kJacobiSweeps sweeps.
GLA_DEV void jacobi_warp(int k, float* C, float* Z) {
  const int lane = threadIdx.x & 31;
  for (int idx = lane; idx < k * k; idx += 32) Z[idx] = (idx % (k + 1) == 0) ? 1.f : 0.f;
  __syncwarp();
  for (int sw = 0; sw < kJacobiSweeps; sw++) {
    float off = 0.f, tot = 0.f;
    for (int idx = lane; idx < k * k; idx += 32) {
      const float v = C[idx];
      tot += v * v;
      if (idx % (k + 1) != 0) off += v * v;
    }
    off = warp_sum(off);
    tot = warp_sum(tot);
    if (!(off > 1e-14f * tot)) break;
    for (int p = 0; p < k - 1; p++) {
      for (int q = p + 1; q < k; q++) {
        const float apq = C[q * k + p];
        if (apq == 0.f) continue;
        const float app = C[p * k + p], aqq = C[q * k + q];
        const float th = (aqq - app) / (2.f * apq);
        const float t = (th == 0.f) ? 1.f : copysignf(1.f, th) / (fabsf(th) + sqrtf(fmaf(th, th, 1.f)));
        const float c = rsqrtf(fmaf(t, t, 1.f)), s = t * c;
        __syncwarp();
        for (int r = lane; r < k; r += 32) {  // columns p, q
          const float cp = C[p * k + r], cq = C[q * k + r];
          C[p * k + r] = c * cp - s * cq;
          C[q * k + r] = s * cp + c * cq;
        }
        __syncwarp();
        for (int r = lane; r < k; r += 32) {  // rows p, q
          const float rp = C[r * k + p], rq = C[r * k + q];
          C[r * k + p] = c * rp - s * rq;
          C[r * k + q] = s * rp + c * rq;
          const float zp = Z[p * k + r], zq = Z[q * k + r];
          Z[p * k + r] = c * zp - s * zq;
          Z[q * k + r] = s * zp + c * zq;
        }
        __syncwarp();
      }
    }
  }
  __syncwarp();
}

// (i, j) = (idx mod n, idx div n) for idx < n^2 <= 2^14 by a float
// reciprocal: the quotient (idx + 1/2)/n stays >= 1/(2n) away from integers,
// far beyond the float rounding of the product.
GLA_DEV void split_idx(int idx, int n, float inv_n, int& i, int& j) {
  j = (int)(((float)idx + 0.5f) * inv_n);
  i = idx - j * n;
}

// The refinement of matrix mid by the whole CTA (kRT threads). TC: the three
// double-float products on the tensor cores through tcx (set up by the
// kernel), else on the FP32 pipe.
template <bool TC>
GLA_DEV void refine_body(int mid, const SmallDesc* __restrict__ descs, const double* __restrict__ A, int lower,
                         const float* __restrict__ X32, double* __restrict__ Vout, double* __restrict__ wout,
                         int* __restrict__ info, const int* __restrict__ scale_exp, const RefineWork& rw,
                         unsigned long long* __restrict__ stats, tcs::Ctx* tcx) {
  __shared__ df64 As[16 * kTP];
  __shared__ df64 Bs2[16 * kTP];
  __shared__ double lam[kSmallMaxN];
  __shared__ df64 lamdf[kSmallMaxN];
  __shared__ float red[kRT / 32];
  __shared__ unsigned long long keys[kSmallMaxN];
  __shared__ int rank[kSmallMaxN], ord[kSmallMaxN], cstart[kSmallMaxN + 1], cid[kSmallMaxN];
  __shared__ int ncl_s, flag_s, big_s;
  __shared__ unsigned brk_mask[kRT / 32];
  __shared__ double gred[kRT / 32];
  __shared__ double gmin_s, lmax_s;
  // scale exponents: A's rows, and the columns of [Y | X] (X's at expQ + n)
  __shared__ int expA[TC ? kSmallMaxN : 1], expQ[TC ? 2 * kSmallMaxN : 1];
  float* Bsf = reinterpret_cast<float*>(Bs2);
  const SmallDesc dsc = descs[mid];
  const int n = dsc.n, tid = threadIdx.x;
  const float inv_n = 1.f / (float)n;
  const size_t ao = dsc.a_off;
  const double* Ag = A + ao;
  double* V = Vout ? Vout + ao : nullptr;
  if (info[mid] < 0) {  // non-finite input, or (capture-safe plans) an unfinished chase
    for (int idx = tid; idx < n * n; idx += kRT)
      if (V) V[idx] = NAN;
    for (int i = tid; i < n; i += kRT) wout[dsc.w_off + i] = NAN;
    return;
  }
  const int se = scale_exp[mid];
  df64* A2 = rw.A2 + ao;
  df64* X = rw.X2 + ao;
  df64* Y = rw.Y2 + ao;
  df64* S = rw.S2 + ao;
  df64* R = rw.R2 + ao;
  df64* S0 = rw.S0 + ao;
  df64* R0 = rw.R0 + ao;
  float* E = rw.E + ao;
  float* jac = rw.J + 2 * ao;  // C and Z of a cluster (k*k each), k <= n
  float* T1 = rw.T + ao;       // X E
  const float* X0 = X32 + ao;
  float* Asf = reinterpret_cast<float*>(As);
  float an2 = 0.f;
  for (int idx = tid; idx < n * n; idx += kRT) {
    int i, k;
    split_idx(idx, n, inv_n, i, k);
    const double a = (lower ? (i >= k) : (i <= k)) ? Ag[idx] : Ag[(size_t)i * n + k];
    const df64 ad = df_from(ldexp(a, -se));
    A2[idx] = ad;
    an2 = fmaf(ad.hi, ad.hi, an2);
  }
  const float anorm = sqrtf(block_sum_f(an2, red));
  if (TC) tcs::col_exps(n, A2, expA);  // A is symmetric: its row exponents
  const df64 zero = df_make(0.f, 0.f);
  auto zinit = [&](int, int) { return zero; };
  df64* cS = S0;
  df64* cR = R0;
  bool converged = false;
  float emax_prev = 1e30f;
  for (int it = 0; it < kMaxRefineIters; it++) {
    if (TC) {
      // Y = A X; S = X'Y and R = I - X'X (upper triangles, mirrored); on the
      // first iteration X is X0, the FP32 eigenvectors (exact floats)
      df64* Sd = it == 0 ? S0 : S;
      df64* Rd = it == 0 ? R0 : R;
      const df64* Xc = X;
      auto xk = [&](int k, int j) { return it == 0 ? df_make(X0[(size_t)j * n + k], 0.f) : Xc[(size_t)j * n + k]; };
      auto xt = [&](int i, int k) { return it == 0 ? df_make(X0[(size_t)i * n + k], 0.f) : Xc[(size_t)i * n + k]; };
      int* expX = expQ + n;
      if (it == 0)
        tcs::col_exps(n, X0, expX);
      else
        tcs::col_exps(n, Xc, expX);
      tcs::gemm(
          *tcx, n, expA, expX, [&](int i, int k) { return A2[(size_t)k * n + i]; }, xk,
          [&](int i, int j, df64 v) { Y[(size_t)j * n + i] = v; }, false);
      tcs::col_exps(n, Y, expQ);
      // [S | X'X] = X' [Y | X] as one product (X' sliced once): columns j < n
      // give S, columns n + j give X'X; upper triangles, mirrored
      tcs::gemm(
          *tcx, n, 2 * n, expX, expQ, xt,
          [&](int k, int j) { return j < n ? Y[(size_t)j * n + k] : xk(k, j - n); },
          [&](int i, int j, df64 v) {
            if (j < n) {
              if (i <= j) {
                Sd[(size_t)j * n + i] = v;
                Sd[(size_t)i * n + j] = v;
              }
            } else {
              const int jj = j - n;
              if (i <= jj) {
                const df64 r = df_add(df_make(i == jj ? 1.f : 0.f, 0.f), df_neg(v));
                Rd[(size_t)jj * n + i] = r;
                Rd[(size_t)i * n + jj] = r;
              }
            }
          },
          false);
      if (!tcs::ok(*tcx)) break;  // a tensor-core wait ran out: reported as not converged
      cS = Sd;
      cR = Rd;
    } else if (it == 0) {
      // ---- first iteration on the FP32 eigenvectors X0 (exact floats)
      tile_gemm_df<float>(
          n, [&](int i, int k) { return A2[(size_t)k * n + i]; }, [&](int k, int j) { return X0[(size_t)j * n + k]; },
          zinit, [&](int i, int j, df64 v) { Y[(size_t)j * n + i] = v; }, As, Bsf, false);
      // S0 = X0'Y computed as (Y'X0) (symmetric): upper triangle, mirrored
      tile_gemm_df<float>(
          n, [&](int i, int k) { return Y[(size_t)i * n + k]; }, [&](int k, int j) { return X0[(size_t)j * n + k]; },
          zinit,
          [&](int i, int j, df64 v) {
            S0[(size_t)j * n + i] = v;
            S0[(size_t)i * n + j] = v;
          },
          As, Bsf, true);
      tile_gemm_df<float>(
          n, [&](int i, int k) { return df_make(X0[(size_t)i * n + k], 0.f); },
          [&](int k, int j) { return X0[(size_t)j * n + k]; }, zinit,
          [&](int i, int j, df64 v) {
            const df64 r = df_add(df_make(i == j ? 1.f : 0.f, 0.f), df_neg(v));
            R0[(size_t)j * n + i] = r;
            R0[(size_t)i * n + j] = r;
          },
          As, Bsf, true);
      cS = S0;
      cR = R0;
    } else {
      // ---- explicit: Y = A X ; S = X'Y ; R = I - X'X (upper triangles, mirrored)
      tile_gemm_df<df64>(
          n, [&](int i, int k) { return A2[(size_t)k * n + i]; }, [&](int k, int j) { return X[(size_t)j * n + k]; },
          zinit, [&](int i, int j, df64 v) { Y[(size_t)j * n + i] = v; }, As, Bs2, false);
      tile_gemm_df<df64>(
          n, [&](int i, int k) { return X[(size_t)i * n + k]; }, [&](int k, int j) { return Y[(size_t)j * n + k]; },
          zinit,
          [&](int i, int j, df64 v) {
            S[(size_t)j * n + i] = v;
            S[(size_t)i * n + j] = v;
          },
          As, Bs2, true);
      tile_gemm_df<df64>(
          n, [&](int i, int k) { return X[(size_t)i * n + k]; }, [&](int k, int j) { return X[(size_t)j * n + k]; },
          zinit,
          [&](int i, int j, df64 v) {
            const df64 r = df_add(df_make(i == j ? 1.f : 0.f, 0.f), df_neg(v));
            R[(size_t)j * n + i] = r;
            R[(size_t)i * n + j] = r;
          },
          As, Bs2, true);
      cS = S;
      cR = R;
    }
    // ---- Rayleigh quotients, delta, E, clusters
    for (int i = tid; i < n; i += kRT) {
      const double l = df_to(cS[(size_t)i * n + i]) / (1.0 - df_to(cR[(size_t)i * n + i]));
      lam[i] = l;
      lamdf[i] = df_from(l);
      keys[i] = sort_key(l);
    }
    __syncthreads();
    float sd2 = 0.f, r2 = 0.f;
    for (int idx = tid; idx < n * n; idx += kRT) {
      int i, j;
      split_idx(idx, n, inv_n, i, j);
      const float sv = (i == j) ? (float)(df_to(cS[idx]) - lam[i]) : cS[idx].hi;
      sd2 = fmaf(sv, sv, sd2);
      r2 = fmaf(cR[idx].hi, cR[idx].hi, r2);
    }
    const float sdn = sqrtf(block_sum_f(sd2, red));
    const float rn = sqrtf(block_sum_f(r2, red));
    const float delta = 2.f * (sdn + anorm * rn);
    for (int i = tid; i < n; i += kRT) {
      const unsigned long long ki = keys[i];
      int rk = 0;
      for (int j = 0; j < n; j++) rk += (keys[j] < ki) || (keys[j] == ki && j < i);
      ord[rk] = i;
    }
    __syncthreads();
    // clusters: runs of the sorted lam with consecutive gaps <= delta.
    // Sorted position r > 0 starts a new cluster when its gap exceeds delta;
    // its cluster id is the number of such starts at positions 1 .. r
    // (warp ballots), and gmin the smallest gap between clusters.
    {
      const int lane = tid & 31, wid = tid >> 5;
      double g = 1e300;
      bool b = false;
      if (tid >= 1 && tid < n) {
        const double gg = lam[ord[tid]] - lam[ord[tid - 1]];
        b = (float)gg > delta;
        if (b) g = gg;
      }
      const unsigned m = __ballot_sync(0xffffffffu, b);
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) g = fmin(g, __shfl_xor_sync(0xffffffffu, g, o));
      if (lane == 0) {
        brk_mask[wid] = m;
        gred[wid] = g;
      }
      __syncthreads();
      int before = 0, nb = 0;
      double gmin = 1e300;
      for (int w = 0; w < kRT / 32; w++) {
        const int pc = __popc(brk_mask[w]);
        if (w < wid) before += pc;
        nb += pc;
        gmin = fmin(gmin, gred[w]);
      }
      if (tid < n) {
        const unsigned upto = lane == 31 ? 0xffffffffu : ((2u << lane) - 1u);
        const int c = before + __popc(m & upto);
        cid[ord[tid]] = c;
        if (b) cstart[c] = tid;
      }
      if (tid == 0) {
        cstart[0] = 0;
        cstart[nb + 1] = n;
        ncl_s = nb + 1;
        flag_s = 0;
        gmin_s = gmin;
        big_s = nb + 1 < n;  // some cluster holds two or more
        lmax_s = fmax(fabs(lam[ord[0]]), fabs(lam[ord[n - 1]]));  // ||A||_2 of the scaled matrix
      }
    }
    __syncthreads();
    // E: the Newton-type correction between clusters; inside a cluster (its
    // end-to-end gaps may exceed delta) only the orthogonality part r/2, the
    // Rayleigh-Ritz rotation below takes care of the rest. A pair at a tight
    // gap whose coupling is at the rounding floor of the double-float
    // products (|s_ij| <= 1e-14 ||A||; s is symmetric, so the pair (j, i)
    // decides alike) is not rotated either: the rotation
    // would be noise of size 2^-47 ||A|| / gap, whose square shows in the
    // orthogonality, and leaving it changes the residual by less than the
    // floor; rotations below 1e-8 cost nothing and are kept
    const float tfloor = (float)(1e-14 * lmax_s);
    float emax = 0.f, rmax = 0.f;
    for (int idx = tid; idx < n * n; idx += kRT) {
      int i, j;
      split_idx(idx, n, inv_n, i, j);
      const float rhalf = 0.5f * (cR[idx].hi + cR[idx].lo);
      rmax = fmaxf(rmax, fabsf(rhalf));
      float e = rhalf;
      if (cid[i] != cid[j]) {
        const float gap = (float)(lam[j] - lam[i]);
        const df64 num = df_mac(cS[idx], lamdf[j], cR[idx]);
        const float rot = (num.hi + num.lo) / gap;
        const float sij = cS[idx].hi + cS[idx].lo;
        if (!(fabsf(sij) <= tfloor && fabsf(sij / gap) > 1e-8f)) e = rot;
      }
      E[idx] = e;
      emax = fmaxf(emax, fabsf(e));
    }
    emax = block_max_f(emax, red);
    rmax = 2.f * block_max_f(rmax, red);
    // ---- X <- X + X E (FP32 product, see above), then Rayleigh-Ritz inside clusters
    tile_gemm_f32(
        n, [&](int i, int k) { return it == 0 ? X0[(size_t)k * n + i] : X[(size_t)k * n + i].hi; },
        [&](int k, int j) { return E[(size_t)j * n + k]; }, [&](int i, int j, float v) { T1[(size_t)j * n + i] = v; },
        Asf, Bsf, false);
    for (int idx = tid; idx < n * n; idx += kRT) {
      const df64 x = it == 0 ? df_make(X0[idx], 0.f) : X[idx];
      Y[idx] = df_add(x, df_make(T1[idx], 0.f));
    }
    __syncthreads();
    if (big_s) {
      const int ncl = ncl_s;
      for (int c = 0; c < ncl; c++) {
        const int r0 = cstart[c], k = cstart[c + 1] - r0;
        if (k < 2) continue;
        float* C = jac;
        float* Z = jac + k * k;
        // C = (I + R/2) S (I + R/2) - mu I restricted to the cluster, shifted by
        // the mean mu of its lam (first order in R, FP32 after the shift)
        double mu = 0;
        for (int a = 0; a < k; a++) mu += lam[ord[r0 + a]];
        mu /= k;
        for (int idx = tid; idx < k * k; idx += kRT) {
          const int a = idx % k, b = idx / k;
          const int ia = ord[r0 + a], ib = ord[r0 + b];
          df64 sv = cS[(size_t)ib * n + ia];
          if (a == b) sv = df_add(sv, df_from(-mu));
          float corr = 0.f;
          for (int q = 0; q < k; q++) {
            const int iq = ord[r0 + q];
            const float sq_b = cS[(size_t)ib * n + iq].hi - (q == b ? (float)mu : 0.f);
            const float sa_q = cS[(size_t)iq * n + ia].hi - (a == q ? (float)mu : 0.f);
            corr = fmaf(cR[(size_t)iq * n + ia].hi, sq_b, corr);
            corr = fmaf(sa_q, cR[(size_t)ib * n + iq].hi, corr);
          }
          C[b * k + a] = (sv.hi + sv.lo) + 0.5f * corr + (float)mu * cR[(size_t)ib * n + ia].hi;
        }
        __syncthreads();
        float offc = 0.f;
        for (int idx = tid; idx < k * k; idx += kRT)
          if (idx % (k + 1) != 0) offc = fmaxf(offc, fabsf(C[idx]));
        offc = block_max_f(offc, red);
        if (tid < 32) jacobi_warp(k, C, Z);
        __syncthreads();
        if (offc > 0x1p-30f * fmaxf(anorm, 1e-30f) && tid == 0) flag_s = 1;
        // Z is orthogonal only to FP32 rounding (its Jacobi sweeps leave up to
        // ~1e-6); rotating by it every iteration would re-inject that much
        // non-orthogonality and stall the iteration there. Two Newton-Schulz
        // steps in double-float, Z <- Z (I + (I - Z'Z)/2), take it to ~1e-15:
        // Z keeps the high parts, Zl (over C, no longer needed) the low parts,
        // G = I - Z'Z (small, FP32 suffices) goes to T1 (consumed by the
        // update above) and the FP32 correction Z G / 2 to the storage of X
        // (whose old values are no longer needed).
        float* Zl = C;
        float* G = T1;
        float* Cr = reinterpret_cast<float*>(X);
        for (int idx = tid; idx < k * k; idx += kRT) Zl[idx] = 0.f;
        __syncthreads();
        for (int ns = 0; ns < 2; ns++) {
          for (int idx = tid; idx < k * k; idx += kRT) {
            const int a = idx % k, b = idx / k;
            df64 g = df_make(a == b ? 1.f : 0.f, 0.f);
            for (int q = 0; q < k; q++)
              g = df_mac(g, df_make(-Z[a * k + q], -Zl[a * k + q]), df_make(Z[b * k + q], Zl[b * k + q]));
            G[idx] = g.hi + g.lo;
          }
          __syncthreads();
          for (int idx = tid; idx < k * k; idx += kRT) {
            const int a = idx % k, b = idx / k;
            float acc = 0.f;
            for (int q = 0; q < k; q++) acc = fmaf(Z[q * k + a], G[b * k + q], acc);
            Cr[idx] = 0.5f * acc;
          }
          __syncthreads();
          for (int idx = tid; idx < k * k; idx += kRT) {
            const df64 z = df_add(df_make(Z[idx], Zl[idx]), df_make(Cr[idx], 0.f));
            Z[idx] = z.hi;
            Zl[idx] = z.lo;
          }
          __syncthreads();
        }
        // Y[:, J] <- Y[:, J] Z  (temporary in X)
        for (int idx = tid; idx < n * k; idx += kRT) {
          const int i = idx % n, b = idx / n;
          df64 acc = zero;
          for (int q = 0; q < k; q++)
            acc = df_mac(acc, Y[(size_t)ord[r0 + q] * n + i], df_make(Z[b * k + q], Zl[b * k + q]));
          X[(size_t)b * n + i] = acc;
        }
        __syncthreads();
        for (int idx = tid; idx < n * k; idx += kRT) {
          const int i = idx % n, b = idx / n;
          Y[(size_t)ord[r0 + b] * n + i] = X[(size_t)b * n + i];
        }
        __syncthreads();
      }
    }
    df64* t = X;
    X = Y;
    Y = t;
    if (tid == 0) atomicAdd(&stats[3], (unsigned long long)n * n * n);
    __syncthreads();
    // stop when no cluster is unresolved and either the next correction
    // would be below 1e-14 (about emax^2 ||A||_2 / gap, quadratic
    // convergence), or the iterate this step started from was already
    // accurate (delta bounds its residual and orthogonality defects), or the
    // corrections have stopped falling quadratically below 1e-6: E then
    // holds only the rounding floor of the double-float products, about
    // 2^-47 ||A|| / gap at the tightest gaps, and the iterate is at the
    // accuracy floor of the scheme
    const bool quad = (double)emax * emax * lmax_s < 1e-14 * gmin_s;
    // (a stall counts only once the orthogonality defect of the iterate is
    // below 1e-13 entrywise, its rounding floor in double-float being about
    // 2e-14: the noise then sits in the tight-gap rotations)
    const bool stalled = it > 0 && emax < 1e-6f && emax > 0.25f * emax_prev && rmax <= 1e-13f;
    emax_prev = emax;
    if (flag_s == 0 && (quad || stalled || delta <= 1e-13f * anorm)) {
      converged = true;
      break;
    }
  }
  if (!converged && tid == 0) info[mid] = n + 1;  // not converged within kMaxRefineIters
  // sorteig!: ascending eigenvalues, columns permuted to match
  __syncthreads();
  for (int i = tid; i < n; i += kRT) {
    const unsigned long long ki = keys[i];
    int rk = 0;
    for (int j = 0; j < n; j++) rk += (keys[j] < ki) || (keys[j] == ki && j < i);
    rank[i] = rk;
    wout[dsc.w_off + rk] = ldexp(lam[i], se);
  }
  __syncthreads();
  if (V)
    for (int j = 0; j < n; j++) {
      const int dst = rank[j];
      for (int i = tid; i < n; i += kRT) V[(size_t)dst * n + i] = df_to(X[(size_t)j * n + i]);
    }
}

// Dynamic shared memory of the refinement kernels: the tensor-core slabs,
// or, in the persistent kernel, the tridiagonalisation's layout if larger.
size_t refine_smem_bytes(bool tc) { return tc ? (size_t)tcs::kSmem : 0; }

// One CTA per matrix; a matrix the persistent kernel below already refined
// (ChaseState.applied == kRefinedInKernel) is skipped.
template <bool TC>
__global__ void __launch_bounds__(kRT) k_refine(const SmallDesc* __restrict__ descs, const int* __restrict__ perm,
                                                const double* __restrict__ A, int lower,
                                                const float* __restrict__ X32, double* __restrict__ Vout,
                                                double* __restrict__ wout, int* __restrict__ info,
                                                const int* __restrict__ scale_exp, RefineWork rw,
                                                unsigned long long* __restrict__ stats,
                                                const ChaseState* __restrict__ cst) {
  extern __shared__ __align__(128) unsigned char rsm[];
  __shared__ tcs::Shared tsh;
  const int mid = perm[blockIdx.x];
  if (cst && cst[mid].applied == kRefinedInKernel) return;  // (uniform) before any TMEM is taken
  tcs::Ctx tcx;
  if (TC) tcs::setup(tcx, &tsh, rsm, rw.err);
  refine_body<TC>(mid, descs, A, lower, X32, Vout, wout, info, scale_exp, rw, stats, &tcx);
  if (TC) tcs::teardown(tcx);
}

// The whole FP32 + refinement solve of a batch in one persistent launch:
// every CTA takes the next matrix (largest orders first, from an atomic
// counter), tridiagonalises it and solves the tridiagonal in FP32
// (tridiag_body with the per-eigenvalue solver), then refines the pair to
// FP64 accuracy (refine_body), and takes the next. A matrix the FP32 solver
// leaves to the QL chase (or with non-finite input) is left to the chase,
// rotation-replay and refinement kernels that follow (they skip the rest).
// The CTA holds its TMEM (256 columns; two CTAs per SM) for its lifetime.
template <bool TC>
__global__ void __launch_bounds__(kRT, 2)
    k_solve_refine(const SmallDesc* __restrict__ descs, const int* __restrict__ order, int count,
                   int* __restrict__ next, const double* __restrict__ A, int lower, float* __restrict__ d,
                   float* __restrict__ e, float* __restrict__ X32, int* __restrict__ info,
                   ChaseState* __restrict__ cst, int* __restrict__ scale_exp, float* __restrict__ w32,
                   float* __restrict__ qtmp, double* __restrict__ Vout, double* __restrict__ wout, RefineWork rw,
                   unsigned long long* __restrict__ stats) {
  extern __shared__ __align__(128) unsigned char smem_raw[];
  __shared__ int s_idx;
  __shared__ tcs::Shared tsh;
  tcs::Ctx tcx;
  if (TC)
    tcs::setup(tcx, &tsh, smem_raw, rw.err,
               rw.pcache ? rw.pcache + (size_t)blockIdx.x * tcs::kPCacheBytes : nullptr);
  for (;;) {
    __syncthreads();
    if (threadIdx.x == 0) s_idx = atomicAdd(next, 1);
    __syncthreads();
    const int idx = s_idx;
    if (idx >= count) break;
    const int mid = order[idx];
    tridiag_body<float, double, true, true>(mid, smem_raw, descs, A, lower, d, e, X32, info, cst, scale_exp, w32,
                                            qtmp);
    __syncthreads();
    if (cst[mid].applied == 1) {  // solved in FP32 (small_stein.cuh)
      refine_body<TC>(mid, descs, A, lower, X32, Vout, wout, info, scale_exp, rw, stats, &tcx);
      __syncthreads();
      if (threadIdx.x == 0) cst[mid].applied = kRefinedInKernel;
    }
  }
  if (TC) tcs::teardown(tcx);
}

namespace {
size_t solve_refine_smem(int nmax, bool tc) {
  return std::max(tridiag_smem_bytes(nmax, kRT, 4), refine_smem_bytes(tc));
}
}  // namespace

cudaError_t refine_kernels_init() {
  cudaFuncSetAttribute(k_solve_refine<false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                       (int)solve_refine_smem(kSmallMaxN, false));
  cudaFuncSetAttribute(k_solve_refine<true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                       (int)solve_refine_smem(kSmallMaxN, true));
  cudaFuncSetAttribute(k_refine<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)refine_smem_bytes(true));
  return cudaGetLastError();
}

cudaError_t launch_refine(const RefineWork* rw, int nblocks, int nmax, cudaStream_t st, const SmallDesc* descs,
                          const int* perm, const double* A, int lower, const float* X32, double* V, double* w,
                          int* info, const int* scale_exp, unsigned long long* stats, const ChaseState* cst,
                          bool tc) {
  if (nblocks <= 0) return cudaSuccess;
  (void)nmax;
  if (tc)
    k_refine<true><<<nblocks, kRT, refine_smem_bytes(true), st>>>(descs, perm, A, lower, X32, V, w, info, scale_exp,
                                                                  *rw, stats, cst);
  else
    k_refine<false><<<nblocks, kRT, 0, st>>>(descs, perm, A, lower, X32, V, w, info, scale_exp, *rw, stats, cst);
  return cudaGetLastError();
}

cudaError_t launch_solve_refine(const RefineWork* rw, int count, int nmax, int grid, cudaStream_t st,
                                const SmallDesc* descs, const int* order, int* next, const double* A, int lower,
                                float* d, float* e, float* X32, int* info, ChaseState* cst, int* scale_exp,
                                float* w32, float* qtmp, double* V, double* w, unsigned long long* stats, bool tc) {
  if (count <= 0) return cudaSuccess;
  const size_t smem = solve_refine_smem(nmax, tc);
  if (tc)
    k_solve_refine<true><<<grid, kRT, smem, st>>>(descs, order, count, next, A, lower, d, e, X32, info, cst,
                                                  scale_exp, w32, qtmp, V, w, *rw, stats);
  else
    k_solve_refine<false><<<grid, kRT, smem, st>>>(descs, order, count, next, A, lower, d, e, X32, info, cst,
                                                   scale_exp, w32, qtmp, V, w, *rw, stats);
  return cudaGetLastError();
}

}  // namespace gla
