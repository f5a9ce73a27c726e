// Implicit-shift QL / QR / root-free PWK iterations on the tridiagonal,
// one matrix per lane (32 matrices per warp, matrices sorted by size so the
// lanes of a warp run similar-length loops).
//
// Replaces, per matrix:
//   eigQL!          (GenericLinearAlgebra.jl src/eigenSelfAdjoint.jl:221-288)
//   singleShiftQL!  (:377-409)
//   eigQR!          (:290-340), singleShiftQR! (:412-444)
//   eigvalsPWK!     (:163-219), singleShiftQLPWK! (:343-374)
//   eig2x2! / eigvals2x2 (:131-161)
//   givensAlgorithm for Float64/Float32 (LinearAlgebra's LAPACK-dlartg port).
//
// The scalar recurrence of a chase is serial, and on GB300 an FP64 warp
// instruction costs the FP64 unit ~64 cycles whatever the active-lane count,
// so running one matrix per lane is 32x cheaper than one per warp. The
// rotations (c, s) are not applied here: they are appended to a per-matrix
// log (plus one header per sweep) that the apply kernel replays on the rows
// of Q in parallel. When a matrix's log is full the lane stops between
// sweeps, saves its state and is resumed by the next pass.
//
// Differences from the reference, all rounding-level: the Givens radius
// uses a Newton-refined hardware rsqrt seed instead of sqrt and two
// divisions; gamma/c uses a refined reciprocal; the deflation test
// |e| <= tol*sqrt|d_i|*sqrt|d_i+1| (:250-256) is decided on exponents when
// the two sides are more than a factor 4 apart and evaluated exactly
// otherwise (identical decisions on identical data). Each chase is capped at
// max_sweeps_per_n * n sweeps (the reference has no cap and loops forever on
// e.g. NaN input); hitting the cap reports the unconverged count as info.
#include "gla_launch.h"
#include "gla_small.cuh"

namespace gla {

template <class T> GLA_DEV bool is_zero(T x) { return (prec<T>::bits(x) << 1) == 0; }

// Deflation test of :250-256 (and of :177 with e holding e^2).
template <class T> GLA_DEV bool negligible(T ev, T d1, T d2, T tol, int tol_e) {
  const int maxe = sizeof(T) == 8 ? 0x7ff : 0xff;
  const int xe = prec<T>::biased_exp(ev), x1 = prec<T>::biased_exp(d1), x2 = prec<T>::biased_exp(d2);
  if (xe != 0 && xe != maxe && x1 != 0 && x1 != maxe && x2 != 0 && x2 != maxe) {
    // q = 2log2|e| - log2|d1| - log2|d2| - 2log2(tol) lies in (L-4, L+2)
    const int L = 2 * xe - x1 - x2 - 2 * tol_e;
    if (L + 2 <= 0) return true;
    if (L - 4 >= 0) return false;
  }
  return tabs(ev) <= tol * prec<T>::sqrt_ieee(tabs(d1)) * prec<T>::sqrt_ieee(tabs(d2));
}

// LAPACK 3.x dlartg convention (as in LinearAlgebra.givensAlgorithm for
// AbstractFloat): r = +-sqrt(f^2+g^2), (c,s,r) negated when |f|>|g| and c<0.
template <class T> GLA_DEV void givens_exact(T f, T g, T& cs, T& sn, T& r) {
  const T safmn2 = sizeof(T) == 8 ? (T)0x1p-485 : (T)0x1p-51f;
  const T safmx2 = T(1) / safmn2;
  T f1 = f, g1 = g;
  T scale = fmax(tabs(f1), tabs(g1));
  int count = 0;
  if (scale >= safmx2) {
    do {
      count++;
      f1 *= safmn2;
      g1 *= safmn2;
      scale = fmax(tabs(f1), tabs(g1));
    } while (scale >= safmx2 && count < 20);
    r = prec<T>::sqrt_ieee(f1 * f1 + g1 * g1);
    cs = prec<T>::div_ieee(f1, r);
    sn = prec<T>::div_ieee(g1, r);
    for (int i = 0; i < count; i++) r *= safmx2;
  } else if (scale <= safmn2) {
    do {
      count++;
      f1 *= safmx2;
      g1 *= safmx2;
      scale = fmax(tabs(f1), tabs(g1));
    } while (scale <= safmn2 && count < 4000);
    r = prec<T>::sqrt_ieee(f1 * f1 + g1 * g1);
    cs = prec<T>::div_ieee(f1, r);
    sn = prec<T>::div_ieee(g1, r);
    for (int i = 0; i < count; i++) r *= safmn2;
  } else {
    r = prec<T>::sqrt_ieee(f1 * f1 + g1 * g1);
    cs = prec<T>::div_ieee(f1, r);
    sn = prec<T>::div_ieee(g1, r);
  }
}

template <class T> GLA_DEV void givens(T f, T g, T& c, T& s, T& r) {
  if (is_zero(g)) {
    c = 1;
    s = 0;
    r = f;
    return;
  }
  if (is_zero(f)) {
    c = 0;
    s = 1;
    r = g;
    return;
  }
  if (prec<T>::tame(f) && prec<T>::tame(g)) {
    const T r2 = fma(f, f, g * g);
    const T y = prec<T>::rsqrt(r2);
    r = r2 * y;
    c = f * y;
    s = g * y;
  } else {
    givens_exact(f, g, c, s, r);
  }
  // |f| > |g| and c < 0 (c has the sign of f)
  if (!abs_le(f, g) && (prec<T>::bits(c) >> (sizeof(T) * 8 - 1))) {
    c = -c;
    s = -s;
    r = -r;
  }
}

// Givens rotation for the sweep step: the refined-rsqrt radius when
// f^2 + g^2 is comfortably inside the normal range, the exact dlartg port
// otherwise. Same convention as givens() (c >= 0 when |f| > |g|; f == 0 gives
// c = 0, s = 1, r = g). FP32 tests use float compares; FP64 tests use the
// exponent bits (an FP64 compare costs a full FP64 warp-instruction slot).
GLA_DEV void givens_step(float f, float g, float& c, float& s, float& r) {
  const float r2 = fmaf(f, f, g * g);
  if (r2 >= 0x1p-120f && r2 <= 0x1p+120f) {
    const float y = prec<float>::rsqrt(r2);
    r = r2 * y;
    c = f * y;
    s = g * y;
    if (f == 0.f) {
      c = 0.f;
      s = 1.f;
      r = g;
    } else if (f < 0.f && fabsf(f) > fabsf(g)) {
      c = -c;
      s = -s;
      r = -r;
    }
  } else {
    givens(f, g, c, s, r);
  }
}
GLA_DEV void givens_step(double f, double g, double& c, double& s, double& r) {
  const double r2 = fma(f, f, g * g);
  const int be = prec<double>::biased_exp(r2);
  if (be >= 1023 - 1000 && be <= 1023 + 1000) {
    const double y = prec<double>::rsqrt(r2);
    r = r2 * y;
    c = f * y;
    s = g * y;
    if (is_zero(f)) {
      c = 0.0;
      s = 1.0;
      r = g;
    } else if (!abs_le(f, g) && (prec<double>::bits(f) >> 63)) {
      c = -c;
      s = -s;
      r = -r;
    }
  } else {
    givens(f, g, c, s, r);
  }
}

// Deflation test on register values: FP32 decides on the squared sides
// (margin 4x each way) and falls back to the exact form near the threshold
// or when a square leaves the normal range; FP64 uses the exponent filter.
GLA_DEV bool negligible_step(float ev, float d1, float d2, float tol, int tol_e) {
  const float e2 = ev * ev;
  const float rhs = (tol * tol) * fabsf(d1 * d2);
  if (rhs >= 0x1p-120f && rhs <= 0x1p+120f && e2 <= 0x1p+120f) {
    if (e2 < 0.25f * rhs) return true;
    if (e2 > 4.f * rhs) return false;
  }
  return negligible(ev, d1, d2, tol, tol_e);
}
GLA_DEV bool negligible_step(double ev, double d1, double d2, double tol, int tol_e) {
  return negligible(ev, d1, d2, tol, tol_e);
}

// gamma / c: FP32 uses rcp.approx (~1 ulp, one rounding in the recurrence)
// guarded by a float compare; FP64 the Newton-refined reciprocal.
GLA_DEV float div_step(float a, float b) {
  if (fabsf(b) < 0x1p-100f) return __fdiv_rn(a, b);
  float y;
  asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(b));
  return a * y;
}

template <class T> GLA_DEV T div_fast(T a, T b) {
  return prec<T>::tame(b) ? a * prec<T>::rcp(b) : prec<T>::div_ieee(a, b);
}

// gamma / c of the QL/QR recurrence. FP32: the hardware reciprocal
// (rcp.approx, ~1 ulp) without refinement, an error of the size of one
// rounding in the recurrence; FP64: the Newton-refined reciprocal.
GLA_DEV float div_chase(float a, float b) {
  if (!prec<float>::tame(b)) return __fdiv_rn(a, b);
  float y;
  asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(b));
  return a * y;
}
GLA_DEV double div_chase(double a, double b) { return div_fast(a, b); }
GLA_DEV double div_step(double a, double b) { return div_fast(a, b); }

// Append (c, s) to the rotation log as one 8- or 16-byte store.
GLA_DEV void store_rot(float* log, int k, float c, float s) {
  reinterpret_cast<float2*>(log)[k] = make_float2(c, s);
}
GLA_DEV void store_rot(double* log, int k, double c, double s) {
  reinterpret_cast<double2*>(log)[k] = make_double2(c, s);
}

// sqrt(m^2 + 1) for the shift computation (:272, :201, :325); exactness of
// the shift only affects the convergence rate, so a refined rsqrt replaces
// the correctly rounded hypot here.
template <class T> GLA_DEV T hypot1_fast(T m) {
  const T am = tabs(m);
  if (!prec<T>::tame(am)) return am < T(1) ? T(1) : am;
  const T q = fma(m, m, T(1));
  return q * prec<T>::rsqrt(q);
}

size_t chase_smem_bytes(int nmax, int elem) { return 512 + (size_t)2 * nmax * 32 * elem; }

// ALGO: kAlgoQL (eigQL!, logs rotations), kAlgoQR (eigQR!, logs), kAlgoPWK
// (eigvalsPWK!, values only). d, e: per-matrix diagonals at w_off (e padded
// to n entries). rot: 2 values per rotation; hdr: one word per sweep.
//
// Deflation bookkeeping: instead of rescanning e from blockstart after every
// chase (:250-256), each lane keeps a bitmask NF of "e[j] is negligible",
// re-evaluating entry j exactly when e[j], d[j] or d[j+1] takes its final
// value for the chase (one test per rotation). The first negligible entry at
// or after blockstart is then found with __ffs, and the decision is the one
// the rescan would make on the same values. This keeps the 32 lanes of a
// warp from serialising on each other's O(n) scans.
template <class T, int ALGO>
__global__ void __launch_bounds__(32) k_chase(const SmallDesc* __restrict__ descs, const int* __restrict__ perm,
                                              int count, T* __restrict__ dg_all, T* __restrict__ eg_all,
                                              ChaseState* __restrict__ cst, T* __restrict__ rot,
                                              unsigned* __restrict__ hdr, int* __restrict__ info, T tol,
                                              int max_sweeps_per_n, int* __restrict__ pending,
                                              unsigned long long* __restrict__ stats, int lanes_per_warp) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int lane = threadIdx.x;
  // lanes_per_warp matrices per warp (the other lanes idle): fewer lanes cut
  // the divergence between lanes that are between sweeps and lanes inside one
  const int slot = blockIdx.x * lanes_per_warp + lane;
  const bool have = lane < lanes_per_warp && slot < count;
  const int mid = have ? perm[slot] : 0;
  SmallDesc dsc;
  dsc.n = 0;
  if (have) dsc = descs[mid];
  const int n = dsc.n;
  int nmax = n;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) nmax = max(nmax, __shfl_xor_sync(0xffffffffu, nmax, o));
  unsigned* NF = reinterpret_cast<unsigned*>(smem_raw) + lane;  // NF[w * 32], w < 4
  T* D = reinterpret_cast<T*>(smem_raw + 512) + lane;
  T* E = reinterpret_cast<T*>(smem_raw + 512) + (size_t)nmax * 32 + lane;
#define DD(i) D[(size_t)(i) * 32]
#define EE(i) E[(size_t)(i) * 32]

  ChaseState st;
  st.status = kChaseDone;
  if (have) st = cst[mid];
  const bool was_running = have && st.status == kChaseRunning;
  bool active = was_running;
  T* dg = dg_all + dsc.w_off;
  T* eg = eg_all + dsc.w_off;
  const int tol_e = prec<T>::biased_exp(tol) - prec<T>::expbias;
  auto test = [&](int j) {  // re-evaluate NF(j), j <= n - 2
    const bool f = negligible(EE(j), DD(j), DD(j + 1), tol, tol_e);
    unsigned& w = NF[(j >> 5) * 32];
    const unsigned b = 1u << (j & 31);
    w = f ? (w | b) : (w & ~b);
  };
  auto first_nf = [&](int from) -> int {  // first j >= from with NF(j), else n - 1
    for (int w = from >> 5; w <= (n - 2) >> 5; w++) {
      unsigned bits = NF[w * 32];
      if (w == (from >> 5)) bits &= ~0u << (from & 31);
      if (bits) return w * 32 + __ffs(bits) - 1;
    }
    return n - 1;
  };
  for (int w = 0; w < 4; w++) NF[w * 32] = 0;
  if (active) {
    for (int k = 0; k < n; k++) {
      DD(k) = dg[k];
      const T e = eg[k];
      // eigvalsPWK! squares the off-diagonal first (:171-173)
      EE(k) = (ALGO == kAlgoPWK && st.nsweeps == 0 && st.bs == 0) ? e * e : e;
    }
    for (int j = 0; j + 1 < n; j++) test(j);
  }
  const int cap = max_sweeps_per_n * n;
  int bs = st.bs, nsw = st.nsweeps;
  int nrot = 0, nhdr = 0;
  T* myrot = rot + 2 * dsc.rot_off;
  unsigned* myhdr = hdr + dsc.hdr_off;
  bool insweep = false, stopped_full = false;
  int i = 0, be = 0;
  T mu = 0, gam = 0, p = 0, c = 1, s = 0;
  // register cache of the sweep: next (e, d) to consume, the d two positions
  // behind (for the deflation test) and e beyond the block end
  T e_nx = 0, d_nx = 0, d_up = 0, e_end = 0;
  // NF word of the current sweep position cached in a register
  unsigned nfw = 0;
  int nfw_idx = -1;
  auto nf_flush = [&]() {
    if (nfw_idx >= 0) NF[nfw_idx * 32] = nfw;
    nfw_idx = -1;
  };
  auto test_v = [&](int j, T ev, T d1, T d2) {  // NF(j) from register values
    const bool f = negligible_step(ev, d1, d2, tol, tol_e);
    const int wi = j >> 5;
    if (wi != nfw_idx) {
      nf_flush();
      nfw_idx = wi;
      nfw = NF[wi * 32];
    }
    const unsigned b = 1u << (j & 31);
    nfw = f ? (nfw | b) : (nfw & ~b);
  };
  int iters = 0;
  const int iter_cap = (max_sweeps_per_n + 4) * 4 * nmax * nmax + 64;  // hard bound on loop trips

  while (__any_sync(0xffffffffu, active)) {
    if (++iters > iter_cap) {  // defensive: never reached when the sweep cap works
      if (active) {
        info[mid] = max(1, n - 1);
        active = false;
        st.status = kChaseDone;
      }
      continue;
    }
    if (active && !insweep) {
      nf_flush();
      if (bs >= n - 1) {
        active = false;
        st.status = kChaseDone;
      } else {
        be = first_nf(bs);
        if (bs == be) {
          bs += 1;
        } else if (bs + 1 == be) {
          if (ALGO == kAlgoPWK) {
            const T d1 = DD(bs), d2 = DD(be), ee = prec<T>::sqrt_ieee(EE(bs));
            const T r1 = (d1 + d2) / 2;
            const T r2 = hypot_borges(d1 - d2, 2 * ee) / 2;
            DD(bs) = r1 + r2;
            DD(be) = r1 - r2;
            EE(bs) = 0;
            test(bs);
            if (be <= n - 2) test(be);
            bs += 1;
          } else if (nrot + 1 > dsc.rot_cap || nhdr + 1 > dsc.hdr_cap) {
            active = false;
            stopped_full = true;
          } else {
            // eig2x2! (:136-161)
            const T dj = DD(bs), dj1 = DD(be), ej = EE(bs);
            const T r1 = (dj + dj1) / 2;
            const T r2 = hypot_borges(dj - dj1, 2 * ej) / 2;
            const T lp = r1 + r2, lm = r1 - r2;
            DD(bs) = lp;
            DD(be) = lm;
            EE(bs) = 0;
            T cc, ss;
            if (is_zero(ej)) {
              cc = 1;
              ss = 0;
            } else if (tabs(lp - dj) > tabs(lm - dj)) {
              cc = prec<T>::div_ieee(-ej, hypot_borges(ej, lp - dj));
              ss = prec<T>::sqrt_ieee(1 - cc * cc);
            } else {
              ss = prec<T>::div_ieee(tabs(ej), hypot_borges(ej, lm - dj));
              cc = tcopysign(prec<T>::sqrt_ieee(1 - ss * ss), -ej);
            }
            myhdr[nhdr++] = pack_hdr(bs, 1, 0);
            myrot[2 * nrot] = cc;
            myrot[2 * nrot + 1] = ss;
            nrot++;
            test(bs);
            if (be <= n - 2) test(be);
            bs += 2;
          }
        } else if (nsw >= cap) {
          int cnt = 0;
          for (int b = 0; b + 1 < n; b++) cnt += !negligible(EE(b), DD(b), DD(b + 1), tol, tol_e);
          info[mid] = max(cnt, 1);
          active = false;
          st.status = kChaseDone;
        } else if (ALGO != kAlgoPWK && (nrot + (be - bs) > dsc.rot_cap || nhdr + 1 > dsc.hdr_cap)) {
          active = false;
          stopped_full = true;
        } else {
          // shift (:199-202 PWK, :271-273 QL, :324-326 QR) and start a chase
          if (ALGO == kAlgoPWK) {
            const T sqrte = prec<T>::sqrt_ieee(EE(bs));
            const T m = div_fast(DD(bs + 1) - DD(bs), 2 * sqrte);
            mu = DD(bs) - div_fast(sqrte, m + tcopysign(hypot1_fast(m), m));
            gam = DD(be) - mu;
            p = gam * gam;
            i = be - 1;
          } else if (ALGO == kAlgoQL) {
            const T m = div_fast(DD(bs + 1) - DD(bs), 2 * EE(bs));
            mu = DD(bs) - div_fast(EE(bs), m + tcopysign(hypot1_fast(m), m));
            gam = DD(be) - mu;
            p = gam;
            i = be - 1;
            myhdr[nhdr++] = pack_hdr(be - 1, be - bs, 0);
          } else {
            const T m = div_fast(DD(be - 1) - DD(be), 2 * EE(be - 1));
            mu = DD(be) - div_fast(EE(be - 1), m + tcopysign(hypot1_fast(m), m));
            gam = DD(bs) - mu;
            p = gam;
            i = bs + 1;
            myhdr[nhdr++] = pack_hdr(bs + 1, be - bs, 1);
          }
          if (ALGO == kAlgoQR) {
            e_nx = EE(bs);
            d_nx = DD(bs + 1);
            d_up = DD(bs);  // d[i-2] of the first test (unused: j < bs)
          } else {
            e_nx = EE(be - 1);
            d_nx = DD(be - 1);
            d_up = (be + 1 <= n - 1) ? DD(be + 1) : T(0);
            e_end = (be <= n - 2) ? EE(be) : T(0);
          }
          c = 1;
          s = 0;
          insweep = true;
          nsw++;
        }
      }
    }
    // tight sweep loop: runs while every active lane is inside a chase
    while (__all_sync(0xffffffffu, !active || insweep) && __any_sync(0xffffffffu, active)) {
      if (++iters > iter_cap) break;
      if (active) {
        if (ALGO == kAlgoQL) {
          // singleShiftQL! step at i (:389-405), operands from registers
          const T ei = e_nx, di = d_nx;
          if (i > bs) {
            e_nx = EE(i - 1);
            d_nx = DD(i - 1);
          }
          const T c1 = c, s1 = s;
          T zeta;
          givens_step(p, ei, c, s, zeta);
          const T enew = (i < be - 1) ? s1 * zeta : e_end;
          if (i < be - 1) EE(i + 1) = enew;
          const T g1 = gam;
          gam = c * c * (di - mu) - s * s * g1;
          const T dnew = g1 + di - gam;
          DD(i + 1) = dnew;
          p = is_zero(c) ? -ei * c1 : div_step(gam, c);
          store_rot(myrot, nrot, c, s);
          nrot++;
          if (i + 1 <= n - 2) test_v(i + 1, enew, dnew, d_up);
          d_up = dnew;
          i--;
          if (i < bs) {
            const T eb = s * p, db = mu + gam;
            EE(bs) = eb;
            DD(bs) = db;
            test_v(bs, eb, db, d_up);
            insweep = false;
          }
        } else if (ALGO == kAlgoQR) {
          // singleShiftQR! step at i (:424-440), operands from registers;
          // d_up holds d[i-2] (the previous step's new d)
          const T ei = e_nx, di = d_nx;
          if (i < be) {
            e_nx = EE(i);
            d_nx = DD(i + 1);
          }
          const T c1 = c, s1 = s;
          T zeta;
          givens_step(p, ei, c, s, zeta);
          const T g1 = gam;
          gam = c * c * (di - mu) - s * s * g1;
          const T dnew = g1 + di - gam;
          DD(i - 1) = dnew;
          if (i > bs + 1) {
            const T enew = s1 * zeta;
            EE(i - 2) = enew;
            test_v(i - 2, enew, d_up, dnew);
          }
          p = is_zero(c) ? -ei * c1 : div_step(gam, c);
          store_rot(myrot, nrot, c, s);
          nrot++;
          d_up = dnew;
          i++;
          if (i > be) {
            const T eb = s * p, db = mu + gam;
            EE(be - 1) = eb;
            DD(be) = db;
            test_v(be - 1, eb, d_up, db);
            if (be <= n - 2) test_v(be, EE(be), db, DD(be + 1));
            insweep = false;
          }
        } else {
          // singleShiftQLPWK! step at i (:356-370); e holds squares
          const T ei = e_nx, di = d_nx;
          if (i > bs) {
            e_nx = EE(i - 1);
            d_nx = DD(i - 1);
          }
          const T zeta = p + ei;
          const T enew = (i < be - 1) ? s * zeta : e_end;
          if (i < be - 1) EE(i + 1) = enew;
          const T c1 = c;
          const T rz = prec<T>::tame(zeta) ? prec<T>::rcp(zeta) : prec<T>::div_ieee(T(1), zeta);
          c = p * rz;
          s = ei * rz;
          const T g1 = gam;
          gam = c * (di - mu) - s * g1;
          const T dnew = g1 + di - gam;
          DD(i + 1) = dnew;
          p = is_zero(c) ? ei * c1 : div_fast(gam * gam, c);
          if (i + 1 <= n - 2) test_v(i + 1, enew, dnew, d_up);
          d_up = dnew;
          i--;
          if (i < bs) {
            const T eb = s * p, db = mu + gam;
            EE(bs) = eb;
            DD(bs) = db;
            test_v(bs, eb, db, d_up);
            insweep = false;
          }
        }
    
      }
    }
  }
  if (was_running) {
    for (int k = 0; k < n; k++) {
      dg[k] = DD(k);
      eg[k] = EE(k);
    }
    const int sweeps_this_pass = nsw - st.nsweeps;
    st.bs = bs;
    st.nsweeps = nsw;
    st.nrot = nrot;
    st.nhdr = nhdr;
    cst[mid] = st;
    if (stopped_full) atomicAdd(pending, 1);
    atomicAdd(&stats[0], (unsigned long long)(ALGO == kAlgoPWK ? 0 : nrot));
    atomicAdd(&stats[1], (unsigned long long)sweeps_this_pass);
    atomicAdd(&stats[2], (unsigned long long)(ALGO == kAlgoPWK ? 0 : nrot) * (unsigned long long)n);
  }
#undef DD
#undef EE
}

template <class T, int ALGO> static void set_chase_attr() {
  cudaFuncSetAttribute(k_chase<T, ALGO>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                       (int)chase_smem_bytes(kSmallMaxN, (int)sizeof(T)));
}

cudaError_t chase_kernels_init() {
  set_chase_attr<double, kAlgoQL>();
  set_chase_attr<double, kAlgoQR>();
  set_chase_attr<double, kAlgoPWK>();
  set_chase_attr<float, kAlgoQL>();
  set_chase_attr<float, kAlgoQR>();
  set_chase_attr<float, kAlgoPWK>();
  return cudaGetLastError();
}

cudaError_t launch_chase(int tcode, int algo, int count, size_t smem, cudaStream_t st, const SmallDesc* descs,
                         const int* perm, void* d, void* e, ChaseState* cst, void* rot, unsigned* hdr, int* info,
                         double tol, int max_sweeps_per_n, int* pending, unsigned long long* stats,
                         int lanes_per_warp) {
  if (count <= 0) return cudaSuccess;
  // Default: FP32 chases are instruction-latency bound, 8 matrices per warp
  // keep the lanes of a warp in step; FP64 pays ~64 cycles per warp
  // instruction, so the cost of divergence and of idle lanes balance at 16.
  // A plan's autotuner may choose another count (1..32).
  const int lpw = (lanes_per_warp >= 1 && lanes_per_warp <= 32) ? lanes_per_warp : (tcode == kF64 ? 16 : 8);
  const int nb = (count + lpw - 1) / lpw;
#define GLA_CH(T, A)                                                                                             \
  k_chase<T, A><<<nb, 32, smem, st>>>(descs, perm, count, (T*)d, (T*)e, cst, (T*)rot, hdr, info, (T)tol,        \
                                      max_sweeps_per_n, pending, stats, lpw)
  if (tcode == kF64) {
    if (algo == kAlgoQL) GLA_CH(double, kAlgoQL);
    else if (algo == kAlgoQR) GLA_CH(double, kAlgoQR);
    else GLA_CH(double, kAlgoPWK);
  } else {
    if (algo == kAlgoQL) GLA_CH(float, kAlgoQL);
    else if (algo == kAlgoQR) GLA_CH(float, kAlgoQR);
    else GLA_CH(float, kAlgoPWK);
  }
#undef GLA_CH
  return cudaGetLastError();
}

}  // namespace gla
