// CPU ORACLE — test infrastructure only, never part of the shipped path.
//
// A line-faithful C++ restatement of the self-adjoint eigensolver of
// GenericLinearAlgebra.jl v0.4.0 (src/eigenSelfAdjoint.jl). Only tests/,
// the smoke check and the CPU-baseline leg of the benchmark may load it.
//
// Parity status: the reference is Julia and Julia is not installed, so the
// restatement cannot be diffed against the reference's own Float64 output.
// It is pinned instead against every known-answer case in the reference's
// test file (test/eigenselfadjoint.jl: the 1x1 case :100-105, issue 52
// :108-117, issue 123 :125-149, #139 :164-170, the prescribed spectrum
// rtol 1e-13*n :73) and against LAPACK (scipy eigh) and a 256-bit mpmath
// restatement of the same algorithm.
//
// Arithmetic follows Julia's evaluation order (no contraction into FMA;
// build with -ffp-contract=off). Three stdlib/BLAS routines sit outside the
// reference (Julia stdlib LinearAlgebra, pinned only by the package's
// `julia = "1.6"` compat): reflector!, givensAlgorithm(::T,::T) for
// T<:AbstractFloat, and BLAS dsymv/dnrm2. They are restated from their
// published algorithms (Householder reflector per Golub & Van Loan 5.1,
// LAPACK 3.x dlartg, netlib reference dsymv, scaled 2-norm).
#pragma once
#include <algorithm>
#include <cmath>
#include <complex>
#include <cstdint>
#include <limits>
#include <numeric>
#include <vector>

#if defined(__x86_64__)
#include <quadmath.h>
typedef __float128 gla_quad;
#define GLA_QUAD_SQRT sqrtq
#define GLA_QUAD_FABS fabsq
#define GLA_QUAD_COPYSIGN copysignq
#else
// aarch64 Linux: long double is IEEE binary128.
typedef long double gla_quad;
#define GLA_QUAD_SQRT sqrtl
#define GLA_QUAD_FABS fabsl
#define GLA_QUAD_COPYSIGN copysignl
#endif

namespace gla_oracle {

template <class T> struct num;

template <> struct num<double> {
  static double sqrt(double x) { return std::sqrt(x); }
  static double abs(double x) { return std::fabs(x); }
  static double copysign(double x, double y) { return std::copysign(x, y); }
  static double fma(double a, double b, double c) { return std::fma(a, b, c); }
  static double eps() { return 0x1p-52; }            // Julia eps(Float64)
  static double floatmin() { return 0x1p-1022; }
  static double floatmax() { return std::numeric_limits<double>::max(); }
  // Julia floatmin2: 2^trunc(log2(floatmin/eps)/2) = 2^((-1022 - -52)/2)
  static double safmn2() { return 0x1p-485; }
  static bool isfinite(double x) { return std::isfinite(x); }
  static bool signbit(double x) { return std::signbit(x); }
};

template <> struct num<float> {
  static float sqrt(float x) { return std::sqrt(x); }
  static float abs(float x) { return std::fabs(x); }
  static float copysign(float x, float y) { return std::copysign(x, y); }
  static float fma(float a, float b, float c) { return std::fma(a, b, c); }
  static float eps() { return 0x1p-23f; }            // Julia eps(Float32)
  static float floatmin() { return 0x1p-126f; }
  static float floatmax() { return std::numeric_limits<float>::max(); }
  // 2^trunc((-126 - -23)/2)
  static float safmn2() { return 0x1p-51f; }
  static bool isfinite(float x) { return std::isfinite(x); }
  static bool signbit(float x) { return std::signbit(x); }
};

template <> struct num<gla_quad> {
  static gla_quad sqrt(gla_quad x) { return GLA_QUAD_SQRT(x); }
  static gla_quad abs(gla_quad x) { return GLA_QUAD_FABS(x); }
  static gla_quad copysign(gla_quad x, gla_quad y) { return GLA_QUAD_COPYSIGN(x, y); }
  static gla_quad fma(gla_quad a, gla_quad b, gla_quad c) { return a * b + c; }
  static gla_quad pow2(int e) {
    gla_quad x = 1;
    for (; e > 0; e--) x *= 2;
    for (; e < 0; e++) x /= 2;
    return x;
  }
  static gla_quad eps() { static const gla_quad v = pow2(-112); return v; }
  static gla_quad floatmin() { static const gla_quad v = pow2(-16382); return v; }
  static gla_quad floatmax() { static const gla_quad v = pow2(16383) * (2 - eps()); return v; }
  // (-16382 - -112)/2 -> -8135
  static gla_quad safmn2() { static const gla_quad v = pow2(-8135); return v; }
  static bool isfinite(gla_quad x) { return x == x && GLA_QUAD_FABS(x) <= floatmax(); }
  static bool signbit(gla_quad x) { return GLA_QUAD_COPYSIGN((gla_quad)1, x) < 0; }
};

// Column-major element access, 0-based.
template <class T> inline T& at(T* A, int64_t ld, int64_t i, int64_t j) { return A[i + j * ld]; }

// hypot: Julia Base's hypot(x::T, y::T) for T<:AbstractFloat follows
// C. F. Borges, "An Improved Algorithm for hypot(a,b)", ACM TOMS 47 (2021),
// the fused-correction variant. Restated from the paper.
template <class T> T hypot_borges(T x, T y) {
  typedef num<T> N;
  T ax = N::abs(x), ay = N::abs(y);
  const T inf = N::floatmax() * 2;
  if (ax == inf || ay == inf) return inf;  // IEEE 754: Inf wins over NaN
  if (ay > ax) std::swap(ax, ay);
  if (ay <= ax * N::sqrt(N::eps() / 2)) return ax;  // widely varying (also ay == 0)
  T scale = N::eps() * N::sqrt(N::floatmin());
  if (ax > N::sqrt(N::floatmax() / 2)) {
    ax = ax * scale;
    ay = ay * scale;
    scale = 1 / scale;
  } else if (ay < N::sqrt(N::floatmin())) {
    ax = ax / scale;
    ay = ay / scale;
  } else {
    scale = 1;
  }
  T h = N::sqrt(N::fma(ax, ax, ay * ay));
  T hsq = h * h;
  T axsq = ax * ax;
  h -= (N::fma(-ay, ay, hsq - axsq) + N::fma(h, h, -hsq) - N::fma(ax, ax, -axsq)) / (2 * h);
  return h * scale;
}

// 2-norm of a strided vector with the overflow/underflow guard of Julia's
// generic_norm2 (scale by the max-abs entry only when the plain sum of
// squares could overflow or underflow).
template <class T> T norm2(const T* x, int64_t n, int64_t inc) {
  typedef num<T> N;
  T maxabs = 0;
  for (int64_t i = 0; i < n; i++) {
    T a = N::abs(x[i * inc]);
    if (!(a <= maxabs)) maxabs = a;  // propagates NaN
  }
  if (maxabs == 0 || !N::isfinite(maxabs)) return maxabs;
  T nT = (T)n;
  if (N::isfinite(nT * maxabs * maxabs) && maxabs * maxabs != 0) {
    T sum = 0;
    for (int64_t i = 0; i < n; i++) sum += x[i * inc] * x[i * inc];
    return N::sqrt(sum);
  }
  T sum = 0;
  for (int64_t i = 0; i < n; i++) {
    T v = x[i * inc] / maxabs;
    sum += v * v;
  }
  return maxabs * N::sqrt(sum);
}

// LinearAlgebra.reflector!(x): x -> [-nu; x[2:end]/(x1+nu)], returns tau.
// (stdlib; called at src/eigenSelfAdjoint.jl:466 and :526)
template <class T> T reflector(T* x, int64_t n, int64_t inc) {
  typedef num<T> N;
  if (n == 0) return 0;
  T xi1 = x[0];
  T normu = norm2(x, n, inc);
  if (normu == 0) return 0;
  T nu = N::copysign(normu, xi1);
  xi1 += nu;
  x[0] = -nu;
  for (int64_t i = 1; i < n; i++) x[i * inc] /= xi1;
  return xi1 / nu;
}

// Givens rotation, LAPACK 3.x dlartg convention as ported in Julia stdlib
// givensAlgorithm(f::T, g::T) where T<:AbstractFloat (the method Float64
// arguments dispatch to from src/eigenSelfAdjoint.jl:393,428): r = sqrt(f^2+g^2)
// with power-of-two rescaling near over/underflow, and (c,s,r) negated when
// |f| > |g| and c < 0.
template <class T> void givens_lapack(T f, T g, T& cs, T& sn, T& r) {
  typedef num<T> N;
  if (g == 0) { cs = 1; sn = 0; r = f; return; }
  if (f == 0) { cs = 0; sn = 1; r = g; return; }
  const T safmn2 = N::safmn2();
  const T safmx2 = 1 / safmn2;
  T f1 = f, g1 = g;
  T scale = std::max(N::abs(f1), N::abs(g1));
  if (scale >= safmx2) {
    int count = 0;
    do {
      count++;
      f1 *= safmn2;
      g1 *= safmn2;
      scale = std::max(N::abs(f1), N::abs(g1));
    } while (scale >= safmx2 && count < 20);
    r = N::sqrt(f1 * f1 + g1 * g1);
    cs = f1 / r;
    sn = g1 / r;
    for (int i = 0; i < count; i++) r *= safmx2;
  } else if (scale <= safmn2) {
    int count = 0;
    do {
      count++;
      f1 *= safmx2;
      g1 *= safmx2;
      scale = std::max(N::abs(f1), N::abs(g1));
    } while (scale <= safmn2);
    r = N::sqrt(f1 * f1 + g1 * g1);
    cs = f1 / r;
    sn = g1 / r;
    for (int i = 0; i < count; i++) r *= safmn2;
  } else {
    r = N::sqrt(f1 * f1 + g1 * g1);
    cs = f1 / r;
    sn = g1 / r;
  }
  if (N::abs(f) > N::abs(g) && cs < 0) {
    cs = -cs;
    sn = -sn;
    r = -r;
  }
}

// The package's own generic method (src/eigenSelfAdjoint.jl:706-709).
template <class T> void givens_generic(T f, T g, T& c, T& s, T& r) {
  T h = hypot_borges(f, g);
  c = f / h;
  s = g / h;
  r = h;
}

template <class T> struct Opts {
  T tol;
  bool generic_givens = false;  // false: stdlib dlartg port (Float64 dispatch)
  int64_t max_sweeps = -1;      // -1: 30*n (the reference has no cap)
  int64_t nrot = 0;             // out: rotations applied to the vectors
  int64_t nsweeps = 0;          // out: implicit-shift chases
};

template <class T> void givens(const Opts<T>& o, T f, T g, T& c, T& s, T& r) {
  if (o.generic_givens) givens_generic(f, g, c, s, r);
  else givens_lapack(f, g, c, s, r);
}

// _updateVectors! (src/eigenSelfAdjoint.jl:121-128): columns j, j+1 (0-based j).
// The vectors' type VT is T, or std::complex<T> for complex Hermitian input
// (real rotations on complex eigenvectors).
template <class T, class VT> void update_vectors(T c, T s, int64_t j, VT* V, int64_t ldv, int64_t m) {
  VT* a = V + j * ldv;
  VT* b = V + (j + 1) * ldv;
  for (int64_t i = 0; i < m; i++) {
    VT v1 = b[i];
    VT v2 = a[i];
    b[i] = c * v1 + s * v2;
    a[i] = c * v2 - s * v1;
  }
}

// eigvals2x2 (:131-135)
template <class T> void eigvals2x2(T d1, T d2, T e, T& lp, T& lm) {
  T r1 = (d1 + d2) / 2;
  T r2 = hypot_borges(d1 - d2, 2 * e) / 2;
  lp = r1 + r2;
  lm = r1 - r2;
}

// eig2x2! (:136-161), j 0-based.
template <class T, class VT> void eig2x2(T* d, T* e, int64_t j, VT* V, int64_t ldv, int64_t m, T& c, T& s) {
  typedef num<T> N;
  T dj = d[j], dj1 = d[j + 1], ej = e[j];
  T r1 = (dj + dj1) / 2;
  T r2 = hypot_borges(dj - dj1, 2 * ej) / 2;
  T lp = r1 + r2, lm = r1 - r2;
  d[j] = lp;
  d[j + 1] = lm;
  e[j] = 0;
  if (ej == 0) {
    c = 1;
    s = 0;
  } else if (N::abs(lp - dj) > N::abs(lm - dj)) {
    c = -ej / hypot_borges(ej, lp - dj);
    s = N::sqrt(1 - c * c);
  } else {
    s = N::abs(ej) / hypot_borges(ej, lm - dj);
    c = N::copysign(N::sqrt(1 - s * s), -ej);
  }
  update_vectors(c, s, j, V, ldv, m);
}

// singleShiftQLPWK! (:343-374), istart/iend 0-based inclusive; e holds squares.
template <class T> void single_shift_ql_pwk(T* d, T* e, T shift, int64_t istart, int64_t iend) {
  T gi = d[iend] - shift;
  T p = gi * gi;
  T ci = 1, s = 0;
  for (int64_t i = iend - 1; i >= istart; i--) {
    T ei = e[i];
    T zeta = p + ei;
    if (i < iend - 1) e[i + 1] = s * zeta;
    T ci1 = ci;
    ci = p / zeta;
    s = ei / zeta;
    T di = d[i];
    T gi1 = gi;
    gi = ci * (di - shift) - s * gi1;
    d[i + 1] = gi1 + di - gi;
    p = ci == 0 ? ei * ci1 : gi * gi / ci;
  }
  e[istart] = s * p;
  d[istart] = shift + gi;
}

// singleShiftQL! (:377-409)
template <class T, class VT>
void single_shift_ql(Opts<T>& o, T* d, T* e, T shift, int64_t istart, int64_t iend, VT* V, int64_t ldv, int64_t m) {
  T gi = d[iend] - shift;
  T p = gi;
  T ci = 1, si = 0;
  for (int64_t i = iend - 1; i >= istart; i--) {
    T ei = e[i];
    T ci1 = ci, si1 = si, zeta;
    givens(o, p, ei, ci, si, zeta);
    if (i < iend - 1) e[i + 1] = si1 * zeta;
    T di = d[i];
    T gi1 = gi;
    gi = ci * ci * (di - shift) - si * si * gi1;
    d[i + 1] = gi1 + di - gi;
    p = ci == 0 ? -ei * ci1 : gi / ci;
    update_vectors(ci, si, i, V, ldv, m);
    o.nrot++;
  }
  e[istart] = si * p;
  d[istart] = shift + gi;
}

// singleShiftQR! (:412-444)
template <class T, class VT>
void single_shift_qr(Opts<T>& o, T* d, T* e, T shift, int64_t istart, int64_t iend, VT* V, int64_t ldv, int64_t m) {
  T gi = d[istart] - shift;
  T p = gi;
  T ci = 1, si = 0;
  for (int64_t i = istart + 1; i <= iend; i++) {
    T ei = e[i - 1];
    T ci1 = ci, si1 = si, zeta;
    givens(o, p, ei, ci, si, zeta);
    if (i > istart + 1) e[i - 2] = si1 * zeta;
    T di = d[i];
    T gi1 = gi;
    gi = ci * ci * (di - shift) - si * si * gi1;
    d[i - 1] = gi1 + di - gi;
    p = ci == 0 ? -ei * ci1 : gi / ci;
    update_vectors(ci, -si, i - 1, V, ldv, m);
    o.nrot++;
  }
  e[iend - 1] = si * p;
  d[iend] = shift + gi;
}

// Deflation scan shared by eigQL!/eigQR!/eigvalsPWK! (:176-182, :250-256, :303-309):
// first be in (blockstart+1 .. n) (1-based) with |e[be-1]| <= tol*sqrt|d[be-1]|*sqrt|d[be]|.
// Returns blockend, 0-based.
template <class T> int64_t find_blockend(const T* d, const T* e, int64_t n, int64_t bs, T tol) {
  typedef num<T> N;
  int64_t blockend = n - 1;
  for (int64_t be = bs + 1; be <= n - 1; be++) {
    if (N::abs(e[be - 1]) <= tol * N::sqrt(N::abs(d[be - 1])) * N::sqrt(N::abs(d[be]))) {
      return be - 1;
    }
    blockend = n - 1;
  }
  return blockend;
}

// Number of off-diagonal entries still above the deflation threshold (LAPACK
// dsteqr reports this count as info when it gives up).
template <class T> int count_unconverged(const T* d, const T* e, int64_t n, T tol) {
  typedef num<T> N;
  int c = 0;
  for (int64_t i = 0; i + 1 < n; i++)
    if (!(N::abs(e[i]) <= tol * N::sqrt(N::abs(d[i])) * N::sqrt(N::abs(d[i + 1])))) c++;
  return c;
}

// eigvalsPWK! (:163-219). Returns 0 or the unconverged count when the sweep
// cap (an addition: the reference loops forever on e.g. NaN input) is hit.
template <class T> int eigvals_pwk(Opts<T>& o, T* d, T* e, int64_t n) {
  typedef num<T> N;
  int64_t cap = o.max_sweeps >= 0 ? o.max_sweeps : 30 * n;
  for (int64_t i = 0; i + 1 < n; i++) e[i] = e[i] * e[i];
  int64_t bs = 0, be = n - 1;
  if (n <= 1) return 0;
  while (true) {
    be = find_blockend(d, e, n, bs, o.tol);
    if (bs == be) {
      bs += 1;
    } else if (bs + 1 == be) {
      T lp, lm;
      eigvals2x2(d[bs], d[be], N::sqrt(e[bs]), lp, lm);
      d[bs] = lp;
      d[be] = lm;
      e[bs] = 0;
      bs += 1;
    } else {
      if (o.nsweeps >= cap) {
        // restore |e| for the count
        std::vector<T> ea(n - 1);
        for (int64_t i = 0; i + 1 < n; i++) ea[i] = N::sqrt(N::abs(e[i]));
        return std::max(1, count_unconverged(d, ea.data(), n, o.tol));
      }
      T sqrte = N::sqrt(e[bs]);
      T mu = (d[bs + 1] - d[bs]) / (2 * sqrte);
      T r = hypot_borges(mu, (T)1);
      mu = d[bs] - sqrte / (mu + N::copysign(r, mu));
      single_shift_ql_pwk(d, e, mu, bs, be);
      o.nsweeps++;
      o.nrot += be - bs;
    }
    if (bs >= n - 1) break;
  }
  return 0;
}

// eigQL! (:221-288); V is m x n (m <= n rows), column-major ldv.
template <class T, class VT> int eig_ql(Opts<T>& o, T* d, T* e, int64_t n, VT* V, int64_t ldv, int64_t m) {
  typedef num<T> N;
  int64_t cap = o.max_sweeps >= 0 ? o.max_sweeps : 30 * n;
  int64_t bs = 0, be = n - 1;
  if (n <= 1) return 0;
  while (true) {
    be = find_blockend(d, e, n, bs, o.tol);
    if (bs == be) {
      bs += 1;
    } else if (bs + 1 == be) {
      T c, s;
      eig2x2(d, e, bs, V, ldv, m, c, s);
      o.nrot++;
      bs += 2;
    } else {
      if (o.nsweeps >= cap) return std::max(1, count_unconverged(d, e, n, o.tol));
      T mu = (d[bs + 1] - d[bs]) / (2 * e[bs]);
      T r = hypot_borges(mu, (T)1);
      mu = d[bs] - (e[bs] / (mu + N::copysign(r, mu)));
      single_shift_ql(o, d, e, mu, bs, be, V, ldv, m);
      o.nsweeps++;
    }
    if (bs >= n - 1) break;
  }
  return 0;
}

// eigQR! (:290-340)
template <class T, class VT> int eig_qr(Opts<T>& o, T* d, T* e, int64_t n, VT* V, int64_t ldv, int64_t m) {
  typedef num<T> N;
  int64_t cap = o.max_sweeps >= 0 ? o.max_sweeps : 30 * n;
  int64_t bs = 0, be = n - 1;
  if (n <= 1) return 0;
  while (true) {
    be = find_blockend(d, e, n, bs, o.tol);
    if (bs == be) {
      bs += 1;
    } else if (bs + 1 == be) {
      T c, s;
      eig2x2(d, e, bs, V, ldv, m, c, s);
      o.nrot++;
      bs += 2;
    } else {
      if (o.nsweeps >= cap) return std::max(1, count_unconverged(d, e, n, o.tol));
      T mu = (d[be - 1] - d[be]) / (2 * e[be - 1]);
      T r = hypot_borges(mu, (T)1);
      mu = d[be] - (e[be - 1] / (mu + N::copysign(r, mu)));
      single_shift_qr(o, d, e, mu, bs, be, V, ldv, m);
      o.nsweeps++;
    }
    if (bs >= n - 1) break;
  }
  return 0;
}

// netlib reference dsymv, lower triangle, y = alpha*A*x (beta = 0).
template <class T> void symv_lower(int64_t n, T alpha, const T* A, int64_t lda, const T* x, T* y) {
  for (int64_t i = 0; i < n; i++) y[i] = 0;
  for (int64_t j = 0; j < n; j++) {
    T temp1 = alpha * x[j];
    T temp2 = 0;
    y[j] += temp1 * A[j + j * lda];
    for (int64_t i = j + 1; i < n; i++) {
      y[i] += temp1 * A[i + j * lda];
      temp2 += A[i + j * lda] * x[i];
    }
    y[j] += alpha * temp2;
  }
}

// netlib reference dsymv, upper triangle, y = alpha*A*x (beta = 0).
template <class T> void symv_upper(int64_t n, T alpha, const T* A, int64_t lda, const T* x, T* y) {
  for (int64_t i = 0; i < n; i++) y[i] = 0;
  for (int64_t j = 0; j < n; j++) {
    T temp1 = alpha * x[j];
    T temp2 = 0;
    for (int64_t i = 0; i < j; i++) {
      y[i] += temp1 * A[i + j * lda];
      temp2 += A[i + j * lda] * x[i];
    }
    y[j] += temp1 * A[j + j * lda] + alpha * temp2;
  }
}

template <class T> T dot(const T* x, const T* y, int64_t n) {
  T s = 0;
  for (int64_t i = 0; i < n; i++) s += x[i] * y[i];
  return s;
}

// symtriLower! (:450-504). On return AS holds the reflectors below the
// subdiagonal, d/e the tridiagonal, tau (n-1, last entry 0).
template <class T> void symtri_lower(int64_t n, T* AS, int64_t lda, T* tau, T* d, T* e) {
  std::vector<T> u(std::max<int64_t>(n, 1));
  for (int64_t k = 0; k + 1 < n; k++) tau[k] = 0;
  for (int64_t k = 0; k + 2 < n; k++) {  // k = 1:(n-2) in 1-based terms
    int64_t m = n - k - 1;                // length of x = AS[k+1:n, k]
    T* x = &at(AS, lda, k + 1, k);
    T tk = reflector(x, m, 1);
    tau[k] = tk;
    T tmp = x[0];
    x[0] = 1;
    T* At = &at(AS, lda, k + 1, k + 1);
    T* ut = u.data() + k + 1;
    symv_lower(m, tk, At, lda, x, ut);
    T xi = tk * dot(x, ut, m);
    for (int64_t j = 0; j < m; j++) {
      T xj = x[j], uj = ut[j], xixj = xi * xj;
      for (int64_t i = j; i < m; i++) {
        at(AS, lda, k + 1 + i, k + 1 + j) += x[i] * xixj - x[i] * uj - ut[i] * xj;
      }
    }
    x[0] = tmp;
  }
  for (int64_t i = 0; i < n; i++) d[i] = at(AS, lda, i, i);
  for (int64_t i = 0; i + 1 < n; i++) e[i] = at(AS, lda, i + 1, i);
}

// symtriUpper! (:507-564). Reflector k (0-based) acts on rows 0..n-k-2 and
// lives in column n-k-1 above the superdiagonal.
template <class T> void symtri_upper(int64_t n, T* AS, int64_t lda, T* tau, T* d, T* e) {
  std::vector<T> u(std::max<int64_t>(n, 1)), xr(std::max<int64_t>(n, 1));
  for (int64_t k = 0; k + 1 < n; k++) tau[k] = 0;
  for (int64_t k = 0; k + 2 < n; k++) {
    int64_t m = n - k - 1;           // x = AS[1:(n-k), n-k+1] (1-based)
    T* x = &at(AS, lda, 0, n - k - 1);
    // reflector on the reversed view xr = AS[(n-k):-1:1, n-k+1]
    T tk = reflector(x + (m - 1), m, -1);
    tau[k] = tk;
    T tmp = x[m - 1];
    x[m - 1] = 1;
    symv_upper(m, tk, AS, lda, x, u.data());
    T xi = tk * dot(x, u.data(), m);
    for (int64_t j = 0; j < m; j++) {
      T xj = x[j], uj = u[j], xixj = xi * xj;
      for (int64_t i = 0; i <= j; i++) {
        at(AS, lda, i, j) += x[i] * xixj - x[i] * uj - u[i] * xj;
      }
    }
    x[m - 1] = tmp;
  }
  for (int64_t i = 0; i < n; i++) d[i] = at(AS, lda, i, i);
  for (int64_t i = 0; i + 1 < n; i++) e[i] = at(AS, lda, i, i + 1);
}

// lmul!(Q::EigenQ, B) (:23-60): B (n x ncols) <- Q*B. Mirrors the reference
// exactly, including that the stored reflector head ends up holding the last
// column's tmp (the restore at :40/:54 writes the loop variable).
template <class T>
void eigenq_lmul(char uplo, int64_t n, T* F, int64_t ldf, const T* tau, T* B, int64_t ldb, int64_t ncols) {
  int64_t ntau = n - 1;
  if (uplo == 'L') {
    for (int64_t k = ntau; k >= 1; k--) {  // 1-based k
      T* h = &at(F, ldf, k, k - 1);        // view(F, (k+1):m, k)
      int64_t len = n - k;
      T t = tau[k - 1];
      T tmp = h[0];
      h[0] = 1;
      for (int64_t j = 0; j < ncols; j++) {
        T* Bj = &at(B, ldb, k, j);
        tmp = t * dot(h, Bj, len);
        for (int64_t i = 0; i < len; i++) Bj[i] -= h[i] * tmp;
      }
      h[0] = tmp;
    }
  } else {
    for (int64_t k = ntau; k >= 1; k--) {
      int64_t len = n - k;
      T* h = &at(F, ldf, 0, n - k);        // view(F, 1:(m-k), m-k+1)
      T t = tau[k - 1];
      T tmp = h[len - 1];
      h[len - 1] = 1;
      for (int64_t j = 0; j < ncols; j++) {
        T* Bj = &at(B, ldb, 0, j);
        tmp = t * dot(h, Bj, len);
        for (int64_t i = 0; i < len; i++) Bj[i] -= h[i] * tmp;
      }
      h[len - 1] = tmp;
    }
  }
}

// rmul!(A, Q::EigenQ) (:62-99): A (mrows x n) <- A*Q.
template <class T>
void eigenq_rmul(char uplo, int64_t n, T* F, int64_t ldf, const T* tau, T* A, int64_t lda, int64_t mrows) {
  int64_t ntau = n - 1;
  if (uplo == 'L') {
    for (int64_t k = 1; k <= ntau; k++) {
      T* h = &at(F, ldf, k, k - 1);
      int64_t len = n - k;
      T t = tau[k - 1];
      T tmp = h[0];
      h[0] = 1;
      for (int64_t i = 0; i < mrows; i++) {
        T s = 0;
        for (int64_t jj = 0; jj < len; jj++) s += at(A, lda, i, k + jj) * h[jj];
        tmp = s * t;
        for (int64_t jj = 0; jj < len; jj++) at(A, lda, i, k + jj) -= tmp * h[jj];
      }
      h[0] = tmp;
    }
  } else {
    for (int64_t k = 1; k <= ntau; k++) {
      int64_t len = n - k;
      T* h = &at(F, ldf, 0, n - k);
      T t = tau[k - 1];
      T tmp = h[len - 1];
      h[len - 1] = 1;
      for (int64_t i = 0; i < mrows; i++) {
        T s = 0;
        for (int64_t jj = 0; jj < len; jj++) s += at(A, lda, i, jj) * h[jj];
        tmp = s * t;
        for (int64_t jj = 0; jj < len; jj++) at(A, lda, i, jj) -= tmp * h[jj];
      }
      h[len - 1] = tmp;
    }
  }
}

// isless on reals: -0.0 before 0.0, NaN last (LinearAlgebra.eigsortby = identity for reals).
template <class T> bool isless(T a, T b) {
  typedef num<T> N;
  if (a != a) return false;
  if (b != b) return true;
  if (a < b) return true;
  if (a == b) return N::signbit(a) && !N::signbit(b);
  return false;
}

// sorteig!: stable ascending sort of w with the columns of V (m x n) permuted to match.
template <class T, class VT = T> void sorteig(T* w, int64_t n, VT* V, int64_t ldv, int64_t m) {
  std::vector<int64_t> p(n);
  std::iota(p.begin(), p.end(), 0);
  std::stable_sort(p.begin(), p.end(), [&](int64_t a, int64_t b) { return isless(w[a], w[b]); });
  std::vector<T> wt(n);
  for (int64_t i = 0; i < n; i++) wt[i] = w[p[i]];
  for (int64_t i = 0; i < n; i++) w[i] = wt[i];
  if (V && m > 0) {
    std::vector<VT> Vt((size_t)m * n);
    for (int64_t j = 0; j < n; j++)
      for (int64_t i = 0; i < m; i++) Vt[i + j * m] = V[i + p[j] * ldv];
    for (int64_t j = 0; j < n; j++)
      for (int64_t i = 0; i < m; i++) V[i + j * ldv] = Vt[i + j * m];
  }
}

template <class T> bool all_finite_tri(char uplo, int64_t n, const T* A, int64_t lda) {
  typedef num<T> N;
  for (int64_t j = 0; j < n; j++) {
    int64_t i0 = uplo == 'L' ? j : 0, i1 = uplo == 'L' ? n : j + 1;
    for (int64_t i = i0; i < i1; i++)
      if (!N::isfinite(A[i + j * lda])) return false;
  }
  return true;
}

// _eigen!(Hermitian) / _eigvals!(Hermitian) (:566-618): symtri!, then
// eigvalsPWK! (values) or Array(Q) + eigQL!/eigQR! (vectors), then sorteig!.
// A is overwritten (as the reference's eigen! does). Returns info:
// 0 ok, >0 unconverged count, -1 non-finite input.
template <class T>
int syev(Opts<T>& o, char jobz, char uplo, int64_t n, T* A, int64_t lda, T* w, T* V, int64_t ldv, bool use_qr) {
  if (n == 0) return 0;
  if (!all_finite_tri(uplo, n, A, lda)) {
    for (int64_t i = 0; i < n; i++) w[i] = std::numeric_limits<double>::quiet_NaN();
    return -1;
  }
  std::vector<T> tau(std::max<int64_t>(n - 1, 1)), e(std::max<int64_t>(n - 1, 1));
  if (uplo == 'L') symtri_lower(n, A, lda, tau.data(), w, e.data());
  else symtri_upper(n, A, lda, tau.data(), w, e.data());
  int info;
  if (jobz == 'N') {
    info = eigvals_pwk(o, w, e.data(), n);
    sorteig<T, T>(w, n, nullptr, 0, 0);
  } else {
    for (int64_t j = 0; j < n; j++)
      for (int64_t i = 0; i < n; i++) V[i + j * ldv] = (i == j) ? 1 : 0;
    eigenq_lmul(uplo, n, A, lda, tau.data(), V, ldv, n);
    info = use_qr ? eig_qr(o, w, e.data(), n, V, ldv, n) : eig_ql(o, w, e.data(), n, V, ldv, n);
    sorteig(w, n, V, ldv, n);
  }
  return info;
}

// _eigen!(SymTridiagonal) / _eigvals!(SymTridiagonal) (:566-567, :602-612).
template <class T> int stev(Opts<T>& o, char jobz, int64_t n, T* d, T* e, T* V, int64_t ldv, bool use_qr) {
  if (n == 0) return 0;
  int info;
  if (jobz == 'N') {
    info = eigvals_pwk(o, d, e, n);
    sorteig<T, T>(d, n, nullptr, 0, 0);
  } else {
    for (int64_t j = 0; j < n; j++)
      for (int64_t i = 0; i < n; i++) V[i + j * ldv] = (i == j) ? 1 : 0;
    info = use_qr ? eig_qr(o, d, e, n, V, ldv, n) : eig_ql(o, d, e, n, V, ldv, n);
    sorteig(d, n, V, ldv, n);
  }
  return info;
}

// ---- Complex and quaternion Hermitian input: the same algorithm with a
// non-real element type F (std::complex<double>, or Quat below). ----
// The reference runs symtriLower!/symtriUpper! on the non-real matrix with
// one more reflector than for real input (loop bound n-2+!(T<:Real),
// :462/:522), which leaves a real tridiagonal; Array(Q) has type F and
// eigQL! applies its real rotations to those vectors. Stdlib pieces
// restated: reflector! (x[i] /= xi1 with xi1 = x1 + nu, nu =
// copysign(norm(x), real(x1)), tau = xi1/nu: the LAPACK zlarfg reflector
// for complex x, H = I - tau v v', H' x = -nu e1), the Hermitian
// matrix-vector product y = (A x) alpha (for complex, BLAS zhemv: the netlib
// reference loops; the same loops serve quaternions, with the scalar applied
// on the right as Julia's generic 5-argument mul! does) and dot(x, y) =
// sum conj(x_i) y_i. Quaternion products do not commute, so every product is
// written in the reference's order.
typedef std::complex<double> zc;

// A quaternion s + i x + j y + k z (Quaternions.jl's Quaternion{Float64}).
struct Quat {
  double s = 0, x = 0, y = 0, z = 0;
  Quat() = default;
  Quat(double a) : s(a) {}
  Quat(double a, double b, double c, double d) : s(a), x(b), y(c), z(d) {}
  Quat& operator+=(const Quat& q) {
    s += q.s, x += q.x, y += q.y, z += q.z;
    return *this;
  }
  Quat& operator-=(const Quat& q) {
    s -= q.s, x -= q.x, y -= q.y, z -= q.z;
    return *this;
  }
};
inline Quat operator+(Quat a, const Quat& b) { return a += b; }
inline Quat operator-(Quat a, const Quat& b) { return a -= b; }
inline Quat operator-(const Quat& a) { return Quat(-a.s, -a.x, -a.y, -a.z); }
inline Quat operator*(const Quat& p, const Quat& q) {  // Hamilton product
  return Quat(p.s * q.s - p.x * q.x - p.y * q.y - p.z * q.z, p.s * q.x + p.x * q.s + p.y * q.z - p.z * q.y,
              p.s * q.y - p.x * q.z + p.y * q.s + p.z * q.x, p.s * q.z + p.x * q.y - p.y * q.x + p.z * q.s);
}
inline Quat operator*(double a, const Quat& q) { return Quat(a * q.s, a * q.x, a * q.y, a * q.z); }
inline Quat operator*(const Quat& q, double a) { return Quat(q.s * a, q.x * a, q.y * a, q.z * a); }
inline Quat operator/(const Quat& q, double a) { return Quat(q.s / a, q.x / a, q.y / a, q.z / a); }

inline zc conj_(const zc& a) { return std::conj(a); }
inline Quat conj_(const Quat& a) { return Quat(a.s, -a.x, -a.y, -a.z); }
inline double real_(const zc& a) { return a.real(); }
inline double real_(const Quat& a) { return a.s; }
inline double abs2_(const zc& a) { return std::norm(a); }
inline double abs2_(const Quat& a) { return a.s * a.s + a.x * a.x + a.y * a.y + a.z * a.z; }
inline double abs_(const zc& a) { return std::abs(a); }
inline double abs_(const Quat& a) { return std::sqrt(abs2_(a)); }
inline bool finite_(const zc& a) { return std::isfinite(a.real()) && std::isfinite(a.imag()); }
inline bool finite_(const Quat& a) {
  return std::isfinite(a.s) && std::isfinite(a.x) && std::isfinite(a.y) && std::isfinite(a.z);
}
// a / b = a inv(b) (Julia's right division)
inline zc rdiv_(const zc& a, const zc& b) { return a / b; }
inline Quat rdiv_(const Quat& a, const Quat& b) {
  const double m = abs2_(b);
  return a * Quat(b.s / m, -b.x / m, -b.y / m, -b.z / m);
}

template <class F> double norm2f(const F* x, int64_t n, int64_t inc) {
  double maxabs = 0;
  for (int64_t i = 0; i < n; i++) {
    double a = abs_(x[i * inc]);
    if (!(a <= maxabs)) maxabs = a;
  }
  if (maxabs == 0 || !std::isfinite(maxabs)) return maxabs;
  if (std::isfinite((double)n * maxabs * maxabs) && maxabs * maxabs != 0) {
    double sum = 0;
    for (int64_t i = 0; i < n; i++) sum += abs2_(x[i * inc]);
    return std::sqrt(sum);
  }
  double sum = 0;
  for (int64_t i = 0; i < n; i++) sum += abs2_(x[i * inc] / maxabs);
  return maxabs * std::sqrt(sum);
}

template <class F> F reflector_f(F* x, int64_t n, int64_t inc) {
  if (n == 0) return F(0);
  F xi1 = x[0];
  double normu = norm2f(x, n, inc);
  if (normu == 0) return F(0);
  double nu = std::copysign(normu, real_(xi1));
  xi1 += F(nu);
  x[0] = F(-nu);
  for (int64_t i = 1; i < n; i++) x[i * inc] = rdiv_(x[i * inc], xi1);
  return rdiv_(xi1, F(nu));
}

template <class F> F dotc(const F* x, const F* y, int64_t n) {
  F s(0);
  for (int64_t i = 0; i < n; i++) s += conj_(x[i]) * y[i];
  return s;
}

// y = (A x) alpha (beta = 0), the Hermitian A given by its lower / upper
// triangle; the netlib zhemv loops.
template <class F> void hemv_lower(int64_t n, F alpha, const F* A, int64_t lda, const F* x, F* y) {
  for (int64_t i = 0; i < n; i++) y[i] = F(0);
  for (int64_t j = 0; j < n; j++) {
    F temp1 = x[j] * alpha, temp2(0);
    y[j] += real_(A[j + j * lda]) * temp1;
    for (int64_t i = j + 1; i < n; i++) {
      y[i] += A[i + j * lda] * temp1;
      temp2 += conj_(A[i + j * lda]) * x[i];
    }
    y[j] += temp2 * alpha;
  }
}
template <class F> void hemv_upper(int64_t n, F alpha, const F* A, int64_t lda, const F* x, F* y) {
  for (int64_t i = 0; i < n; i++) y[i] = F(0);
  for (int64_t j = 0; j < n; j++) {
    F temp1 = x[j] * alpha, temp2(0);
    for (int64_t i = 0; i < j; i++) {
      y[i] += A[i + j * lda] * temp1;
      temp2 += conj_(A[i + j * lda]) * x[i];
    }
    y[j] += real_(A[j + j * lda]) * temp1 + temp2 * alpha;
  }
}

// symtriLower! (:450-504) for non-real AS: n-1 reflectors; d, e real.
template <class F> void symtri_lower_f(int64_t n, F* AS, int64_t lda, F* tau, double* d, double* e) {
  std::vector<F> u(std::max<int64_t>(n, 1));
  for (int64_t i = 0; i < n; i++) at(AS, lda, i, i) = F(real_(at(AS, lda, i, i)));
  for (int64_t k = 0; k + 1 < n; k++) {  // k = 1:(n-1) in 1-based terms
    int64_t m = n - k - 1;
    F* x = &at(AS, lda, k + 1, k);
    F tk = reflector_f(x, m, 1);
    tau[k] = tk;
    F tmp = x[0];
    x[0] = F(1);
    F* ut = u.data() + k + 1;
    hemv_lower(m, tk, &at(AS, lda, k + 1, k + 1), lda, x, ut);
    double xi = real_(conj_(tk) * dotc(x, ut, m));
    for (int64_t j = 0; j < m; j++) {
      F xj = x[j], uj = ut[j], xixj = xi * xj;
      for (int64_t i = j; i < m; i++)
        at(AS, lda, k + 1 + i, k + 1 + j) += x[i] * conj_(xixj) - x[i] * conj_(uj) - ut[i] * conj_(xj);
    }
    x[0] = tmp;
  }
  for (int64_t i = 0; i < n; i++) d[i] = real_(at(AS, lda, i, i));
  for (int64_t i = 0; i + 1 < n; i++) e[i] = real_(at(AS, lda, i + 1, i));
}

// symtriUpper! (:507-564) for non-real AS.
template <class F> void symtri_upper_f(int64_t n, F* AS, int64_t lda, F* tau, double* d, double* e) {
  std::vector<F> u(std::max<int64_t>(n, 1));
  for (int64_t i = 0; i < n; i++) at(AS, lda, i, i) = F(real_(at(AS, lda, i, i)));
  for (int64_t k = 0; k + 1 < n; k++) {
    int64_t m = n - k - 1;
    F* x = &at(AS, lda, 0, n - k - 1);
    F tk = reflector_f(x + (m - 1), m, -1);  // the reversed view AS[(n-k):-1:1, n-k+1]
    tau[k] = tk;
    F tmp = x[m - 1];
    x[m - 1] = F(1);
    hemv_upper(m, tk, AS, lda, x, u.data());
    double xi = real_(conj_(tk) * dotc(x, u.data(), m));
    for (int64_t j = 0; j < m; j++) {
      F xj = x[j], uj = u[j], xixj = xi * xj;
      for (int64_t i = 0; i <= j; i++) at(AS, lda, i, j) += x[i] * conj_(xixj) - x[i] * conj_(uj) - u[i] * conj_(xj);
    }
    x[m - 1] = tmp;
  }
  for (int64_t i = 0; i < n; i++) d[i] = real_(at(AS, lda, i, i));
  for (int64_t i = 0; i + 1 < n; i++) e[i] = real_(at(AS, lda, i, i + 1));
}

// lmul!(Q::EigenQ, B) (:23-60) for non-real factors: B (n x ncols) <- Q*B,
// tmp = tau * (h' * b), b -= h * tmp.
template <class F>
void eigenq_lmul_f(char uplo, int64_t n, F* Fm, int64_t ldf, const F* tau, F* B, int64_t ldb, int64_t ncols) {
  for (int64_t k = n - 1; k >= 1; k--) {  // 1-based k over length(tau) = n-1
    const int64_t len = n - k;
    F* h = uplo == 'L' ? &at(Fm, ldf, k, k - 1) : &at(Fm, ldf, 0, n - k);
    const int64_t head = uplo == 'L' ? 0 : len - 1;
    const F t = tau[k - 1];
    F tmp = h[head];
    h[head] = F(1);
    for (int64_t j = 0; j < ncols; j++) {
      F* Bj = uplo == 'L' ? &at(B, ldb, k, j) : &at(B, ldb, 0, j);
      tmp = t * dotc(h, Bj, len);
      for (int64_t i = 0; i < len; i++) Bj[i] -= h[i] * tmp;
    }
    h[head] = tmp;
  }
}

// _eigen!/_eigvals!(Hermitian{F}): symtri!, then eigvalsPWK! (values) or
// Array(Q) + eigQL! (vectors), then sorteig!. Returns info.
template <class F>
int heev(Opts<double>& o, char jobz, char uplo, int64_t n, F* A, int64_t lda, double* w, F* V, int64_t ldv) {
  if (n == 0) return 0;
  for (int64_t j = 0; j < n; j++) {
    int64_t i0 = uplo == 'L' ? j : 0, i1 = uplo == 'L' ? n : j + 1;
    for (int64_t i = i0; i < i1; i++)
      if (!finite_(A[i + j * lda])) {
        for (int64_t q = 0; q < n; q++) w[q] = std::numeric_limits<double>::quiet_NaN();
        return -1;
      }
  }
  std::vector<F> tau(std::max<int64_t>(n - 1, 1));
  std::vector<double> e(std::max<int64_t>(n - 1, 1));
  if (uplo == 'L') symtri_lower_f(n, A, lda, tau.data(), w, e.data());
  else symtri_upper_f(n, A, lda, tau.data(), w, e.data());
  int info;
  if (jobz == 'N') {
    info = eigvals_pwk(o, w, e.data(), n);
    sorteig<double, double>(w, n, nullptr, 0, 0);
  } else {
    for (int64_t j = 0; j < n; j++)
      for (int64_t i = 0; i < n; i++) V[i + j * ldv] = F(i == j ? 1.0 : 0.0);
    eigenq_lmul_f(uplo, n, A, lda, tau.data(), V, ldv, n);
    info = eig_ql(o, w, e.data(), n, V, ldv, n);
    sorteig(w, n, V, ldv, n);
  }
  return info;
}

// numnegevals (src/tridiag.jl:20-36): the number of negative eigenvalues of
// T - sigma I by the LDL' (Sturm) recurrence of Parlett, "The symmetric
// eigenvalue problem", 3.3.1: delta_1 = a_1 - sigma,
// delta_{k+1} = (a_{k+1} - sigma) - b_k (b_k / delta_k), counting the
// negative deltas; a zero delta is replaced by eps (b_k + eps) as the
// reference does. Evaluated in exactly this operation order (the oracle is
// built without contraction).
template <class T> int64_t numnegevals(const T* a, const T* b, int64_t n, T sigma) {
  if (n <= 0) return 0;
  const T eps = num<T>::eps();
  T delta = a[0] - sigma;
  int64_t nu = delta < T(0) ? 1 : 0;
  for (int64_t k = 0; k + 1 < n; k++) {
    if (delta == T(0)) delta = eps * (b[k] + eps);
    delta = (a[k + 1] - sigma) - b[k] * (b[k] / delta);
    nu += delta < T(0) ? 1 : 0;
  }
  return nu;
}

}  // namespace gla_oracle
