// CPU ORACLE — test infrastructure only (tests/, the smoke check and the
// CPU-baseline leg of the benchmark). C entry points over gla_ref.hpp, the
// restatement of GenericLinearAlgebra.jl src/eigenSelfAdjoint.jl.
//
// Suffixes: _d Float64, _s Float32, _q binary128 (inputs/outputs as double;
// _q results are additionally returned as a (hi, lo) double pair so that the
// extra precision survives the trip to numpy).
#include <omp.h>

#include <cstring>

#include "gla_ref.hpp"

using namespace gla_oracle;

namespace {

template <class T>
Opts<T> make_opts(T tol, int generic_givens, int64_t max_sweeps) {
  Opts<T> o;
  o.tol = tol;
  o.generic_givens = generic_givens != 0;
  o.max_sweeps = max_sweeps;
  return o;
}

template <class T>
int syev_one(char jobz, char uplo, int64_t n, T* A, int64_t lda, T* w, T* V, int64_t ldv, T tol, int use_qr,
             int generic_givens, int64_t max_sweeps, int64_t* nrot, int64_t* nsweeps) {
  Opts<T> o = make_opts<T>(tol, generic_givens, max_sweeps);
  int info = syev(o, jobz, uplo, n, A, lda, w, V, ldv, use_qr != 0);
  if (nrot) *nrot = o.nrot;
  if (nsweeps) *nsweeps = o.nsweeps;
  return info;
}

}  // namespace

extern "C" {

// eigen!/eigvals! on Hermitian(A, uplo): A (n x n, column-major lda) is
// overwritten by the factorisation. jobz 'N' -> eigvalsPWK!, 'V' -> Array(Q)
// then eigQL! (use_qr: eigQR!). tol <= 0 selects eps(T). Returns info.
int gla_oracle_syev_d(char jobz, char uplo, int64_t n, double* A, int64_t lda, double* w, double* V, int64_t ldv,
                      double tol, int use_qr, int generic_givens, int64_t max_sweeps, int64_t* nrot,
                      int64_t* nsweeps) {
  if (tol <= 0) tol = num<double>::eps();
  return syev_one<double>(jobz, uplo, n, A, lda, w, V, ldv, tol, use_qr, generic_givens, max_sweeps, nrot, nsweeps);
}

int gla_oracle_syev_s(char jobz, char uplo, int64_t n, float* A, int64_t lda, float* w, float* V, int64_t ldv,
                      float tol, int use_qr, int generic_givens, int64_t max_sweeps, int64_t* nrot,
                      int64_t* nsweeps) {
  if (tol <= 0) tol = num<float>::eps();
  return syev_one<float>(jobz, uplo, n, A, lda, w, V, ldv, tol, use_qr, generic_givens, max_sweeps, nrot, nsweeps);
}

// binary128 run of the same algorithm; A is given in double and rounded up
// exactly. w_hi/w_lo and V_hi/V_lo receive the quad results as double pairs.
int gla_oracle_syev_q(char jobz, char uplo, int64_t n, const double* A, int64_t lda, double* w_hi, double* w_lo,
                      double* V_hi, double* V_lo, int64_t ldv, int use_qr, int generic_givens, int64_t* nrot) {
  std::vector<gla_quad> Aq((size_t)n * n), wq(n), Vq((size_t)n * n);
  for (int64_t j = 0; j < n; j++)
    for (int64_t i = 0; i < n; i++) Aq[i + j * n] = (gla_quad)A[i + j * lda];
  Opts<gla_quad> o = make_opts<gla_quad>(num<gla_quad>::eps(), generic_givens, -1);
  int info = syev(o, jobz, uplo, n, Aq.data(), n, wq.data(), Vq.data(), n, use_qr != 0);
  for (int64_t i = 0; i < n; i++) {
    w_hi[i] = (double)wq[i];
    w_lo[i] = (double)(wq[i] - (gla_quad)w_hi[i]);
  }
  if (jobz == 'V') {
    for (int64_t j = 0; j < n; j++)
      for (int64_t i = 0; i < n; i++) {
        gla_quad v = Vq[i + j * n];
        V_hi[i + j * ldv] = (double)v;
        V_lo[i + j * ldv] = (double)(v - (gla_quad)V_hi[i + j * ldv]);
      }
  }
  if (nrot) *nrot = o.nrot;
  return info;
}

// eigen!/eigvals! on SymTridiagonal(d, e) (d: n, e: n-1, overwritten).
int gla_oracle_stev_d(char jobz, int64_t n, double* d, double* e, double* V, int64_t ldv, double tol, int use_qr,
                      int generic_givens, int64_t max_sweeps, int64_t* nrot) {
  if (tol <= 0) tol = num<double>::eps();
  Opts<double> o = make_opts<double>(tol, generic_givens, max_sweeps);
  int info = stev(o, jobz, n, d, e, V, ldv, use_qr != 0);
  if (nrot) *nrot = o.nrot;
  return info;
}

int gla_oracle_stev_s(char jobz, int64_t n, float* d, float* e, float* V, int64_t ldv, float tol, int use_qr,
                      int generic_givens, int64_t max_sweeps, int64_t* nrot) {
  if (tol <= 0) tol = num<float>::eps();
  Opts<float> o = make_opts<float>(tol, generic_givens, max_sweeps);
  int info = stev(o, jobz, n, d, e, V, ldv, use_qr != 0);
  if (nrot) *nrot = o.nrot;
  return info;
}

// eigQL!/eigQR! on (d, e) with an m x n vectors matrix (m <= n rows), no sort
// (the raw sweep, as eigen2! uses it with m = 2).
int gla_oracle_eigql_d(int64_t n, double* d, double* e, double* V, int64_t ldv, int64_t m, double tol, int use_qr,
                       int generic_givens, int64_t* nrot) {
  if (tol <= 0) tol = num<double>::eps();
  Opts<double> o = make_opts<double>(tol, generic_givens, -1);
  int info = use_qr ? eig_qr(o, d, e, n, V, ldv, m) : eig_ql(o, d, e, n, V, ldv, m);
  if (nrot) *nrot = o.nrot;
  return info;
}

// symtri! on Hermitian(A, uplo): reflectors left in A, tau (n-1), d (n), e (n-1).
void gla_oracle_symtri_d(char uplo, int64_t n, double* A, int64_t lda, double* tau, double* d, double* e) {
  if (uplo == 'L') symtri_lower(n, A, lda, tau, d, e);
  else symtri_upper(n, A, lda, tau, d, e);
}

// eigen!/eigvals! on Hermitian{ComplexF64}(A, uplo): A is n x n complex,
// interleaved (re, im) doubles, column-major lda, overwritten by the
// factorisation; w real ascending; V (jobz 'V') complex, interleaved.
// tol <= 0 selects eps(Float64). Returns info.
int gla_oracle_heev_z(char jobz, char uplo, int64_t n, double* A, int64_t lda, double* w, double* V, int64_t ldv,
                      double tol) {
  Opts<double> o;
  o.tol = tol > 0 ? tol : num<double>::eps();
  return heev(o, jobz, uplo, n, reinterpret_cast<zc*>(A), lda, w, reinterpret_cast<zc*>(V), ldv);
}

// symtri! on Hermitian{ComplexF64}: factors (interleaved complex) in A, tau
// (n-1 complex, interleaved), d and e real.
void gla_oracle_symtri_z(char uplo, int64_t n, double* A, int64_t lda, double* tau, double* d, double* e) {
  if (uplo == 'L') symtri_lower_f(n, reinterpret_cast<zc*>(A), lda, reinterpret_cast<zc*>(tau), d, e);
  else symtri_upper_f(n, reinterpret_cast<zc*>(A), lda, reinterpret_cast<zc*>(tau), d, e);
}

// The same for Hermitian{Quaternion{Float64}}: quaternions are 4 doubles
// (s, i, j, k), matrices column-major with lda counted in quaternions.
int gla_oracle_heev_q(char jobz, char uplo, int64_t n, double* A, int64_t lda, double* w, double* V, int64_t ldv,
                      double tol) {
  static_assert(sizeof(Quat) == 4 * sizeof(double), "Quat is four packed doubles");
  Opts<double> o;
  o.tol = tol > 0 ? tol : num<double>::eps();
  return heev(o, jobz, uplo, n, reinterpret_cast<Quat*>(A), lda, w, reinterpret_cast<Quat*>(V), ldv);
}
void gla_oracle_symtri_qt(char uplo, int64_t n, double* A, int64_t lda, double* tau, double* d, double* e) {
  if (uplo == 'L') symtri_lower_f(n, reinterpret_cast<Quat*>(A), lda, reinterpret_cast<Quat*>(tau), d, e);
  else symtri_upper_f(n, reinterpret_cast<Quat*>(A), lda, reinterpret_cast<Quat*>(tau), d, e);
}
// lmul!(Q::EigenQ, B) for quaternion factors (B: n x ncols quaternions).
void gla_oracle_eigenq_lmul_qt(char uplo, int64_t n, double* F, int64_t ldf, const double* tau, double* B,
                               int64_t ldb, int64_t ncols) {
  eigenq_lmul_f(uplo, n, reinterpret_cast<Quat*>(F), ldf, reinterpret_cast<const Quat*>(tau),
                reinterpret_cast<Quat*>(B), ldb, ncols);
}

// lmul!(Q::EigenQ, B) and rmul!(B, Q::EigenQ) with Q given by (uplo, F, tau).
void gla_oracle_eigenq_lmul_d(char uplo, int64_t n, double* F, int64_t ldf, const double* tau, double* B, int64_t ldb,
                              int64_t ncols) {
  eigenq_lmul(uplo, n, F, ldf, tau, B, ldb, ncols);
}
void gla_oracle_eigenq_rmul_d(char uplo, int64_t n, double* F, int64_t ldf, const double* tau, double* B, int64_t ldb,
                              int64_t mrows) {
  eigenq_rmul(uplo, n, F, ldf, tau, B, ldb, mrows);
}

// eig2x2! (d[j], d[j+1], e[j]) with a 2 x 2 vectors matrix; returns c, s.
void gla_oracle_eig2x2_d(double* d, double* e, double* V, double* c, double* s) {
  eig2x2<double>(d, e, 0, V, 2, 2, *c, *s);
}

void gla_oracle_givens_d(double f, double g, int generic, double* c, double* s, double* r) {
  if (generic) givens_generic(f, g, *c, *s, *r);
  else givens_lapack(f, g, *c, *s, *r);
}

double gla_oracle_hypot_d(double x, double y) { return hypot_borges(x, y); }

// Batched eigen!/eigvals! over a packed arena: matrix b is n[b] x n[b]
// column-major (lda = n[b]) at A + a_off[b]; values at w + w_off[b]; vectors
// at V + a_off[b]. One matrix per OpenMP thread (dynamic schedule).
int gla_oracle_syev_batched_d(char jobz, char uplo, int64_t batch, const int64_t* n, const int64_t* a_off, double* A,
                              double* w, const int64_t* w_off, double* V, int* info, double tol, int nthreads) {
  if (tol <= 0) tol = num<double>::eps();
  if (nthreads > 0) omp_set_num_threads(nthreads);
  int bad = 0;
#pragma omp parallel for schedule(dynamic, 1) reduction(+ : bad)
  for (int64_t b = 0; b < batch; b++) {
    Opts<double> o = make_opts<double>(tol, 0, -1);
    int inf = syev(o, jobz, uplo, n[b], A + a_off[b], n[b], w + w_off[b], V ? V + a_off[b] : nullptr, n[b], false);
    info[b] = inf;
    bad += inf != 0;
  }
  return bad;
}

int gla_oracle_syev_batched_s(char jobz, char uplo, int64_t batch, const int64_t* n, const int64_t* a_off, float* A,
                              float* w, const int64_t* w_off, float* V, int* info, float tol, int nthreads) {
  if (tol <= 0) tol = num<float>::eps();
  if (nthreads > 0) omp_set_num_threads(nthreads);
  int bad = 0;
#pragma omp parallel for schedule(dynamic, 1) reduction(+ : bad)
  for (int64_t b = 0; b < batch; b++) {
    Opts<float> o = make_opts<float>(tol, 0, -1);
    int inf = syev(o, jobz, uplo, n[b], A + a_off[b], n[b], w + w_off[b], V ? V + a_off[b] : nullptr, n[b], false);
    info[b] = inf;
    bad += inf != 0;
  }
  return bad;
}

int gla_oracle_max_threads(void) { return omp_get_max_threads(); }

// Sturm counts for m shifts (src/tridiag.jl:20-36).
void gla_oracle_numnegevals_d(int64_t n, const double* a, const double* b, int64_t m, const double* sigma,
                              int64_t* counts) {
  for (int64_t i = 0; i < m; i++) counts[i] = numnegevals(a, b, n, sigma[i]);
}

}  // extern "C"
