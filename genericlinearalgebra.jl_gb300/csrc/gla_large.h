// Internal interface of the large-matrix (n > 128) path: blocked
// tridiagonalisation, divide-and-conquer tridiagonal eigensolver,
// back-transformation and the drivers that chain them.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "gemm_simt.cuh"

struct gla_plan_s;

namespace gla {

constexpr int kLargeMaxN = 16384;
constexpr int kSytrdNB = 32;    // panel width of the tridiagonalisation
constexpr int kBacktrNB = 64;   // reflectors per compact-WY block of the back-transformation

// ---- GEMM launchers (gemm_simt.cuh). With splits > 1, g.ksplit and
// g.split_stride describe the split-K partial outputs written to g.C.
cudaError_t gemm_launch(bool f64, bool ta, bool tb, bool lower, const GemmDesc& g, int splits, cudaStream_t st);
// Problems whose sizes are only known on the device: one launch over
// nprob descriptors, grid sized for max_m x max_n outputs (A, B not transposed).
cudaError_t gemm_launch_grouped(bool f64, const GemmDesc* d_descs, int nprob, int max_m, int max_n, cudaStream_t st);

// ---- double-float GEMM (dfgemm.cu): C = op(A) B with A = Ahi + Alo and
// B = Bhi + Blo (Alo / Blo may be null), column-major; lower: write only the
// lower triangle of C.
struct DfGemmDesc {
  int m, n, k;
  int lower;
  const float* Ahi;
  const float* Alo;
  long long lda;
  const float* Bhi;
  const float* Blo;
  long long ldb;
  float* Chi;
  float* Clo;
  long long ldc;
};
cudaError_t dfgemm_launch(const DfGemmDesc& g, bool ta, cudaStream_t st);

// ---- tcgen05 Ozaki GEMM (ozaki.cuh / ozaki.cu): C = A B to double-float
// accuracy on the bf16 tensor cores. Operands are sliced first: the A operand
// from the columns of a float-pair matrix (its rows after transposition, or
// the rows of a symmetric matrix), the B operand from its columns; S = 7
// slices of 7 bits each (oz_create; the slice count must match the work
// object's), relative to the largest entry of the row or column:
// double-float accuracy whatever the spread of the entries. oz_create with
// m = 0 or n = 0 allocates only the other operand.
struct OzWork;
int oz_create(OzWork** out, int m, int n, int K);
// FP32-accuracy configuration: S = 4 slices (28 bits relative to the row and
// column maxima, pairs up to 2^-35), 128 x 128 tiles, C written in FP32 to
// Chi (Clo unused).
int oz_create_f32(OzWork** out, int m, int n, int K);
void oz_destroy(OzWork* w);
cudaError_t oz_slice(OzWork* w, bool a_operand, const float* hi, const float* lo, long long ld, int count, int len,
                     int S, cudaStream_t st);
cudaError_t oz_gemm(OzWork* w, int M, int N, int K, float* Chi, float* Clo, long long ldc, bool lower,
                    cudaStream_t st);
// A operand from wa, B operand from wb (error word of wa).
cudaError_t oz_gemm2(OzWork* wa, OzWork* wb, int M, int N, int K, float* Chi, float* Clo, long long ldc, bool lower,
                     cudaStream_t st);
int* oz_error_word(OzWork* w);
// A operand from the rows of a column-major matrix (element (r, k) at r + k ld).
cudaError_t oz_slice_rows(OzWork* w, const float* hi, const float* lo, long long ld, int rows, int len, int S,
                          cudaStream_t st);
bool oz_fits(const OzWork* w, int m, int n, int K);

// ---- adjoint of one large eigen-decomposition (large_adjoint.cu):
// Abar = V (diag(wbar) + sym(F o (V' Vbar))) V' for orders up to nmax of
// the context (its tensor-core slice buffers and float-pair planes,
// ~70 n^2 bytes).
struct LargeAdjoint;
int large_adjoint_create(LargeAdjoint** out, int nmax);
void large_adjoint_destroy(LargeAdjoint* a);
cudaError_t large_adjoint(LargeAdjoint* a, int n, const double* w, const double* V, long long ldv,
                          const double* wbar, const double* Vbar, long long ldvb, double* Abar, long long lda,
                          double gap_rel, cudaStream_t st);

// ---- stage plans (one order, one working precision)
struct SytrdPlan;
// tc (FP32 only): trailing updates on the tensor cores (3xTF32, tc_gemm.cuh).
cudaError_t sytrd_plan_create(SytrdPlan** out, int n, bool f64, bool tc = false);
void sytrd_plan_destroy(SytrdPlan* p);
cudaError_t sytrd_enqueue(SytrdPlan* p, void* A, long long lda, void* d, void* e, void* tau, cudaStream_t st);
int* sytrd_error_word(SytrdPlan* p);

struct DcPlan;
// bisect_leaves (FP32 only): the leaves go through the per-eigenvalue solver
// (GLA_FLAG_F32_BISECT) instead of the QL chase; for the FP32 stage of the
// FP32 + refinement path, whose refinement absorbs its ~1e-4 orthogonality.
int dc_plan_create(DcPlan** out, int n, bool f64, bool bisect_leaves = false);
void dc_plan_destroy(DcPlan* p);
// Z has leading dimension n; info gets one word per leaf.
int dc_enqueue(DcPlan* p, void* d, const void* e, void* Z, int* leaf_info, cudaStream_t st);
int* dc_fail_word(DcPlan* p);
int dc_leaf_count(const DcPlan* p);
size_t dc_plan_bytes(const DcPlan* p);

struct BacktrPlan;
// tc (FP32 only): both GEMMs of every block on the tensor cores (3xTF32).
int backtr_plan_create(BacktrPlan** out, int n, bool f64, bool tc = false);
void backtr_plan_destroy(BacktrPlan* p);
// Error word the back-transformation's tensor-core GEMMs set when a bounded
// wait runs out (the large context passes its reduction's word).
void backtr_set_error_word(BacktrPlan* p, int* err);
// Z := Q Z, or Q' Z when trans, for Z of ncol columns (-1: n).
int backtr_enqueue(BacktrPlan* p, const void* A, long long lda, const void* tau, void* Z, long long ldz,
                   cudaStream_t st, int ncol = -1, bool trans = false);

// ---- large-path context: workspace for one order n and one working precision
struct LargeCtx;
// refine_stage (FP32 only): the context solves the FP32 stage of the FP32 +
// refinement path, whose refinement absorbs errors of ~1e-4: its
// divide-and-conquer leaves go through the per-eigenvalue solver and its
// trailing updates and back-transformation through the 3xTF32 tensor-core
// GEMM. Plain FP32 solves keep the QL leaves and the FP32 SIMT GEMMs.
int large_create(LargeCtx** out, int n, bool f64, bool refine_stage = false);
void large_destroy(LargeCtx* c);
size_t large_workspace_bytes(const LargeCtx* c);
// Stage times of the last large_syev (ms): tridiagonalisation (with the
// load), divide and conquer, back-transformation (with the store).
void large_stage_ms(const LargeCtx* c, float* ms3);

// Householder tridiagonalisation of the lower triangle of A (n x n, leading
// dimension lda, working precision), in place: d, e, tau and the reflectors
// below the subdiagonal (symtri! layout, unit element implicit).
int large_sytrd(LargeCtx* c, void* A, long long lda, void* d, void* e, void* tau, cudaStream_t st);
// The context's n x n working matrix (leading dimension n).
void* large_work_matrix(LargeCtx* c);
// Eigenpairs of the symmetric tridiagonal (d, e): d becomes the ascending
// eigenvalues, Z (ldz) the eigenvectors. info: 0, or > 0 if a subproblem
// did not converge.
int large_stedc(LargeCtx* c, void* d, const void* e, void* Z, long long ldz, int* info, cudaStream_t st);
// Z := Q Z with Q = H_0 H_1 ... H_{n-2} from large_sytrd.
int large_ormtr(LargeCtx* c, const void* A, long long lda, const void* tau, void* Z, long long ldz, cudaStream_t st,
                int ncol = -1, bool trans = false);
// Full eigen-decomposition of one matrix. tcode: kF64, kF32 or kF32FromF64
// (double input solved in FP32; outputs float). Ain has leading dimension
// lda and uplo 'L'/'U'; w gets the ascending eigenvalues, V (ldv) the
// eigenvectors when wantv. *info_host: 0, -1 (non-finite input), > 0
// unconverged. Synchronises st before returning.
int large_syev(LargeCtx* c, int tcode, bool wantv, bool lower, const void* Ain, long long lda, void* w, void* V,
               long long ldv, int* info_host, cudaStream_t st);

// SymTridiagonal (d, e) of the context's order (FP64 context): ascending
// eigenvalues into w, eigenvectors into Z (ldz, may be null). *info_host: 0,
// -1 (non-finite input), > 0 unconverged. Synchronises st.
int large_stev(LargeCtx* c, const double* d, const double* e, double* w, double* Z, long long ldz, int* info_host,
               cudaStream_t st);

// ---- refinement of FP32 eigenpairs of one large matrix (large_refine.cu)
struct RefineLarge;
int refine_large_create(RefineLarge** out, int n);
void refine_large_destroy(RefineLarge* r);
// Buffers the FP32 solve can write straight into: eigenvectors (n x n,
// leading dimension n) and eigenvalues (n).
float* refine_large_xbuf(RefineLarge* r);
float* refine_large_wbuf(RefineLarge* r);
// A: FP64 input (uplo triangle, leading dimension lda); X32/w32: FP32
// eigenpairs (ascending); outputs w (FP64, ascending) and V (ldv, may be
// null). Synchronises st. Returns 0, -1 for non-finite input, or a status.
int refine_large_run(RefineLarge* r, const double* A, long long lda, bool lower, const float* X32, long long ldx,
                     const float* w32, double* w, double* V, long long ldv, cudaStream_t st);
int refine_large_iters(const RefineLarge* r);
int refine_large_rotations(const RefineLarge* r);  // cluster Rayleigh-Ritz steps of the last run

// ---- leaf solves of the divide and conquer: a batched small-matrix plan
// over the leaf orders, fed with tridiagonal (d, e) in its arena layout.
int plan_stev_batched(gla_plan_s* p, int tcode, const void* din, const void* ein, void* Q, void* w, int* info,
                      cudaStream_t st);

}  // namespace gla
