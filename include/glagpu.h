/*
 * glagpu.h — C ABI of the GB300 (sm_103a) self-adjoint eigensolver.
 *
 * Drop-in for the eigen/eigvals path of GenericLinearAlgebra.jl v0.4.0
 * (src/eigenSelfAdjoint.jl). Each entry point names the reference
 * interface it replaces. Conventions follow the reference's own native
 * boundary (src/lapack.jl:40-62, ccall into LAPACK): plain C types,
 * column-major storage, character flags, an integer status, no exceptions
 * across the ABI.
 *
 *   status   0  success
 *           <0  argument -status is invalid (LAPACK xerbla convention)
 *         -1000 - e  CUDA runtime error e (see gla_status_string)
 *         -2001 order above GLA_STATIC_MAX_N (gla_dsyev_static only)
 *         -2002 operation not supported for this plan
 *           >0  number of matrices whose per-matrix info is nonzero
 *   info[b]  0  converged
 *           >0  number of off-diagonal entries still above the deflation
 *               threshold after the sweep cap (30*n chases per matrix;
 *               the reference has no cap and never returns on such input)
 *          n+1  (GLA_PREC_F32_REFINED) the refinement did not reach its
 *               accuracy target within its iteration cap (outputs are the
 *               last iterate)
 *           -1  the referenced triangle held NaN or Inf (outputs are NaN)
 *           -2  (GLA_FLAG_GRAPH plans only) the chase needed more passes than
 *               the captured sequence holds (outputs are not valid)
 *
 * Buffers are caller-owned; the library owns only plans and their
 * workspace. All pointers passed to *_execute are device pointers unless
 * the function name ends in _host. Calls are asynchronous on `stream`
 * (a cudaStream_t, NULL = legacy default stream) except where stated.
 */
#ifndef GLAGPU_H
#define GLAGPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define GLA_VERSION 100

/* Arithmetic of a plan. */
#define GLA_PREC_F64 0         /* plain FP64 end to end */
#define GLA_PREC_F32 1         /* plain FP32 end to end (float in/out) */
#define GLA_PREC_F32_REFINED 2 /* FP32 solve + Ogita-Aishima refinement, FP64 in/out */

/* Chase algorithm (flags bits 0-1). */
#define GLA_ALG_QL 0 /* eigQL!  (src/eigenSelfAdjoint.jl:221-288), the default */
#define GLA_ALG_QR 1 /* eigQR!  (src/eigenSelfAdjoint.jl:290-340) */

/* Flag bit: shrink the per-pass rotation log to ~n^2/8 so that the chase
 * runs in several passes (exercises the resume path; results are identical). */
#define GLA_FLAG_SMALL_LOG 4
/* Flag bit: record CUDA events around each phase of every execute (see
 * gla_plan_phase_times). */
#define GLA_FLAG_TIMING 8
/* Flag bit: capture-safe execute for CUDA graphs. gla_plan_execute then never
 * synchronizes the host: it enqueues a fixed four chase passes (8 n^2
 * rotations, twice what random spectra need) and a matrix that would need more
 * is reported with info = -2 instead of being finished by extra passes. */
#define GLA_FLAG_GRAPH 16
/* Flag bit: choose each size bucket's launch shapes (threads per CTA of the
 * tridiagonalisation, 1-4 per row; matrices per warp of the chase, 4-32) from the process-wide
 * autotune table; shapes missing from it are measured during plan creation
 * on synthetic matrices of the bucket's order and count (synchronizes the
 * device; a few seconds for a fresh table) and added. See gla_autotune_*. */
#define GLA_FLAG_AUTOTUNE 32
/* Flag bit (GLA_PREC_F32_REFINED, orders <= 128): run the FP32 stage with the
 * reference's QL chase (as GLA_PREC_F32 does) instead of the default
 * per-eigenvalue solver (bisection on Sturm counts plus one twisted
 * factorisation per eigenvector, inside the tridiagonalisation kernel, with
 * the QL chase only for matrices whose eigenvalues come within 1e-6 ||T||
 * of each other). Both feed the same refinement. */
#define GLA_FLAG_REFINE_QL 64
/* Flag bit (GLA_PREC_F32, orders <= 128): solve with that per-eigenvalue
 * solver instead of the QL chase (matrices with eigenvalues within
 * 1e-6 ||T|| of each other still take the chase). Eigenvalues as accurate
 * as the chase's; eigenvectors orthogonal to about 1e-4 (eps(Float32)
 * ||T|| over the smallest gap outside its Gram-Schmidt clusters) instead of
 * n eps(Float32). The FP32 + refinement path uses it for its internal FP32
 * solves (cluster matrices, divide-and-conquer leaves). */
#define GLA_FLAG_F32_BISECT 128
/* Flag bit (GLA_PREC_F32_REFINED, orders <= 128): evaluate the refinement's
 * double-float products (A X, X'(A X), X'X) on the FP32 pipe in double-float
 * arithmetic instead of the default tcgen05 tensor-core Ozaki products (seven
 * bf16 slices per operand, exact integer accumulation). Both are ~2^-47
 * relative; results agree within the refinement's 1e-13 bounds. */
#define GLA_FLAG_REFINE_SIMT 256

/* Phases reported by gla_plan_phase_times. */
#define GLA_PHASE_TRIDIAG 0 /* symtri! + Array(Q)          */
#define GLA_PHASE_CHASE 1   /* eigQL!/eigQR!/eigvalsPWK! scalar chase */
#define GLA_PHASE_APPLY 2   /* rotations on Q + sorteig!   */
#define GLA_PHASE_REFINE 3  /* Ogita-Aishima refinement    */
#define GLA_NUM_PHASES 4

#define GLA_MAX_SMALL_N 128   /* largest order of the batched one-CTA-per-matrix path */
#define GLA_MAX_N 16384       /* largest order accepted by plans (orders above
                                 GLA_MAX_SMALL_N run the blocked large-matrix path) */
#define GLA_STATIC_MAX_N 128
#define GLA_ERR_STATIC_TOO_LARGE (-2001)
#define GLA_ERR_UNSUPPORTED (-2002) /* operation not available for this plan */

typedef struct gla_plan_s* gla_plan_t;

int gla_version(void);
const char* gla_status_string(int status);

/*
 * Batched plan over `batch` independent real symmetric matrices of orders
 * n[0..batch) (host array, 0 <= n[b] <= GLA_MAX_N).
 *
 * Orders up to GLA_MAX_SMALL_N are solved together (one CTA per matrix,
 * size-bucketed). Larger orders are solved one at a time with the whole GPU:
 * blocked Householder tridiagonalisation, divide and conquer on the
 * tridiagonal, compact-WY back-transformation; such plans synchronise the
 * stream inside execute and do not support GLA_FLAG_GRAPH or
 * GLA_PREC_F32_REFINED (those return -8 / -2).
 *
 * Packed arena layout used by the execute calls: matrix b is n[b] x n[b],
 * column-major with leading dimension n[b], at element offset
 * a_off(b) = sum_{c<b} n[c]^2; its eigenvalues at w_off(b) = sum_{c<b} n[c].
 *
 * jobz 'V' -> eigen!(Hermitian(A, uplo))  (src/eigenSelfAdjoint.jl:614-630:
 *             symtri!, Array(Q), eigQL!, sorteig!)
 * jobz 'N' -> eigvals!(Hermitian(A, uplo)) (:572-588: symtri!, eigvalsPWK!,
 *             sorteig!)
 * tol <= 0 selects eps of the working precision, the reference default
 * (tol = eps(real(eltype(A)))). Allocates the plan's device workspace
 * (synchronous).
 */
int gla_plan_create(gla_plan_t* plan, int precision, char jobz, char uplo, int64_t batch, const int64_t* n,
                    double tol, int flags);
int gla_plan_destroy(gla_plan_t plan);
/* Device workspace held by the plan, in bytes. */
int gla_plan_workspace_size(gla_plan_t plan, size_t* bytes);
/* Total arena sizes (elements) of A/V and of w for this plan. */
int gla_plan_arena_sizes(gla_plan_t plan, int64_t* a_elems, int64_t* w_elems);

/*
 * Run the plan. A: packed input arena (double for F64 and F32_REFINED,
 * float for F32), only the uplo triangle of each matrix is read and A is
 * not modified. w: packed eigenvalues, ascending per matrix. V: packed
 * eigenvectors (columns in eigenvalue order; unused for jobz 'N'; may be
 * the same buffer as A). info: one int per matrix (device). Asynchronous.
 */
int gla_plan_execute(gla_plan_t plan, const void* A, void* w, void* V, int* info, void* stream);

/*
 * eigen2 (src/eigenSelfAdjoint.jl:633-644): the ascending eigenvalues and
 * only rows 1 and n of the eigenvector matrix, the reference's cheap form:
 * rows 1 and n of Q are formed from the reflectors (rmul!(V, Q) on a 2 x n V,
 * :62-80) instead of Q itself, and the QL (or QR) rotations are replayed on
 * those two rows only. V2: per matrix a 2 x n column-major block at twice
 * its eigenvalue offset (2 sum_{c<b} n_c). Plans with jobz 'V' and
 * precision GLA_PREC_F64 or GLA_PREC_F32 whose orders are all <= 128;
 * others return GLA_ERR_UNSUPPORTED. Synchronization as gla_plan_execute.
 */
int gla_plan_execute_eigen2(gla_plan_t plan, const void* A, void* w, void* V2, int* info, void* stream);
/* Same from and to HOST buffers (V2: 2 w_elems entries); synchronizes the
 * stream and returns the number of matrices with nonzero info. */
int gla_plan_execute_eigen2_host(gla_plan_t plan, const void* A_host, void* w_host, void* V2_host, int* info_host,
                                 void* stream);

/*
 * Same, from and to HOST buffers: copies A in, runs, copies w, V and info
 * out, and synchronizes `stream` before returning. Uses plan-owned device
 * buffers (allocated on first use). Pinned host memory is fastest: for a
 * GLA_PREC_F32_REFINED plan of orders <= GLA_MAX_SMALL_N (none larger)
 * holding at least two matrices per CTA of its persistent launch (two CTAs
 * per SM), without GLA_FLAG_GRAPH or GLA_FLAG_TIMING, and with A, w and V
 * (jobz 'V') in page-locked memory, the batch is solved in two to four
 * contiguous chunks and the copies of one chunk overlap the solve of
 * another (same results, bit for bit).
 */
int gla_plan_execute_host(gla_plan_t plan, const void* A_host, void* w_host, void* V_host, int* info_host,
                          void* stream);
/* The number of chunks gla_plan_execute_host pipelines this plan over (0:
 * never), and whether its last call did (1) or copied all of A in before
 * the solve and all of w and V out after it (0). */
int gla_plan_host_pipeline(gla_plan_t plan, int* chunks, int* last_pipelined);

/*
 * Adjoint of the plan's eigen-decomposition (reverse mode; the kernel behind
 * an rrule / autograd rule for eigen, no counterpart in the reference).
 * Inputs, packed like the execute outputs (FP64, device): w and V, the
 * eigenpairs; wbar and Vbar, the cotangents of the loss with respect to them.
 * Output Abar (packed like A, full symmetric matrices):
 *     Abar = V (diag(wbar) + sym(F o (V' Vbar))) V',  sym(X) = (X + X')/2,
 *     F_ij = 1/(w_j - w_i) when |w_j - w_i| > gap_rel * max|w|, else 0.
 * gap_rel <= 0 selects 1e-10. The three products (V'Vbar, V S, (V S) V')
 * run to double-float accuracy (~2^-47 relative to the row and column
 * maxima) on the tensor cores: one CTA per matrix for orders <=
 * GLA_MAX_SMALL_N, three tensor-core GEMMs per matrix above. The first call
 * allocates the adjoint workspace (32 bytes per arena element, plus about
 * 70 n^2 bytes for the largest order above GLA_MAX_SMALL_N); later calls
 * allocate nothing. A bounded tensor-core wait that ran out leaves the
 * matrix's Abar NaN. Asynchronous on `stream`.
 */
int gla_plan_adjoint(gla_plan_t plan, const double* w, const double* V, const double* wbar, const double* Vbar,
                     double* Abar, double gap_rel, void* stream);
/* Same, from and to HOST buffers (the library stages them on the device;
 * synchronizes `stream`). For host-language glue without device arrays. */
int gla_plan_adjoint_host(gla_plan_t plan, const double* w, const double* V, const double* wbar, const double* Vbar,
                          double* Abar, double gap_rel, void* stream);

/*
 * Statistics of the last execute: total Givens rotations applied to the
 * eigenvectors, implicit-shift chases and chase passes. Synchronizes the
 * plan's last stream.
 */
int gla_plan_stats(gla_plan_t plan, int64_t* rotations, int64_t* sweeps, int* passes);

/*
 * Work counters of the last execute (synchronizes the plan's last stream):
 * the algorithmic-work figures a roofline needs.
 */
#define GLA_COUNTER_ROTATIONS 0     /* Givens rotations applied to eigenvectors */
#define GLA_COUNTER_SWEEPS 1        /* implicit-shift chases */
#define GLA_COUNTER_ROW_ROTATIONS 2 /* sum over matrices of n * rotations (rows rotated) */
#define GLA_COUNTER_REFINE_N3 3     /* sum over matrices of refinement iterations * n^3 */
#define GLA_COUNTER_PASSES 4        /* chase passes */
#define GLA_NUM_COUNTERS 5
int gla_plan_counters(gla_plan_t plan, int64_t* counters);

/*
 * Milliseconds spent in each phase (GLA_PHASE_*) by the last execute, from
 * CUDA events recorded on the execute's stream (plan created with
 * GLA_FLAG_TIMING; otherwise all zero). Synchronizes that stream.
 */
int gla_plan_phase_times(gla_plan_t plan, float* ms);

/*
 * Single-matrix LAPACK-style driver (device pointers), the in-place form of
 * LinearAlgebra.eigen!(Hermitian(A, uplo)) (src/eigenSelfAdjoint.jl:626):
 * on return A holds the eigenvectors (jobz 'V') and w the ascending
 * eigenvalues. lda >= n. *info is written on the host (synchronizes).
 */
int gla_dsyev(char jobz, char uplo, int64_t n, double* A, int64_t lda, double* w, int* info, void* stream);
int gla_ssyev(char jobz, char uplo, int64_t n, float* A, int64_t lda, float* w, int* info, void* stream);

/*
 * FP32 GEMM on the tcgen05 tensor cores in split TF32 (3xTF32), the product
 * the FP32 large-matrix path uses for its rank-2k trailing updates and its
 * eigenvector back-transformation: C = alpha A B + beta C with A (m x k)
 * given transposed, At (k x m, column-major, element (i, l) of A at
 * At[l + i ldat]), B (k x n, column-major) and C (m x n, column-major).
 * Operands are loaded by TMA: At and B 16-byte aligned, ldat and ldb
 * multiples of 4 (else the argument's index is returned). Error about
 * 2^-21 relative to sum |a||b| per entry. Asynchronous on the stream; a
 * bounded wait that ran out inside the kernel is reported by the next call
 * (status -1000 - cudaErrorLaunchTimeout). No counterpart in the reference.
 */
int gla_sgemm_3xtf32(int64_t m, int64_t n, int64_t k, float alpha, const float* At, int64_t ldat, const float* B,
                     int64_t ldb, float beta, float* C, int64_t ldc, void* stream);

/*
 * Frees the device workspaces that the single-call entry points keep for the
 * life of the process, one per distinct order or size: gla_dsyev, gla_ssyev,
 * gla_dstev, gla_gemm_df, gla_zheev, gla_qheev, gla_dsytrd and gla_dormtr.
 * Plans are the caller's and are not touched. Waits for the whole device
 * first (cudaDeviceSynchronize), since queued work may still use the
 * buffers; the next call of an entry point allocates its workspace again.
 * Call it when no other host thread is inside one of those entry points.
 * No counterpart in the reference (Julia's garbage collector owns its
 * workspaces).
 */
int gla_release_workspaces(void);

/*
 * gla_dsyev without any device allocation: same arguments, results and
 * synchronisation as gla_dsyev, for callers that cannot call cudaMalloc when
 * they need the decomposition (e.g. an application whose memory pool already
 * owns the whole device, a latency-critical loop where an allocation would
 * synchronise the device, a fixed memory budget). No counterpart in the
 * reference.
 *
 * Limit: n <= GLA_STATIC_MAX_N (128); larger orders return
 * GLA_ERR_STATIC_TOO_LARGE. Scratch comes from one file-scope device array of
 * about 660 KB that every GPU loading the library holds until exit. The
 * first call on a device looks up that array's device address (and sets the
 * kernels' shared-memory limits), so make it before any stream capture.
 * Like gla_dsyev, every call reads info back to the host and waits for its
 * stream before returning. All calls share the array: calls whose GPU work
 * overlaps (other streams, other host threads on the same device) race and
 * must be serialised.
 */
int gla_dsyev_static(char jobz, char uplo, int64_t n, double* A, int64_t lda, double* w, int* info, void* stream);

/*
 * Double-float-accurate GEMM on the tcgen05 tensor cores (the product the
 * FP32 + refinement path runs on): C = A B with A (m x k) and B (k x n) as
 * float pairs A = Ahi + Alo, B = Bhi + Blo (column-major device arrays with
 * leading dimensions lda, ldb; Alo / Blo may be NULL), returned as
 * C = Chi + Clo (ldc). Ozaki scheme: every row of A and column of B is split
 * into seven 7-bit integer slices relative to its largest entry (exact in
 * bf16); the 28 slice products with s + t <= 8 are accumulated exactly in
 * TMEM and summed in double-float, ~2^-47 of sum |a_ik||b_kj|. Slice
 * buffers (~28 (m + n) k bytes) are allocated by the first call of a given
 * size and kept for later calls. Asynchronous on `stream`; returns -1000 -
 * cudaErrorLaunchTimeout at the next call if a bounded wait ran out.
 */
int gla_gemm_df(int64_t m, int64_t n, int64_t k, const float* Ahi, const float* Alo, int64_t lda, const float* Bhi,
                const float* Blo, int64_t ldb, float* Chi, float* Clo, int64_t ldc, void* stream);
/* Stream-event durations of the most recent gla_gemm_df call (synchronizes
 * with its end): the operand slicing and the tensor-core GEMM kernel. */
int gla_gemm_df_last_ms(float* slice_ms, float* gemm_ms);

/*
 * eigen!/eigvals! of SymTridiagonal(d, e) (src/eigenSelfAdjoint.jl:581,
 * :602-612, :623): d (n), e (n-1) device arrays; on return d holds the
 * ascending eigenvalues (e may be overwritten) and Z (n x n, ldz) the
 * eigenvectors (jobz 'V'). Orders up to GLA_MAX_SMALL_N run the QL (default)
 * or QR chase selected by flags; larger orders (up to GLA_MAX_N) the divide
 * and conquer of the large-matrix path (flags ignored). Synchronizes.
 */
int gla_dstev(char jobz, int64_t n, double* d, double* e, double* Z, int64_t ldz, int flags, int* info,
              void* stream);

/*
 * Complex Hermitian eigenproblem (the reference's eigen!/eigvals! on
 * Hermitian{<:Complex}): A is n x n complex, interleaved (re, im) doubles,
 * column-major with leading dimension lda (in complex elements); only the
 * uplo triangle is read (a diagonal's imaginary part is ignored). w: n
 * ascending eigenvalues; V (jobz 'V'): n x n complex orthonormal eigenvectors,
 * interleaved, leading dimension ldv. Device pointers; synchronizes. Solved
 * through the real symmetric embedding [[B, -C], [C, B]] of order 2n
 * (2n <= GLA_MAX_N). Status and info as for gla_dsyev.
 */
int gla_zheev(char jobz, char uplo, int64_t n, const double* A, int64_t lda, double* w, double* V, int64_t ldv,
              int* info, void* stream);
/* Same, from and to host buffers. */
int gla_zheev_host(char jobz, char uplo, int64_t n, const double* A, int64_t lda, double* w, double* V, int64_t ldv,
                   int* info);

/*
 * Quaternion Hermitian eigenproblem (the reference's eigen!/eigvals! on
 * Hermitian{Quaternion{Float64}}, test/eigenselfadjoint.jl:54-84): A is
 * n x n quaternions of 4 doubles (s, i, j, k; the field order of
 * Quaternion{Float64}), column-major with leading dimension lda (in
 * quaternions); only the uplo triangle is read (a diagonal's i, j, k parts
 * are ignored). w: n ascending eigenvalues (real); V (jobz 'V'): n x n
 * orthonormal right eigenvectors (A v = v lambda), same layout, leading
 * dimension ldv. Device pointers; synchronizes. Solved through the real
 * symmetric matrix of left multiplication, of order 4n (4n <= GLA_MAX_N).
 * Status and info as for gla_dsyev.
 */
int gla_qheev(char jobz, char uplo, int64_t n, const double* A, int64_t lda, double* w, double* V, int64_t ldv,
              int* info, void* stream);
/* Same, from and to host buffers. */
int gla_qheev_host(char jobz, char uplo, int64_t n, const double* A, int64_t lda, double* w, double* V, int64_t ldv,
                   int* info);

/*
 * The Householder factorisation on its own (the reference's symtri! /
 * SymmetricTridiagonalFactorization and lmul!/rmul! with its EigenQ,
 * src/eigenSelfAdjoint.jl:6-118, 446-564; FP64, device pointers,
 * asynchronous):
 *   gla_dsytrd: A = Q T Q' from the uplo triangle, returned in that
 *     triangle in the reference's layout. uplo 'L' (symtriLower!): d on the
 *     diagonal, e (the betas) on the first subdiagonal, reflector k in
 *     A[k+2:n, k] below its implicit unit at row k+1. uplo 'U'
 *     (symtriUpper!): e on the first superdiagonal, reflector k in
 *     A[1:n-k-1, n-k+1] above its implicit unit at row n-k. d, e, tau (n-1)
 *     are also returned. The other triangle is not touched.
 *   gla_dormtr: C := op(Q) C (side 'L', C is nq x n with nq = m) or
 *     C := C op(Q) (side 'R', C is m x nq with nq = n); trans 'N' or 'T';
 *     A and tau from gla_dsytrd of order nq with the same uplo.
 * Calls for one order share a cached workspace: issue them on one stream,
 * or synchronize between streams.
 */
int gla_dsytrd(char uplo, int64_t n, double* A, int64_t lda, double* d, double* e, double* tau, void* stream);
int gla_dormtr(char side, char uplo, char trans, int64_t m, int64_t n, const double* A, int64_t lda,
               const double* tau, double* C, int64_t ldc, void* stream);
/* Same, from and to host buffers (synchronous). */
int gla_dsytrd_host(char uplo, int64_t n, double* A, int64_t lda, double* d, double* e, double* tau);
int gla_dormtr_host(char side, char uplo, char trans, int64_t m, int64_t n, const double* A, int64_t lda,
                    const double* tau, double* C, int64_t ldc);

/*
 * Spectrum slicing on SymTridiagonal(d, e) (d: n, e: n-1; device pointers;
 * asynchronous on `stream`):
 *   gla_numnegevals: counts[i] = the number of negative eigenvalues of
 *     T - sigma[i] I, the reference's numnegevals (src/tridiag.jl:20-36) with
 *     its exact operation order (bit-identical counts);
 *   gla_dstebz: w[0 .. iu-il] = the eigenvalues il..iu (1-based, ascending)
 *     by Sturm-count multisection, each to max(abstol, 2 eps |lambda|).
 */
int gla_numnegevals(int64_t n, const double* d, const double* e, int64_t m, const double* sigma, int64_t* counts,
                    void* stream);
int gla_dstebz(int64_t n, const double* d, const double* e, int64_t il, int64_t iu, double abstol, double* w,
               void* stream);
/* Same, from and to host buffers (synchronous). */
int gla_numnegevals_host(int64_t n, const double* d, const double* e, int64_t m, const double* sigma,
                         int64_t* counts);
int gla_dstebz_host(int64_t n, const double* d, const double* e, int64_t il, int64_t iu, double abstol, double* w);

/*
 * Autotune table (GLA_FLAG_AUTOTUNE): drop every entry; write the entries to
 * a text file; merge the entries of such a file (returns how many were
 * loaded, <0 when the file cannot be read).
 */
int gla_autotune_clear(void);
int gla_autotune_save(const char* path);
int gla_autotune_load(const char* path);
/* The plan's size buckets (orders <= GLA_MAX_SMALL_N) and the launch shapes
 * each one runs with. */
int gla_plan_buckets(gla_plan_t plan, int* count);
int gla_plan_bucket_config(gla_plan_t plan, int bucket, int* nmax, int* matrices, int* nt_tri, int* lanes_per_warp);

#ifdef __cplusplus
}
#endif

#endif /* GLAGPU_H */
