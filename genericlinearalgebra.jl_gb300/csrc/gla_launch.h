// Host-side launchers of the small-matrix kernels (one per kernel family;
// each returns the launch error). Element type codes: kF64 = double,
// kF32 = float, kF32FromF64 = float work type loading double input.
#pragma once
#include <cuda_runtime.h>
#include <stddef.h>

#include "gla_small.cuh"

namespace gla {

enum TypeCode { kF64 = 0, kF32 = 1, kF32FromF64 = 2 };

// Limits shared by every driver of the small-matrix kernels (plans, the
// single-matrix entry points and the allocation-free one), so that they stop
// on the same conditions.
constexpr int kMaxSweepsPerN = 30;  // chase cap per matrix: 30 n sweeps (src/eigenGeneral.jl:52 uses 30n)
constexpr int kMaxPasses = 64;      // chase passes before a full rotation log is given up on
constexpr double kTolF64 = 0x1p-52;  // default deflation tolerance, eps(Float64)
constexpr double kTolF32 = (double)0x1p-23f;  // eps(Float32)

size_t tridiag_smem_bytes(int n, int nt, int elem, bool stein = false);
size_t chase_smem_bytes(int nmax, int elem);
size_t apply_smem_bytes(int n, int elem);

// Raise the dynamic shared-memory limit of every kernel instantiation once.
cudaError_t small_kernels_init();

// stein (FP32 work type with Q only): the CTA also solves the tridiagonal
// (bisection + twisted factorisation) and writes X = Q Y and the eigenvalues
// (to w) for every matrix it does not leave to the QL chase; qtmp: a float
// scratch arena of the plan's a_elems entries. rows2 (wantq false): rows 1
// and n of Q instead (2 x n column-major per matrix, at twice its w offset),
// for eigen2.
cudaError_t launch_tridiag(int tcode, bool wantq, int nblocks, int nt, size_t smem, cudaStream_t st,
                           const SmallDesc* descs, const int* perm, const void* A, int lower, void* d, void* e,
                           void* Q, int* info, ChaseState* cst, int* scale_exp, bool stein = false,
                           void* w = nullptr, void* qtmp = nullptr, void* rows2 = nullptr);

cudaError_t launch_chase(int tcode, int algo, int count, size_t smem, cudaStream_t st, const SmallDesc* descs,
                         const int* perm, void* d, void* e, ChaseState* cst, void* rot, unsigned* hdr, int* info,
                         double tol, int max_sweeps_per_n, int* pending, unsigned long long* stats,
                         int lanes_per_warp = 0);

// rows2: V holds rows 1 and n only (eigen2; 2 x n at twice the w offset).
cudaError_t launch_apply(int tcode, int nblocks, int nt, size_t smem, cudaStream_t st, const SmallDesc* descs,
                         const int* perm, void* V, const void* d, void* w, ChaseState* cst, const void* rot,
                         const unsigned* hdr, const int* info, const int* scale_exp, bool rows2 = false);

cudaError_t launch_sort_values(int tcode, int nblocks, cudaStream_t st, const SmallDesc* descs, const int* perm,
                               const void* d, void* w, const int* info, const int* scale_exp);

// SymTridiagonal input on the FP32 stage: the per-eigenvalue solver
// (small_stein.cuh) for every matrix still running (after
// launch_init_tridiagonal); solved ones are marked done and applied.
cudaError_t launch_stein_tri(int nblocks, int nmax, cudaStream_t st, const SmallDesc* descs, const int* perm,
                             const void* d, const void* e, void* Q, void* w, ChaseState* cst, const int* info);

// Capture-safe executes: info = -2 for matrices whose chase is still running.
cudaError_t launch_mark_unfinished(int nblocks, cudaStream_t st, const SmallDesc* descs, const int* perm,
                                   const ChaseState* cst, int* info);

// SymTridiagonal input: copy (d, e) into the working arrays, Q := I, reset state.
cudaError_t launch_init_tridiagonal(int tcode, int nblocks, cudaStream_t st, const SmallDesc* descs,
                                    const int* perm, const void* din, const void* ein, void* d, void* e, void* Q,
                                    int* info, ChaseState* cst, bool wantq);

}  // namespace gla
