// Ogita-Aishima eigenpair refinement of FP32 eigenvectors back to FP64
// accuracy (batched, n <= 128). No reference counterpart: it is the second
// half of the FP32 + refinement path.
#pragma once
#include <cuda_runtime.h>
#include <stddef.h>
#include <stdint.h>

#include "gla_small.cuh"

namespace gla {

struct df64;

struct RefineWork {
  df64* A2 = nullptr;  // scaled A as double-float (a_elems)
  df64* X2 = nullptr;  // current eigenvector approximation
  df64* Y2 = nullptr;  // A X, then X + X E
  df64* S2 = nullptr;  // X'AX
  df64* R2 = nullptr;  // I - X'X
  df64* S0 = nullptr;  // first-iteration X0'AX0 (kept for the implicit iterations)
  df64* R0 = nullptr;  // first-iteration I - X0'X0
  float* E = nullptr;  // correction E
  float* J = nullptr;  // Jacobi scratch of cluster rotations (2 * a_elems)
  float* T = nullptr;  // FP32 product X E (a_elems)
  int* err = nullptr;  // tensor-core wait error word (zeroed by each execute)
  unsigned char* pcache = nullptr;  // persistent kernel: per-CTA slice scratch of the products (or null)
};

size_t refine_workspace_bytes(int64_t a_elems, int64_t w_elems, int64_t batch);
// Bytes of one persistent CTA's slice scratch (RefineWork.pcache).
size_t refine_pcache_bytes();
void refine_carve(RefineWork* rw, char* base, int64_t a_elems, int64_t w_elems, int64_t batch);
cudaError_t refine_kernels_init();
// ChaseState.applied of a matrix that k_solve_refine has solved and refined.
constexpr int kRefinedInKernel = 2;

// One CTA per matrix (perm[0..nblocks)); with cst, matrices already refined
// by the persistent kernel are skipped. tc: the double-float products on the
// tensor cores (tc_small.cuh), else on the FP32 pipe.
cudaError_t launch_refine(const RefineWork* rw, int nblocks, int nmax, cudaStream_t st, const SmallDesc* descs,
                          const int* perm, const double* A, int lower, const float* X32, double* V, double* w,
                          int* info, const int* scale_exp, unsigned long long* stats,
                          const ChaseState* cst = nullptr, bool tc = true);

// The persistent FP32 + refinement solve of count matrices (order: largest
// first) on grid CTAs; *next must be zero on entry.
cudaError_t launch_solve_refine(const RefineWork* rw, int count, int nmax, int grid, cudaStream_t st,
                                const SmallDesc* descs, const int* order, int* next, const double* A, int lower,
                                float* d, float* e, float* X32, int* info, ChaseState* cst, int* scale_exp,
                                float* w32, float* qtmp, double* V, double* w, unsigned long long* stats,
                                bool tc = true);

}  // namespace gla
