// Ogita-Aishima eigenpair refinement of FP32 eigenvectors back to FP64
// accuracy (batched, n <= 128). No reference counterpart: it is the second
// half of the FP32 + refinement path.
#pragma once
#include <cuda_runtime.h>
#include <stddef.h>
#include <stdint.h>

#include "gla_small.cuh"

namespace gla {

struct RefineWork {
  double* X = nullptr;  // current eigenvector approximation (a_elems)
  double* Y = nullptr;  // A*X, then X + X*E (a_elems)
  double* S = nullptr;  // X'AX, then E (a_elems)
  double* R = nullptr;  // I - X'X (a_elems)
};

constexpr int kRefineIters = 2;

size_t refine_workspace_bytes(int64_t a_elems, int64_t w_elems, int64_t batch);
void refine_carve(RefineWork* rw, char* base, int64_t a_elems, int64_t w_elems, int64_t batch);
cudaError_t refine_kernels_init();
cudaError_t launch_refine(const RefineWork* rw, int nblocks, int nmax, cudaStream_t st, const SmallDesc* descs,
                          const int* perm, const double* A, int lower, const float* X32, const float* w32,
                          double* V, double* w, const int* info, unsigned long long* stats);

}  // namespace gla
