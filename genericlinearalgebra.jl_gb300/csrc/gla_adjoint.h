// Adjoint of the batched symmetric eigen-decomposition (see adjoint.cu).
#pragma once
#include <cuda_runtime.h>
#include <stddef.h>
#include <stdint.h>

#include "df64.cuh"
#include "gla_small.cuh"

namespace gla {

size_t adjoint_workspace_bytes(int64_t a_elems);
cudaError_t adjoint_kernels_init();
cudaError_t launch_adjoint(int nblocks, cudaStream_t st, const SmallDesc* descs, const int* perm, const double* w,
                           const double* V, const double* wbar, const double* Vbar, double* Abar, df64* ws,
                           int64_t a_elems, double gap_rel);

}  // namespace gla
