// Batched Householder tridiagonalisation and explicit Q, one CTA per matrix,
// the whole matrix staged in shared memory (n <= 128).
//
// Replaces, per matrix:
//   symtriLower! (GenericLinearAlgebra.jl src/eigenSelfAdjoint.jl:450-504)
//   with LinearAlgebra.reflector! (called at :466) and BLAS symv (:477),
//   and Array(Q::EigenQ) = lmul!(Q, I) (:101, :23-41).
// uplo 'U' input is mirrored into the lower triangle on load, so both
// triangles run the 'L' reduction (the 'U' variant :507-564 reduces the
// mirrored matrix in reverse order and yields the same eigenpairs).
//
// Work split (FP64 on GB300 costs ~68 cycles per warp instruction no matter
// how many lanes are active, so every FP64 loop is spread over all lanes):
//   norm / dot products: one element per thread + block reduction,
//   SYMV: rows x (1, 2 or 4 column parts),
//   rank-2 update: flat index over the trailing lower triangle,
//   Q formation: dorg2l-style backward accumulation in place of the
//   reflectors (H_k applied only to the already-formed trailing block).
#include <algorithm>

#include "gla_launch.h"
#include "gla_small.cuh"
#include "small_stein.cuh"
#include "small_tridiag.cuh"

namespace gla {

size_t tridiag_smem_bytes(int n, int nt, int elem, bool) {
  // redm[32] u64 | red[32] (8-byte slots) | S[n*ld] | vv,uu,ww,taus [n] | part[8*nt]
  // (the FP32 tridiagonal solver reuses S and part once Q is in global memory)
  const size_t ld = (size_t)((n + 1) | 1);
  return 512 + (size_t)elem * ((size_t)n * ld + 4 * (size_t)n + 8 * (size_t)nt);
}

template <class T, class Tin, bool WANTQ, bool STEIN>
__global__ void __launch_bounds__(256) k_tridiag(const SmallDesc* __restrict__ descs, const int* __restrict__ perm,
                                                 const Tin* __restrict__ A, int lower, T* __restrict__ dout,
                                                 T* __restrict__ eout, T* __restrict__ Qout, int* __restrict__ info,
                                                 ChaseState* __restrict__ cst, int* __restrict__ scale_exp,
                                                 T* __restrict__ wout, T* __restrict__ qtmp,
                                                 T* __restrict__ rows2) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  tridiag_body<T, Tin, WANTQ, STEIN>(perm[blockIdx.x], smem_raw, descs, A, lower, dout, eout, Qout, info, cst,
                                     scale_exp, wout, qtmp, rows2);
}

size_t stein_tri_smem_bytes(int n) { return 512 + 4 * (2 * (size_t)n + stein_extra_words(n)); }

// Tridiagonal input on the FP32 stage (the leaves of the divide and conquer
// of the FP32 + refinement path): the per-eigenvalue solver of
// small_stein.cuh on (d, e) as the chase would take them, one CTA per
// matrix (blockDim >= n). A solved matrix gets its ascending eigenvalues in
// wout and its eigenvectors in Q, and is marked done for the chase and the
// rotation replay; the others keep Q = I and their "running" chase state.
__global__ void __launch_bounds__(128) k_stein_tri(const SmallDesc* __restrict__ descs, const int* __restrict__ perm,
                                                   const float* __restrict__ dg_all, const float* __restrict__ eg_all,
                                                   float* __restrict__ Qout, float* __restrict__ wout,
                                                   ChaseState* __restrict__ cst, const int* __restrict__ info) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int mid = perm[blockIdx.x];
  const SmallDesc dsc = descs[mid];
  const int n = dsc.n, tid = threadIdx.x;
  if (n < 1 || info[mid] != 0 || cst[mid].status != kChaseRunning) return;
  float* fscr = reinterpret_cast<float*>(smem_raw);  // 128 floats
  float* dd = reinterpret_cast<float*>(smem_raw + 512);
  float* ee = dd + n;
  const int ldy = stein_ldy(n);
  float* Ys = ee + n;
  float* e2s = Ys + (size_t)n * ldy;
  float* lams = e2s + n;
  int* misc = reinterpret_cast<int*>(lams + n);
  for (int i = tid; i < n; i += blockDim.x) {
    dd[i] = dg_all[dsc.w_off + i];
    ee[i] = (i + 1 < n) ? eg_all[dsc.w_off + i] : 0.f;
  }
  __syncthreads();
  if (!stein_solve(n, dd, ee, e2s, lams, Ys, ldy, misc, fscr)) return;
  float* Qg = Qout + dsc.a_off;
  for (int j = 0; j < n; j++)
    for (int i = tid; i < n; i += blockDim.x) Qg[(size_t)j * n + i] = Ys[(size_t)i * ldy + j];
  for (int k = tid; k < n; k += blockDim.x) wout[dsc.w_off + k] = lams[k];
  if (tid == 0) {
    ChaseState st;
    st.bs = n;
    st.nsweeps = 0;
    st.nrot = 0;
    st.nhdr = 0;
    st.status = kChaseDone;
    st.applied = 1;
    cst[mid] = st;
  }
}

cudaError_t launch_stein_tri(int nblocks, int nmax, cudaStream_t st, const SmallDesc* descs, const int* perm,
                             const void* d, const void* e, void* Q, void* w, ChaseState* cst, const int* info) {
  if (nblocks <= 0) return cudaSuccess;
  const int nt = std::max(32, (nmax + 31) / 32 * 32);
  k_stein_tri<<<nblocks, nt, stein_tri_smem_bytes(nmax), st>>>(descs, perm, (const float*)d, (const float*)e,
                                                               (float*)Q, (float*)w, cst, info);
  return cudaGetLastError();
}

template <class T, class Tin, bool Q, bool ST = false> static void set_tri_attr() {
  cudaFuncSetAttribute(k_tridiag<T, Tin, Q, ST>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                       (int)tridiag_smem_bytes(kSmallMaxN, 256, sizeof(T), ST));
}

cudaError_t tridiag_kernels_init() {
  set_tri_attr<double, double, true>();
  set_tri_attr<double, double, false>();
  set_tri_attr<float, float, true>();
  set_tri_attr<float, float, false>();
  set_tri_attr<float, double, true>();
  set_tri_attr<float, double, false>();
  set_tri_attr<float, double, true, true>();
  set_tri_attr<float, float, true, true>();
  cudaFuncSetAttribute(k_stein_tri, cudaFuncAttributeMaxDynamicSharedMemorySize,
                       (int)stein_tri_smem_bytes(kSmallMaxN));
  return cudaGetLastError();
}

cudaError_t launch_tridiag(int tcode, bool wantq, int nblocks, int nt, size_t smem, cudaStream_t st,
                           const SmallDesc* descs, const int* perm, const void* A, int lower, void* d, void* e,
                           void* Q, int* info, ChaseState* cst, int* scale_exp, bool stein, void* w,
                           void* qtmp, void* rows2) {
  if (nblocks <= 0) return cudaSuccess;
#define GLA_TRI(T, Tin, WQ, ST)                                                                                 \
  k_tridiag<T, Tin, WQ, ST><<<nblocks, nt, smem, st>>>(descs, perm, (const Tin*)A, lower, (T*)d, (T*)e, (T*)Q, \
                                                       info, cst, scale_exp, (T*)w, (T*)qtmp, (T*)rows2)
  if (tcode == kF64) {
    if (wantq) GLA_TRI(double, double, true, false);
    else GLA_TRI(double, double, false, false);
  } else if (tcode == kF32) {
    if (wantq && stein) GLA_TRI(float, float, true, true);
    else if (wantq) GLA_TRI(float, float, true, false);
    else GLA_TRI(float, float, false, false);
  } else {
    if (wantq && stein) GLA_TRI(float, double, true, true);
    else if (wantq) GLA_TRI(float, double, true, false);
    else GLA_TRI(float, double, false, false);
  }
#undef GLA_TRI
  return cudaGetLastError();
}

}  // namespace gla
