// Instantiations and launchers of the SIMT GEMM (gemm_simt.cuh).
#include "gla_large.h"

namespace gla {

// Two CTAs per SM (at most 128 registers per thread): one CTA of eight
// warps leaves the FP32 pipe idle behind shared-memory and global latency.
template <class T, bool TA, bool TB, bool LOWER, bool REMAP>
__global__ void __launch_bounds__(kGemmThreads, 2) k_gemm(const GemmDesc g) {
  gemm_body<T, TA, TB, LOWER, REMAP>(g, blockIdx.x, blockIdx.y);
}

template <class T>
__global__ void __launch_bounds__(kGemmThreads, 2) k_gemm_grouped(const GemmDesc* __restrict__ gs) {
  const GemmDesc g = gs[blockIdx.y];
  using Cf = GemmCfg<T>;
  if (g.m <= 0 || g.n <= 0) return;
  const int tiles = ((g.m + Cf::BM - 1) / Cf::BM) * ((g.n + Cf::BN - 1) / Cf::BN);
  if ((int)blockIdx.x >= tiles) return;
  gemm_body<T, false, false, false, true>(g, blockIdx.x, 0);
}

namespace {
template <class T>
cudaError_t launch_t(bool ta, bool tb, bool lower, const GemmDesc& g, int splits, cudaStream_t st) {
  using Cf = GemmCfg<T>;
  if (g.m <= 0 || g.n <= 0) return cudaSuccess;
  const int tiles = ((g.m + Cf::BM - 1) / Cf::BM) * ((g.n + Cf::BN - 1) / Cf::BN);
  const dim3 grid(tiles, splits > 1 ? splits : 1);
  const bool remap = g.a_kidx || g.b_kidx || g.c_nidx;
  const int code = (ta ? 4 : 0) | (tb ? 2 : 0) | (lower ? 1 : 0);
  if (remap) {
    switch (code) {  // used with B transposed and a k remap (symmetric rank-2k updates)
      case 3: k_gemm<T, false, true, true, true><<<grid, kGemmThreads, 0, st>>>(g); break;
      case 0: k_gemm<T, false, false, false, true><<<grid, kGemmThreads, 0, st>>>(g); break;
      default: return cudaErrorInvalidValue;
    }
    return cudaGetLastError();
  }
  switch (code) {
    case 0: k_gemm<T, false, false, false, false><<<grid, kGemmThreads, 0, st>>>(g); break;
    case 1: k_gemm<T, false, false, true, false><<<grid, kGemmThreads, 0, st>>>(g); break;
    case 2: k_gemm<T, false, true, false, false><<<grid, kGemmThreads, 0, st>>>(g); break;
    case 3: k_gemm<T, false, true, true, false><<<grid, kGemmThreads, 0, st>>>(g); break;
    case 4: k_gemm<T, true, false, false, false><<<grid, kGemmThreads, 0, st>>>(g); break;
    case 5: k_gemm<T, true, false, true, false><<<grid, kGemmThreads, 0, st>>>(g); break;
    case 6: k_gemm<T, true, true, false, false><<<grid, kGemmThreads, 0, st>>>(g); break;
    default: k_gemm<T, true, true, true, false><<<grid, kGemmThreads, 0, st>>>(g); break;
  }
  return cudaGetLastError();
}
}  // namespace

cudaError_t gemm_launch(bool f64, bool ta, bool tb, bool lower, const GemmDesc& g, int splits, cudaStream_t st) {
  return f64 ? launch_t<double>(ta, tb, lower, g, splits, st) : launch_t<float>(ta, tb, lower, g, splits, st);
}

cudaError_t gemm_launch_grouped(bool f64, const GemmDesc* d_descs, int nprob, int max_m, int max_n, cudaStream_t st) {
  if (nprob <= 0 || max_m <= 0 || max_n <= 0) return cudaSuccess;
  if (f64) {
    using Cf = GemmCfg<double>;
    const int tiles = ((max_m + Cf::BM - 1) / Cf::BM) * ((max_n + Cf::BN - 1) / Cf::BN);
    k_gemm_grouped<double><<<dim3(tiles, nprob), kGemmThreads, 0, st>>>(d_descs);
  } else {
    using Cf = GemmCfg<float>;
    const int tiles = ((max_m + Cf::BM - 1) / Cf::BM) * ((max_n + Cf::BN - 1) / Cf::BN);
    k_gemm_grouped<float><<<dim3(tiles, nprob), kGemmThreads, 0, st>>>(d_descs);
  }
  return cudaGetLastError();
}

}  // namespace gla
