// Host side of the tcgen05 Ozaki GEMM (ozaki.cuh): slice buffers, slicing
// launches, the GEMM launch and its error word.
#include <algorithm>
#include <mutex>
#include <new>

#include "gla_large.h"
#include "ozaki.cuh"

namespace gla {

struct OzWork {
  oz::Sliced A{}, B{};
  size_t abytes = 0, bbytes = 0;
  int* err = nullptr;
};

namespace {
size_t sliced_bytes(int rows, int K, int H, int S) {
  const int nblk = (rows + H - 1) / H, nks = (K + oz::kKS - 1) / oz::kKS;
  return (size_t)S * nblk * nks * oz::block_bytes(H);
}
void init_sliced(oz::Sliced& s, int rows, int K, int H) {
  s.rows = rows;
  s.H = H;
  s.nblk = (rows + H - 1) / H;
  s.nks = (K + oz::kKS - 1) / oz::kKS;
  s.S = 0;
}
constexpr size_t kGemmSmem = oz::kStages * oz::stage_bytes(oz::kMaxSlices, oz::kMaxSlices);
}  // namespace

int oz_create(OzWork** out, int m, int n, int K) {
  *out = nullptr;
  OzWork* w = new (std::nothrow) OzWork();
  if (!w) return -1000 - (int)cudaErrorMemoryAllocation;
  init_sliced(w->A, std::max(m, 1), K, oz::kBM);
  init_sliced(w->B, std::max(n, 1), K, oz::kBN);
  w->abytes = m > 0 ? sliced_bytes(m, K, oz::kBM, oz::kMaxSlices) : 16;
  w->bbytes = n > 0 ? sliced_bytes(n, K, oz::kBN, oz::kMaxSlices) : 16;
  cudaError_t e = cudaMalloc((void**)&w->A.base, w->abytes);
  if (e == cudaSuccess) e = cudaMalloc((void**)&w->B.base, w->bbytes);
  if (e == cudaSuccess) e = cudaMalloc((void**)&w->A.exps, sizeof(int) * w->A.nblk * oz::kBM);
  if (e == cudaSuccess) e = cudaMalloc((void**)&w->B.exps, sizeof(int) * w->B.nblk * oz::kBN);
  if (e == cudaSuccess) e = cudaMalloc((void**)&w->err, sizeof(int));
  if (e == cudaSuccess) e = cudaMemset(w->err, 0, sizeof(int));
  static std::once_flag once;
  static cudaError_t attr = cudaSuccess;
  std::call_once(once, [] {
    attr = cudaFuncSetAttribute((const void*)oz::k_oz_gemm, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                (int)kGemmSmem);
  });
  if (e == cudaSuccess) e = attr;
  if (e != cudaSuccess) {
    oz_destroy(w);
    return -1000 - (int)e;
  }
  *out = w;
  return 0;
}

void oz_destroy(OzWork* w) {
  if (!w) return;
  cudaFree(w->A.base);
  cudaFree(w->B.base);
  cudaFree(w->A.exps);
  cudaFree(w->B.exps);
  cudaFree(w->err);
  delete w;
}

cudaError_t oz_slice(OzWork* w, bool a_operand, const float* hi, const float* lo, long long ld, int count, int len,
                     int S, cudaStream_t st) {
  oz::Sliced& s = a_operand ? w->A : w->B;
  if (S != oz::kMaxSlices || count > s.nblk * s.H || (len + oz::kKS - 1) / oz::kKS > s.nks)
    return cudaErrorInvalidValue;
  s.S = S;
  oz::k_oz_slice<<<s.nblk * s.H, 256, 0, st>>>(hi, lo, ld, len, count, s);
  return cudaGetLastError();
}

cudaError_t oz_slice_rows(OzWork* w, const float* hi, const float* lo, long long ld, int rows, int len, int S,
                          cudaStream_t st) {
  oz::Sliced& s = w->A;
  if (S != oz::kMaxSlices || rows > s.nblk * s.H || (len + oz::kKS - 1) / oz::kKS > s.nks)
    return cudaErrorInvalidValue;
  s.S = S;
  oz::k_oz_slice_rows<<<s.nblk, 256, 0, st>>>(hi, lo, ld, len, rows, s);
  return cudaGetLastError();
}

bool oz_fits(const OzWork* w, int m, int n, int K) {
  return w->A.nblk * w->A.H >= m && w->B.nblk * w->B.H >= n && w->A.nks == (K + oz::kKS - 1) / oz::kKS;
}

cudaError_t oz_gemm(OzWork* w, int M, int N, int K, float* Chi, float* Clo, long long ldc, bool lower,
                    cudaStream_t st) {
  return oz_gemm2(w, w, M, N, K, Chi, Clo, ldc, lower, st);
}

cudaError_t oz_gemm2(OzWork* wa, OzWork* wb, int M, int N, int K, float* Chi, float* Clo, long long ldc, bool lower,
                     cudaStream_t st) {
  if (M <= 0 || N <= 0) return cudaSuccess;
  if (wa->A.S != oz::kMaxSlices || wb->B.S != oz::kMaxSlices || wa->A.nks != wb->B.nks) return cudaErrorInvalidValue;
  oz::GemmArgs g;
  g.A = wa->A;
  g.B = wb->B;
  OzWork* w = wa;
  g.M = M;
  g.N = N;
  g.K = K;
  g.ntn = (N + oz::kBN - 1) / oz::kBN;
  g.Chi = Chi;
  g.Clo = Clo;
  g.ldc = ldc;
  g.lower = lower ? 1 : 0;
  g.err = w->err;
  const int ntm = (M + oz::kBM - 1) / oz::kBM;
  oz::k_oz_gemm<<<ntm * g.ntn, oz::kThreads, kGemmSmem, st>>>(g);
  return cudaGetLastError();
}

int* oz_error_word(OzWork* w) { return w->err; }

}  // namespace gla
