// Host side of the tcgen05 Ozaki GEMM (ozaki.cuh): slice buffers, slicing
// launches, the GEMM launch and its error word. A work object is made for
// one kernel configuration: double-float products (oz_create, 7 slices,
// 128 x 64 tiles) or FP32-accuracy products (oz_create_f32, 4 slices,
// 128 x 128 tiles).
#include <algorithm>
#include <mutex>
#include <new>

#include "gla_large.h"
#include "ozaki.cuh"

namespace gla {

struct OzWork {
  oz::Sliced A{}, B{};
  size_t abytes = 0, bbytes = 0;
  int a_nks_cap = 0, b_nks_cap = 0;  // k slabs the buffers hold (the slicing sets the current count)
  int S = oz::kMaxSlices;  // slices per value of this configuration
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

cudaError_t set_attributes() {
  static std::once_flag once;
  static cudaError_t attr = cudaSuccess;
  std::call_once(once, [] {
    auto set = [](const void* f, size_t bytes) {
      if (attr == cudaSuccess) attr = cudaFuncSetAttribute(f, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
    };
    set((const void*)oz::k_oz_gemm<oz::CfgDF>, oz::CfgDF::kSmem);
    set((const void*)oz::k_oz_gemm<oz::CfgF32>, oz::CfgF32::kSmem);
    set((const void*)oz::k_oz_tile<false, 7>, 7 * oz::block_bytes(oz::kBM));
    set((const void*)oz::k_oz_tile<true, 7>, 7 * oz::block_bytes(oz::kBM));
    set((const void*)oz::k_oz_tile<false, 4>, 4 * oz::block_bytes(oz::kBM));
    set((const void*)oz::k_oz_tile<true, 4>, 4 * oz::block_bytes(oz::kBM));
  });
  return attr;
}

int create(OzWork** out, int m, int n, int K, int S, int bn) {
  *out = nullptr;
  OzWork* w = new (std::nothrow) OzWork();
  if (!w) return -1000 - (int)cudaErrorMemoryAllocation;
  w->S = S;
  init_sliced(w->A, std::max(m, 1), K, oz::kBM);
  init_sliced(w->B, std::max(n, 1), K, bn);
  w->a_nks_cap = w->A.nks;
  w->b_nks_cap = w->B.nks;
  w->abytes = m > 0 ? sliced_bytes(m, K, oz::kBM, S) : 16;
  w->bbytes = n > 0 ? sliced_bytes(n, K, bn, S) : 16;
  cudaError_t e = cudaMalloc((void**)&w->A.base, w->abytes);
  if (e == cudaSuccess) e = cudaMalloc((void**)&w->B.base, w->bbytes);
  if (e == cudaSuccess) e = cudaMalloc((void**)&w->A.exps, sizeof(int) * w->A.nblk * oz::kBM);
  if (e == cudaSuccess) e = cudaMalloc((void**)&w->B.exps, sizeof(int) * w->B.nblk * bn);
  if (e == cudaSuccess) e = cudaMalloc((void**)&w->A.mbits, sizeof(unsigned) * w->A.nblk * oz::kBM);
  if (e == cudaSuccess) e = cudaMalloc((void**)&w->B.mbits, sizeof(unsigned) * w->B.nblk * bn);
  if (e == cudaSuccess) e = cudaMalloc((void**)&w->err, sizeof(int));
  if (e == cudaSuccess) e = cudaMemset(w->err, 0, sizeof(int));
  if (e == cudaSuccess) e = set_attributes();
  if (e != cudaSuccess) {
    oz_destroy(w);
    return -1000 - (int)e;
  }
  *out = w;
  return 0;
}

template <bool ROWS>
void launch_tile(int S, const float* hi, const float* lo, long long ld, int len, int count, const oz::Sliced& s,
                 cudaStream_t st) {
  const dim3 grid(s.nblk, s.nks);
  const size_t smem = (size_t)S * oz::block_bytes(s.H);
  if (S == 7)
    oz::k_oz_tile<ROWS, 7><<<grid, 256, smem, st>>>(hi, lo, ld, len, count, s);
  else
    oz::k_oz_tile<ROWS, 4><<<grid, 256, smem, st>>>(hi, lo, ld, len, count, s);
}
}  // namespace

int oz_create(OzWork** out, int m, int n, int K) { return create(out, m, n, K, oz::CfgDF::S, oz::CfgDF::BN); }

int oz_create_f32(OzWork** out, int m, int n, int K) {
  return create(out, m, n, K, oz::CfgF32::S, oz::CfgF32::BN);
}

void oz_destroy(OzWork* w) {
  if (!w) return;
  cudaFree(w->A.base);
  cudaFree(w->B.base);
  cudaFree(w->A.exps);
  cudaFree(w->B.exps);
  cudaFree(w->A.mbits);
  cudaFree(w->B.mbits);
  cudaFree(w->err);
  delete w;
}

cudaError_t oz_slice(OzWork* w, bool a_operand, const float* hi, const float* lo, long long ld, int count, int len,
                     int S, cudaStream_t st) {
  oz::Sliced& s = a_operand ? w->A : w->B;
  const int nks = std::max(1, (len + oz::kKS - 1) / oz::kKS);
  if (S != w->S || count > s.nblk * s.H || nks > (a_operand ? w->a_nks_cap : w->b_nks_cap))
    return cudaErrorInvalidValue;
  s.S = S;
  s.nks = nks;
  const int rows_pad = s.nblk * s.H;
  oz::k_oz_rowmax_cols<<<(rows_pad + 7) / 8, 256, 0, st>>>(hi, ld, len, count, rows_pad, s.mbits);
  launch_tile<false>(S, hi, lo, ld, len, count, s, st);
  return cudaGetLastError();
}

cudaError_t oz_slice_rows(OzWork* w, const float* hi, const float* lo, long long ld, int rows, int len, int S,
                          cudaStream_t st) {
  oz::Sliced& s = w->A;
  const int nks = std::max(1, (len + oz::kKS - 1) / oz::kKS);
  if (S != w->S || rows > s.nblk * s.H || nks > w->a_nks_cap) return cudaErrorInvalidValue;
  s.S = S;
  s.nks = nks;
  const int rows_pad = s.nblk * s.H;
  cudaError_t e = cudaMemsetAsync(s.mbits, 0, sizeof(unsigned) * rows_pad, st);
  if (e != cudaSuccess) return e;
  const int kchunk = 128, nch = (len + kchunk - 1) / kchunk;
  if (rows > 0 && nch > 0)
    oz::k_oz_rowmax_rows<<<dim3((rows + 255) / 256, nch), 256, 0, st>>>(hi, ld, len, rows, kchunk, s.mbits);
  launch_tile<true>(S, hi, lo, ld, len, rows, s, st);
  return cudaGetLastError();
}

bool oz_fits(const OzWork* w, int m, int n, int K) {
  const int nks = std::max(1, (K + oz::kKS - 1) / oz::kKS);
  return w->A.nblk * w->A.H >= m && w->B.nblk * w->B.H >= n && w->a_nks_cap >= nks && w->b_nks_cap >= nks;
}

cudaError_t oz_gemm(OzWork* w, int M, int N, int K, float* Chi, float* Clo, long long ldc, bool lower,
                    cudaStream_t st) {
  return oz_gemm2(w, w, M, N, K, Chi, Clo, ldc, lower, st);
}

cudaError_t oz_gemm2(OzWork* wa, OzWork* wb, int M, int N, int K, float* Chi, float* Clo, long long ldc, bool lower,
                     cudaStream_t st) {
  if (M <= 0 || N <= 0) return cudaSuccess;
  if (wa->S != wb->S || wa->A.S != wa->S || wb->B.S != wb->S || wa->A.nks != wb->B.nks)
    return cudaErrorInvalidValue;
  const bool df = wa->S == oz::CfgDF::S;
  const int bn = df ? oz::CfgDF::BN : oz::CfgF32::BN;
  if (wb->B.H != bn || (df && !Clo)) return cudaErrorInvalidValue;
  oz::GemmArgs g;
  g.A = wa->A;
  g.B = wb->B;
  g.M = M;
  g.N = N;
  g.K = K;
  g.ntn = (N + bn - 1) / bn;
  g.Chi = Chi;
  g.Clo = Clo;
  g.ldc = ldc;
  g.lower = lower ? 1 : 0;
  g.err = wa->err;
  const int ntm = (M + oz::kBM - 1) / oz::kBM;
  if (df)
    oz::k_oz_gemm<oz::CfgDF><<<ntm * g.ntn, oz::kThreads, oz::CfgDF::kSmem, st>>>(g);
  else
    oz::k_oz_gemm<oz::CfgF32><<<ntm * g.ntn, oz::kThreads, oz::CfgF32::kSmem, st>>>(g);
  return cudaGetLastError();
}

int* oz_error_word(OzWork* w) { return w->err; }

}  // namespace gla
