// FP32 GEMM on the tcgen05 tensor cores in split TF32 ("3xTF32"), operands
// fed by TMA tensor-map loads. Used by the FP32 large-matrix path for the
// rank-2k trailing updates of the Householder reduction and for the two
// GEMMs of the compact-WY back-transformation (large_sytrd.cu,
// large_backtr.cu), and exported as gla_sgemm_3xtf32.
//
//   D(i, j) = alpha * sum_seg sum_k A_seg(i, k) B_seg(k, j) + beta * D(i, j)
//
// Both operands are K-major: A(i, k) at a[k + i lda] and B(k, j) at
// b[k + j ldb] (the transpose of a column-major A, and a column-major B).
// Each value x ~ hi + lo with hi = x rounded to TF32 (19 bits) and lo = the
// remainder x - hi rounded to TF32 (|x - hi - lo| <= 2^-22 |x|), and
// A B ~ Ahi Bhi + Ahi Blo + Alo Bhi with FP32 accumulation in TMEM: the
// dropped Alo Blo and the split's remainder are ~2^-21 relative to |A||B|
// per product; a few FP32 roundings.
#pragma once
#include <cuda.h>
#include <cuda_runtime.h>
#include <stdint.h>

namespace gla {
namespace tc {

constexpr int kBM = 128;   // D tile rows (MMA M, TMEM lanes)
constexpr int kBN = 128;   // D tile columns (MMA N, TMEM columns)
constexpr int kBK = 32;    // k per stage: 32 floats = one 128-byte swizzle row

struct TcArgs {
  int M, N;           // extent of D
  int nseg;           // 1 or 2 segments of K, accumulated into the same D
  int K[2];           // K extent of each segment
  int a_x[2], b_x[2]; // tensor-map K coordinate where each segment starts (multiples of 4)
  int a_y, b_y;       // tensor-map row coordinate of A's row 0 and B's column 0
  int ksplit;         // split-K (one segment only): k per split (multiple of kBK), 0 = none
  long long split_stride;  // split s writes D + s split_stride (beta must be 0)
  float* D;
  long long ldd;
  float alpha, beta;
  int lower;          // only tiles meeting the lower triangle, only i >= j stored
  int* err;           // set when a bounded wait runs out
};

// The driver's tensor-map encoder, looked up once (false when unavailable).
bool tc_available();

// Tensor map of a K-major operand stored as a column-major float array:
// element (r, k) at base[k + r ld], k < kext, r < rows; box kBK x box_rows;
// 128-byte swizzle; loads past the extents read zeros. Requires base
// 16-byte aligned and ld a multiple of 4 (returns false otherwise).
bool tc_make_map(CUtensorMap* m, const float* base, long long kext, long long rows, long long ld, int box_rows);

cudaError_t tc_gemm_launch(const CUtensorMap& mA, const CUtensorMap& mB, const TcArgs& g, int splits,
                           cudaStream_t st);

}  // namespace tc
}  // namespace gla
