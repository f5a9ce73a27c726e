// Double-float-accurate GEMM on the tcgen05 tensor cores (Ozaki scheme).
//
//   C = A B,  A (M x K) and B (K x N) given as float pairs (hi + lo, ~48
//   significant bits), C returned as a float pair, ~2^-47 relative to
//   sum_k |a_ik b_kj|.
//
// Scheme (K. Ozaki, T. Ogita, S. Oishi, S. M. Rump, "Error-free
// transformations of matrix multiplication by using fast routines of matrix
// multiplication and its applications", Numer. Algorithms 59 (2012)):
// every row i of A is scaled by sigma_i = 2^e_i >= max_k |a_ik| and split
// into integer slices, a_ik / sigma_i = sum_s d_s 2^(-7 s) (|d_1| <= 128,
// |d_s| <= 65 after), likewise every column of B; all slices are exact in
// bf16. A slice product sum_k d_s e_t is a sum of integers of at most 2^14,
// so an FP32 accumulator holds it exactly while the running sum stays below
// 2^24. Pairs with s + t = L share one TMEM accumulator per "level" L
// (L = 2 .. 8, the pairs with s + t <= 8: 2^-47 of the scaled product), and
// every 256 k the accumulators are drained into double-float registers.
// Exactness of a 256-k group: |d_1| <= 129, |d_s| <= 65 (s >= 2), so a level
// adds per k at most 129^2 (L = 2) or 2 x 129 x 65 + 5 x 65^2 = 37,895
// (L = 8, the largest), and 256 x 37,895 < 2^24.
//
// Kernel layout: CTA tile 128 x 64 of C, 10 warps. Warp 0 (one lane)
// streams each 32-wide k slab with two 1D bulk copies (all A slices, all B
// slices; they are stored pre-tiled in the MMA's canonical no-swizzle
// K-major layout, slab-major) into a two-stage shared-memory ring; warp 1
// (one lane) issues tcgen05.mma (M = 128, N = 64, K = 16, bf16 -> f32) into
// the level accumulators, the 28 pairs unrolled with constant descriptor
// offsets, and commits to mbarriers; warps 2-9 drain TMEM (tcgen05.ld)
// after each 256-k group, each thread keeping the double-float sums of 32
// columns of its row, then scale and store. Every mbarrier wait is bounded:
// a wait that runs out sets the error word, the CTA stops issuing work,
// waits (bounded) for its own copies and MMAs, frees its TMEM and returns.
#pragma once
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include "df64.cuh"
#include "oz_prims.cuh"

namespace gla {
namespace oz {

constexpr int kBM = 128;        // C tile rows (MMA M)
constexpr int kGroupK = 256;    // k per TMEM drain (exactness bound)
constexpr int kMaxSlices = 7;
constexpr int kDrainWarps = 8;  // two per TMEM lane quarter
constexpr int kThreads = 64 + 32 * kDrainWarps;

// Bytes of one tiled slab block: rows x kKS k, bf16.
__host__ __device__ constexpr int block_bytes(int rows) { return rows * kKS * 2; }
constexpr int kABlock = block_bytes(kBM);  // 8 KB

// Kernel configurations. S slices per operand, pairs with s + t <= S + 1
// (levels 2 .. S + 1, one TMEM accumulator of BN columns each), C tiles of
// 128 x BN:
//   double-float products: 7 slices (49 bits), 28 pairs, BN = 64, output as
//     a float pair;
//   FP32-accuracy products: 4 slices (28 bits, relative to the row and
//     column maxima), 10 pairs, BN = 128 (four levels fill the 512 TMEM
//     columns), output in FP32.
// Exactness of a 256-k group for S = 4: the largest level (5) adds at most
// 2 x 129 x 65 + 2 x 65^2 = 25,220 per k, 256 x 25,220 < 2^24.
template <int S_, int BN_, bool DF_>
struct OzCfg {
  static constexpr int S = S_;
  static constexpr int BN = BN_;
  static constexpr bool DF = DF_;
  static constexpr int kMaxLevel = S + 1;
  static constexpr int kBBlock = block_bytes(BN);
  static constexpr uint32_t kAAll = S * kABlock, kBAll = S * kBBlock;
  static constexpr size_t kStageBytes = (size_t)kAAll + kBAll;
  static constexpr int kStages = kStageBytes <= 65536 ? 3 : 2;
  static constexpr size_t kSmem = kStages * kStageBytes;
  static constexpr int kDrainCols = BN / (kDrainWarps / 4);
  // kind::f16 instruction descriptor: F32 accumulate, bf16 A and B, both
  // K-major, M = kBM, N = nn
  __host__ __device__ static constexpr uint32_t idesc(int nn) {
    return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(nn >> 3) << 17) | ((uint32_t)(kBM >> 4) << 24);
  }
  static_assert(S * BN <= 512, "level accumulators exceed the TMEM columns");
  static_assert(kSmem + 1024 <= 232448, "stage ring exceeds shared memory");
};
using CfgDF = OzCfg<7, 64, true>;
using CfgF32 = OzCfg<4, 128, false>;

// Sliced operand: slice s, row block b (height H rows), k slab q at
// base + ((b * nks + q) * S + s) * block_bytes(H): the slices of one slab are
// adjacent, so one bulk copy moves all of them.
struct Sliced {
  __nv_bfloat16* base;
  int* exps;   // per row: scale exponent e (rows scaled by 2^-e)
  unsigned* mbits;  // per row: bits of max |hi| (slicing scratch)
  int rows, nblk, nks, H, S;  // S: slices per value once sliced, 0 before
};

struct GemmArgs {
  Sliced A, B;           // A: rows = M (H = 128); B: rows = N (H = BN)
  int M, N, K;
  int ntn;               // column tiles
  float* Chi;            // FP32-accuracy configuration: the result
  float* Clo;            // (double-float configuration only)
  long long ldc;
  int lower;             // only tiles touching the lower triangle, only i >= j stored
  int* err;
};

// ---------------------------------------------------------------- slicing
//
// A float-pair matrix becomes the tiled operand in two passes:
//   1. the largest |hi| of every operand row (a column of the source for
//      k_oz_rowmax_cols, a row for k_oz_rowmax_rows), as float bits;
//   2. k_oz_tile: one CTA per (row block, 32-k slab) loads its H x 32 pairs
//      coalesced, forms the seven slices of each, lays them out in shared
//      memory in the MMA's canonical layout and writes the slab's seven
//      contiguous blocks with 16-byte stores.
// Slices of a value scaled to |v| < 1 by 2^-e, e = ilogb(max |hi|) + 1:
// d_1 = rint(128 v), then repeatedly the remainder times 128 (the remainder
// r = (hi, lo) 2^-e is kept exactly in double-float: scalings by powers of
// two, TwoSum); |d_1| <= 128 (129 for an edge value reaching 1, still exact
// in bf16 and inside the accumulation bound), |d_s| <= 65 after.

// Source columns c (len entries from hi + c ld): one warp per column.
__global__ void __launch_bounds__(256) k_oz_rowmax_cols(const float* __restrict__ hi, long long ld, int len,
                                                        int count, int rows_pad, unsigned* __restrict__ mbits) {
  const int c = blockIdx.x * 8 + (threadIdx.x >> 5), lane = threadIdx.x & 31;
  if (c >= rows_pad) return;
  float m = 0.f;
  if (c < count)
    for (int k = lane; k < len; k += 32) m = fmaxf(m, fabsf(hi[(long long)c * ld + k]));
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
  if (lane == 0) mbits[c] = __float_as_uint(m);
}

// Source rows c (element (c, k) at hi[c + k ld]): one thread per row and
// k chunk, merged by an atomic max on the (non-negative) float bits; mbits
// must be zero on entry.
__global__ void __launch_bounds__(256) k_oz_rowmax_rows(const float* __restrict__ hi, long long ld, int len,
                                                        int rows, int kchunk, unsigned* __restrict__ mbits) {
  const int c = blockIdx.x * 256 + threadIdx.x;
  if (c >= rows) return;
  const int k0 = blockIdx.y * kchunk, k1 = min(len, k0 + kchunk);
  float m = 0.f;
  for (int k = k0; k < k1; k++) m = fmaxf(m, fabsf(hi[c + (long long)k * ld]));
  if (m > 0.f) atomicMax(&mbits[c], __float_as_uint(m));
}

// ROWS = false: operand row c is source column c (element (c, k) at
// c ld + k); ROWS = true: operand row c is source row c (at c + k ld).
// Dynamic shared memory: S x block_bytes(H).
template <bool ROWS, int S>
__global__ void __launch_bounds__(256) k_oz_tile(const float* __restrict__ hi, const float* __restrict__ lo,
                                                 long long ld, int len, int count, Sliced out) {
  extern __shared__ __align__(16) unsigned char tsm[];
  const int b = blockIdx.x, q = blockIdx.y, H = out.H, tid = threadIdx.x;
  const int bb = block_bytes(H);
  const int per = H * kKS / 256;  // elements per thread
  for (int t = 0; t < per; t++) {
    int r, kk;
    if (ROWS) {  // a warp covers 32 consecutive rows of one k
      const int e = t * 256 + tid;
      r = e % H;
      kk = e / H;
    } else {  // a warp covers the 32 k of one row
      r = t * (256 / kKS) + tid / kKS;
      kk = tid % kKS;
    }
    const int c = b * H + r, k = q * kKS + kk;
    float vh = 0.f, vl = 0.f;
    if (c < count && k < len) {
      const long long idx = ROWS ? c + (long long)k * ld : (long long)c * ld + k;
      const int ex = slice_exp(out.mbits[c]);
      vh = ldexpf(hi[idx], -ex);
      vl = lo ? ldexpf(lo[idx], -ex) : 0.f;
    }
    unsigned char* dst = tsm + tile_off(r, kk);
#pragma unroll
    for (int s = 0; s < S; s++) {
      const float th = vh * 128.f, tl = vl * 128.f;
      const float d = rintf(th);
      float sh, se;
      two_sum(th - d, tl, sh, se);  // th - d is exact (|th - d| <= 1/2, same binade scale)
      vh = sh;
      vl = se;
      *reinterpret_cast<__nv_bfloat16*>(dst + s * bb) = __float2bfloat16_rn(d);
    }
  }
  if (q == 0)
    for (int r = tid; r < H; r += 256) out.exps[b * H + r] = slice_exp(out.mbits[b * H + r]);
  __syncthreads();
  uint4* g = reinterpret_cast<uint4*>(reinterpret_cast<char*>(out.base) +
                                      ((size_t)b * out.nks + q) * S * (size_t)bb);
  const uint4* sv = reinterpret_cast<const uint4*>(tsm);
  for (int v = tid; v < S * bb / 16; v += 256) g[v] = sv[v];
}

// ---------------------------------------------------------------- GEMM

template <class Cfg>
__global__ void __launch_bounds__(kThreads, 1) k_oz_gemm(const GemmArgs g) {
  constexpr int kStages = Cfg::kStages, kBN = Cfg::BN, kMaxLevel = Cfg::kMaxLevel, kDrainCols = Cfg::kDrainCols;
  constexpr int kBBlock = Cfg::kBBlock;
  extern __shared__ __align__(1024) unsigned char sm[];
  __shared__ __align__(8) uint64_t full_bar[kStages], empty_bar[kStages], drain_full, drain_empty, fin_bar;
  __shared__ uint32_t tmem_base;
  __shared__ int s_abort_raw;
  volatile int* s_abort = &s_abort_raw;
  const int tid = threadIdx.x, wid = tid >> 5, lane = tid & 31;
  const int tm = blockIdx.x / g.ntn, tn = blockIdx.x % g.ntn;
  const int row0 = tm * kBM, col0 = tn * kBN;
  if (g.lower && row0 + kBM <= col0) return;  // (uniform) no TMEM touched yet
  const int nks = g.A.nks;
  const int ngroups = (nks * kKS + kGroupK - 1) / kGroupK;
  const int spg = kGroupK / kKS;  // stages per drain group
  volatile int* err = g.err;
  if (tid == 0) {
    for (int i = 0; i < kStages; i++) {
      mbar_init(&full_bar[i], 1);
      mbar_init(&empty_bar[i], 1);
    }
    mbar_init(&drain_full, 1);
    mbar_init(&drain_empty, 32 * kDrainWarps);
    mbar_init(&fin_bar, 1);
    *s_abort = 0;
    asm volatile("fence.mbarrier_init.release.cluster;");
  }
  if (wid == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&tmem_base)),
                 "r"(512));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  asm volatile("tcgen05.fence::before_thread_sync;");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;");
  const uint32_t tmem = tmem_base;
  constexpr size_t stB = Cfg::kStageBytes;
  constexpr uint32_t kAAll = Cfg::kAAll, kBAll = Cfg::kBAll;

  if (wid == 0) {
    // ---- producer: slabs of every slice into the stage ring
    if (lane == 0) {
      const char* Ab = reinterpret_cast<const char*>(g.A.base);
      const char* Bb = reinterpret_cast<const char*>(g.B.base);
      int issued = 0;  // slabs whose copies were started
      for (int q = 0; q < nks && !*s_abort; q++) {
        const int st = q % kStages;
        if (q >= kStages && !mbar_wait(&empty_bar[st], ((q / kStages) - 1) & 1, err)) {
          *s_abort = 1;
          break;
        }
        issued = q + 1;
        unsigned char* dst = sm + st * stB;
        mbar_expect_tx(&full_bar[st], (uint32_t)stB);
        bulk_g2s(dst, Ab + ((size_t)tm * nks + q) * kAAll, kAAll, &full_bar[st]);
        bulk_g2s(dst + kAAll, Bb + ((size_t)tn * nks + q) * kBAll, kBAll, &full_bar[st]);
      }
      // before the CTA may exit, its last copies must have landed (bounded;
      // already true unless the CTA aborted)
      for (int q = (issued > kStages ? issued - kStages : 0); q < issued; q++)
        for (long long it = 0; it < kWaitLimit && !mbar_try(&full_bar[q % kStages], (q / kStages) & 1); it++) {
        }
    }
  } else if (wid == 1) {
    // ---- MMA issuer: per slab the slice pairs, unrolled with constant
    // descriptor offsets (the descriptor's address field is addr >> 4 and
    // shared-memory offsets stay below 2^18, so adding offset >> 4 is exact)
    if (lane == 0) {
      for (int gi = 0; gi < ngroups && !*s_abort; gi++) {
        if (gi > 0 && !mbar_wait(&drain_empty, (gi - 1) & 1, err)) {  // the drain of group gi-1 is done
          *s_abort = 1;
          break;
        }
        asm volatile("tcgen05.fence::after_thread_sync;");
        for (int qq = 0; qq < spg; qq++) {
          const int q = gi * spg + qq;
          if (q >= nks) break;
          const int st = q % kStages;
          if (!mbar_wait(&full_bar[st], (q / kStages) & 1, err)) {
            *s_abort = 1;
            break;
          }
          asm volatile("tcgen05.fence::after_thread_sync;");
          const uint64_t a0 = make_desc(smem_u32(sm + st * stB));
          const uint64_t b0 = a0 + (uint64_t)(kAAll >> 4);
          // A slice s times B slices t = 1 .. kMaxLevel - s at once: those
          // are adjacent BN-row blocks of the stage (one K-major operand of
          // BN (kMaxLevel - s) rows in the same layout, split at the MMA's
          // N <= 256) and their levels s + 1 .. kMaxLevel adjacent BN-column
          // accumulators: A is read once per group instead of once per pair
#pragma unroll
          for (int ks = 0; ks < kKS / 16; ks++)  // K = 16 per instruction: 2 K-core matrices = 256 B
#pragma unroll
            for (int s = 1; s <= Cfg::S; s++) {
              // s = 1 reaches every level first and starts the group's
              // accumulators from zero
              const uint32_t accumulate = (qq == 0 && ks == 0 && s == 1) ? 0u : 1u;
              constexpr int kMaxT = 256 / kBN;  // B slices per MMA (N <= 256)
#pragma unroll
              for (int t0 = 1; t0 <= Cfg::S; t0 += kMaxT) {
                const int nt = kMaxLevel - s - t0 + 1;  // slices t0 .. kMaxLevel - s left
                if (nt <= 0) continue;
                const int cnt = nt < kMaxT ? nt : kMaxT;
                mma_f16(tmem + (uint32_t)((s + t0 - 2) * kBN),
                        a0 + (uint64_t)(((s - 1) * kABlock + ks * 256) >> 4),
                        b0 + (uint64_t)(((t0 - 1) * kBBlock + ks * 256) >> 4), Cfg::idesc(cnt * kBN), accumulate);
              }
            }
          mma_commit(&empty_bar[st]);  // stage buffer reusable once these MMAs finish
        }
        mma_commit(&drain_full);  // the group's accumulators are complete
      }
    }
  } else {
    // ---- drain warps: TMEM lanes 32 (wid % 4) .. +31 = C rows of this
    // thread; columns cbase .. cbase + kDrainCols - 1 of the tile
    const int quarter = wid & 3;
    const int cbase = ((wid - 2) / 4) * kDrainCols;
    const int r = row0 + quarter * 32 + lane;
    // double-float sums (DF) or FP32 sums of the groups
    df64 acc[Cfg::DF ? kDrainCols : 1];
    float accf[Cfg::DF ? 1 : kDrainCols];
#pragma unroll
    for (int c = 0; c < kDrainCols; c++) {
      if (Cfg::DF)
        acc[c] = df_make(0.f, 0.f);
      else
        accf[c] = 0.f;
    }
    bool ok = true;
    for (int gi = 0; gi < ngroups && ok; gi++) {
      if (!mbar_wait(&drain_full, gi & 1, err)) {
        ok = false;
        break;
      }
      asm volatile("tcgen05.fence::after_thread_sync;");
      // level values of each column, exact integers; combine small to large
#pragma unroll
      for (int c0 = 0; c0 < kDrainCols; c0 += 16) {
        float part_hi[16], part_lo[16];
#pragma unroll
        for (int q = 0; q < 16; q++) part_hi[q] = part_lo[q] = 0.f;
#pragma unroll 1
        for (int L = kMaxLevel; L >= 2; L--) {
          uint32_t v[16];
          tmem_ld16(tmem + ((uint32_t)(quarter * 32) << 16) + (uint32_t)((L - 2) * kBN + cbase + c0), v);
          asm volatile("tcgen05.wait::ld.sync.aligned;");
          const float sc = ldexpf(1.f, -7 * L);
#pragma unroll
          for (int q = 0; q < 16; q++) {
            if (Cfg::DF) {
              float sh, se;
              two_sum(part_hi[q], __uint_as_float(v[q]) * sc, sh, se);
              part_hi[q] = sh;
              part_lo[q] += se;
            } else {
              part_hi[q] = fmaf(__uint_as_float(v[q]), sc, part_hi[q]);
            }
          }
        }
#pragma unroll
        for (int q = 0; q < 16; q++) {
          if (Cfg::DF)
            acc[c0 + q] = df_add(acc[c0 + q], df_make(part_hi[q], part_lo[q]));
          else
            accf[c0 + q] += part_hi[q];
        }
      }
      asm volatile("tcgen05.fence::before_thread_sync;");
      mbar_arrive(&drain_empty);
    }
    if (ok && !*err) {
      const int ei = r < g.M ? g.A.exps[r] : 0;
#pragma unroll
      for (int c = 0; c < kDrainCols; c++) {
        const int col = col0 + cbase + c;
        if (r >= g.M || col >= g.N || (g.lower && r < col)) continue;
        const int e = ei + g.B.exps[col];
        const long long idx = (long long)r + (long long)col * g.ldc;
        if (Cfg::DF) {
          g.Chi[idx] = ldexpf(acc[c].hi, e);
          g.Clo[idx] = ldexpf(acc[c].lo, e);
        } else {
          g.Chi[idx] = ldexpf(accf[c], e);
        }
      }
    }
  }
  // teardown: every MMA this CTA issued has finished (a final commit, waited
  // for with a bound) before TMEM is freed
  __syncthreads();
  if (wid == 1 && lane == 0) {
    mma_commit(&fin_bar);
    for (long long it = 0; it < kWaitLimit && !mbar_try(&fin_bar, 0); it++) {
    }
  }
  asm volatile("tcgen05.fence::before_thread_sync;");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;");
  if (wid == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(512));
}

}  // namespace oz
}  // namespace gla
