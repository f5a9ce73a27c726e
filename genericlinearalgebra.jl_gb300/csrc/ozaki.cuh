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

namespace gla {
namespace oz {

constexpr int kBM = 128;        // C tile rows (MMA M)
constexpr int kBN = 64;         // C tile columns (MMA N)
constexpr int kKS = 32;         // k per pipeline stage (two K = 16 MMAs per slice pair)
constexpr int kStages = 2;
constexpr int kGroupK = 256;    // k per TMEM drain (exactness bound)
constexpr int kMaxSlices = 7;
constexpr int kMaxLevel = 8;    // pairs with s + t <= kMaxLevel
constexpr int kLevels = kMaxLevel - 1;  // levels 2 .. 8
constexpr int kDrainWarps = 8;  // two per TMEM lane quarter, 32 columns each
constexpr int kThreads = 64 + 32 * kDrainWarps;
constexpr int kDrainCols = kBN / (kDrainWarps / 4);
constexpr long long kWaitLimit = 1ll << 26;

// Bytes of one tiled slab block: rows x kKS k, bf16.
__host__ __device__ constexpr int block_bytes(int rows) { return rows * kKS * 2; }
constexpr int kABlock = block_bytes(kBM);  // 8 KB
constexpr int kBBlock = block_bytes(kBN);  // 4 KB
__host__ __device__ constexpr size_t stage_bytes(int sa, int sb) { return (size_t)sa * kABlock + (size_t)sb * kBBlock; }

// Byte offset of element (r, kk) inside a tiled slab block (8-row x 8-k core
// matrices of 128 contiguous bytes; K-neighbours 128 B apart = LBO, row
// groups kSBO = 512 B apart = SBO).
constexpr int kSBO = kKS * 16;
__host__ __device__ __forceinline__ int tile_off(int r, int kk) {
  return (r >> 3) * kSBO + (kk >> 3) * 128 + (r & 7) * 16 + (kk & 7) * 2;
}

// Sliced operand: slice s, row block b (height H rows), k slab q at
// base + ((b * nks + q) * kMaxSlices + s) * block_bytes(H): the slices of one
// slab are adjacent, so one bulk copy moves all of them.
struct Sliced {
  __nv_bfloat16* base;
  int* exps;   // per row: scale exponent e (rows scaled by 2^-e)
  int rows, nblk, nks, H, S;  // S: kMaxSlices once sliced, 0 before
};

GLA_DEV uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

GLA_DEV uint64_t make_desc(uint32_t saddr) {
  uint64_t d = 0;
  d |= (uint64_t)((saddr >> 4) & 0x3FFF);
  d |= (uint64_t)((128u >> 4) & 0x3FFF) << 16;  // LBO: K-neighbour core matrices
  d |= (uint64_t)(((uint32_t)kSBO >> 4) & 0x3FFF) << 32;  // SBO: next 8-row group
  d |= (uint64_t)1 << 46;                        // descriptor version (tcgen05)
  return d;                                      // base offset 0, no swizzle
}

// kind::f16 instruction descriptor: F32 accumulate, bf16 A and B, both
// K-major, N = kBN, M = kBM.
constexpr uint32_t kIdesc = (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(kBN >> 3) << 17) |
                            ((uint32_t)(kBM >> 4) << 24);

GLA_DEV void mbar_init(uint64_t* b, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(b)), "r"(count));
}
GLA_DEV bool mbar_try(uint64_t* b, uint32_t parity) {
  uint32_t done;
  asm volatile(
      "{\n.reg .pred p;\nmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\nselp.u32 %0, 1, 0, p;\n}"
      : "=r"(done)
      : "r"(smem_u32(b)), "r"(parity)
      : "memory");
  return done != 0;
}
// Bounded wait; false when it ran out or another thread flagged an error.
GLA_DEV bool mbar_wait(uint64_t* b, uint32_t parity, volatile int* err) {
  for (long long it = 0; it < kWaitLimit; it++) {
    if (mbar_try(b, parity)) return true;
    if ((it & 1023) == 1023 && *err) return false;
  }
  atomicExch((int*)err, 1);
  return false;
}
GLA_DEV void mbar_arrive(uint64_t* b) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(b)) : "memory");
}
GLA_DEV void mbar_expect_tx(uint64_t* b, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(b)), "r"(bytes) : "memory");
}
GLA_DEV void bulk_g2s(void* dst, const void* src, uint32_t bytes, uint64_t* bar) {
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                   smem_u32(dst)),
               "l"(src), "r"(bytes), "r"(smem_u32(bar))
               : "memory");
}
GLA_DEV void mma_f16(uint32_t tmem_d, uint64_t ad, uint64_t bd, uint32_t accumulate) {
  asm volatile(
      "{\n.reg .pred p;\nsetp.ne.b32 p, %4, 0;\ntcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}" ::"r"(
          tmem_d),
      "l"(ad), "l"(bd), "r"(kIdesc), "r"(accumulate));
}
GLA_DEV void mma_commit(uint64_t* bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(bar))
               : "memory");
}
GLA_DEV void tmem_ld16(uint32_t taddr, uint32_t (&r)[16]) {
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
        "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
      : "r"(taddr));
}

struct GemmArgs {
  Sliced A, B;           // A: rows = M (H = 128); B: rows = N (H = 64)
  int M, N, K;
  int ntn;               // column tiles
  float* Chi;
  float* Clo;
  long long ldc;
  int lower;             // only tiles touching the lower triangle, only i >= j stored
  int* err;
};

// ---------------------------------------------------------------- slicing

// Column c of a float-pair matrix (len entries, leading dimension ld; for a
// symmetric A its column c is its row c) -> S integer slices of the scaled
// values, written as row c of a tiled operand. One CTA per column. The
// slicing runs in double-float arithmetic on the FP32 pipe: the remainder
// r = (hi, lo) 2^-e is kept exactly (scalings by powers of two, TwoSum), the
// next slice is rint of its leading float (|d_1| <= 128, |d_s| <= 65 after).
__global__ void __launch_bounds__(256) k_oz_slice(const float* __restrict__ hi, const float* __restrict__ lo,
                                                  long long ld, int len, int ncols, Sliced out) {
  const int c = blockIdx.x;
  __shared__ float red[8];
  const float* h = hi + (long long)c * ld;
  const float* l = lo ? lo + (long long)c * ld : nullptr;
  float m = 0.f;
  if (c < ncols)
    for (int k = threadIdx.x; k < len; k += 256) m = fmaxf(m, fabsf(h[k]));
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = m;
  __syncthreads();
  m = 0.f;
  for (int w = 0; w < 8; w++) m = fmaxf(m, red[w]);
  // |hi + lo| < 2^(ilogb(m) + 1) up to the last ulp: |value| 2^-e < 1 (an
  // edge value reaching 1 gives d_1 = 129, still exact in bf16 and inside
  // the accumulation bound)
  const int e = m > 0.f ? ilogbf(m) + 1 : 0;
  if (threadIdx.x == 0) out.exps[c] = e;
  const int b = c / out.H, r = c % out.H;
  const size_t bb = (size_t)block_bytes(out.H);
  char* base = reinterpret_cast<char*>(out.base);
  const int kpad = out.nks * kKS;
  for (int k = threadIdx.x; k < kpad; k += 256) {
    float vh = 0.f, vl = 0.f;
    if (c < ncols && k < len) {
      vh = ldexpf(h[k], -e);
      vl = l ? ldexpf(l[k], -e) : 0.f;
    }
    const int q = k / kKS, kk = k % kKS;
    char* blk = base + (((size_t)b * out.nks + q) * kMaxSlices * bb) + tile_off(r, kk);
    for (int s = 0; s < kMaxSlices; s++) {
      const float th = vh * 128.f, tl = vl * 128.f;
      const float d = rintf(th);
      float sh, se;
      two_sum(th - d, tl, sh, se);  // th - d is exact (|th - d| <= 1/2, same binade scale)
      vh = sh;
      vl = se;
      *reinterpret_cast<__nv_bfloat16*>(blk + s * bb) = __float2bfloat16_rn(d);
    }
  }
}

// Rows of a column-major float-pair matrix (element (c, k) at c + k ld) ->
// tiled operand rows, same slicing as k_oz_slice. One CTA per block of
// out.H rows; for each k the block's rows are read contiguously.
__global__ void __launch_bounds__(256) k_oz_slice_rows(const float* __restrict__ hi, const float* __restrict__ lo,
                                                       long long ld, int len, int nrows, Sliced out) {
  const int b = blockIdx.x, H = out.H, tid = threadIdx.x;
  const int per = 256 / H;            // threads per row (2 for H = 128, 4 for H = 64)
  const int r = tid % H, part = tid / H;
  const int c = b * H + r;
  __shared__ float smax[256];
  float m = 0.f;
  if (c < nrows)
    for (int k = part; k < len; k += per) m = fmaxf(m, fabsf(hi[c + (long long)k * ld]));
  smax[tid] = m;
  __syncthreads();
  m = 0.f;
  for (int q = 0; q < per; q++) m = fmaxf(m, smax[q * H + r]);
  const int e = m > 0.f ? ilogbf(m) + 1 : 0;
  if (part == 0) out.exps[c] = e;
  const size_t bb = (size_t)block_bytes(H);
  char* base = reinterpret_cast<char*>(out.base);
  const int kpad = out.nks * kKS;
  for (int k = part; k < kpad; k += per) {
    float vh = 0.f, vl = 0.f;
    if (c < nrows && k < len) {
      vh = ldexpf(hi[c + (long long)k * ld], -e);
      vl = lo ? ldexpf(lo[c + (long long)k * ld], -e) : 0.f;
    }
    const int q = k / kKS, kk = k % kKS;
    char* blk = base + (((size_t)b * out.nks + q) * kMaxSlices * bb) + tile_off(r, kk);
    for (int s = 0; s < kMaxSlices; s++) {
      const float th = vh * 128.f, tl = vl * 128.f;
      const float d = rintf(th);
      float sh, se;
      two_sum(th - d, tl, sh, se);
      vh = sh;
      vl = se;
      *reinterpret_cast<__nv_bfloat16*>(blk + s * bb) = __float2bfloat16_rn(d);
    }
  }
}

// ---------------------------------------------------------------- GEMM

__global__ void __launch_bounds__(kThreads, 1) k_oz_gemm(const GemmArgs g) {
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
  constexpr size_t stB = stage_bytes(kMaxSlices, kMaxSlices);
  constexpr uint32_t kAAll = kMaxSlices * kABlock, kBAll = kMaxSlices * kBBlock;

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
    // ---- MMA issuer: per slab the 28 slice pairs, unrolled with constant
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
#pragma unroll
          for (int ks = 0; ks < kKS / 16; ks++)  // K = 16 per instruction: 2 K-core matrices = 256 B
#pragma unroll
            for (int s = 1; s <= kMaxSlices; s++)
#pragma unroll
              for (int t = 1; t <= kMaxSlices; t++) {
                if (s + t > kMaxLevel) continue;
                // in this order (s = 1 first) the group's first MMA into
                // level s + t has s = 1 and starts the accumulator from zero
                const uint32_t accumulate = (qq == 0 && ks == 0 && s == 1) ? 0u : 1u;
                mma_f16(tmem + (uint32_t)((s + t - 2) * kBN),
                        a0 + (uint64_t)(((s - 1) * kABlock + ks * 256) >> 4),
                        b0 + (uint64_t)(((t - 1) * kBBlock + ks * 256) >> 4), accumulate);
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
    df64 acc[kDrainCols];
#pragma unroll
    for (int c = 0; c < kDrainCols; c++) acc[c] = df_make(0.f, 0.f);
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
            float sh, se;
            two_sum(part_hi[q], __uint_as_float(v[q]) * sc, sh, se);
            part_hi[q] = sh;
            part_lo[q] += se;
          }
        }
#pragma unroll
        for (int q = 0; q < 16; q++) acc[c0 + q] = df_add(acc[c0 + q], df_make(part_hi[q], part_lo[q]));
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
        g.Chi[idx] = ldexpf(acc[c].hi, e);
        g.Clo[idx] = ldexpf(acc[c].lo, e);
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
